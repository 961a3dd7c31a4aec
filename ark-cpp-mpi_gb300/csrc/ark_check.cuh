// Bounds-checked builds (-DARK_CHECK; ark_build.py --check puts them in lib_check/).
//
// compute-sanitizer is not available on every machine this library runs on, so a checked
// build compares the indices of the kernels' global-memory accesses, and the cell coordinates
// their blocks decode, with the extents they must stay inside:
//   ARK_CK(idx, n)                    an element index of an array of n elements;
//   ARK_CK_IN(v, lo, hi)              a coordinate or work-item index that must lie in [lo, hi].
// A value outside is counted and the first one recorded (value, bound, source line); the index
// is replaced by 0 so the access stays inside its array, and a coordinate check answers false
// so the caller skips the cell.  Nothing traps: the host reads the record with
// ark_bounds_check() after the kernels ran.  In ordinary builds both macros cost nothing
// (ARK_CK is the index itself, ARK_CK_IN is true).
//
// Each translation unit that includes this header has its own record (device variables are
// per module) and registers a reader for it when the library loads.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ark {

// hits; first value, its bound, the source line
struct CheckRecord {
    unsigned long long hits;
    long long value, bound, line;
};
// The readers of the translation units' records (ark_api.cu): read (and with reset, clear) one.
typedef int (*CheckReader)(CheckRecord *out, int reset);
int check_register(CheckReader reader);

#ifdef ARK_CHECK
static __device__ CheckRecord g_check_record;

static __device__ __noinline__ void check_hit(long long value, long long bound, int line) {
    if (atomicAdd(&g_check_record.hits, 1ull) == 0ull) {
        g_check_record.value = value;
        g_check_record.bound = bound;
        g_check_record.line = line;
    }
}
template <class I> __device__ __forceinline__ I check_index(I idx, long long n, int line) {
    if ((long long)idx >= 0 && (long long)idx < n) return idx;
    check_hit((long long)idx, n, line);
    return (I)0;
}
__device__ __forceinline__ bool check_in(long long v, long long lo, long long hi, int line) {
    if (v >= lo && v <= hi) return true;
    check_hit(v, v < lo ? lo : hi, line);
    return false;
}
#define ARK_CK(idx, n) (::ark::check_index((idx), (long long)(n), __LINE__))
#define ARK_CK_IN(v, lo, hi) (::ark::check_in((long long)(v), (long long)(lo), (long long)(hi), __LINE__))

static int read_check_record(CheckRecord *out, int reset) {
    if (cudaMemcpyFromSymbol(out, g_check_record, sizeof(CheckRecord)) != cudaSuccess) return 1;
    if (reset) {
        CheckRecord z = {0ull, 0, 0, 0};
        if (cudaMemcpyToSymbol(g_check_record, &z, sizeof z) != cudaSuccess) return 1;
    }
    return 0;
}
static const int check_registered = check_register(&read_check_record);
#else
#define ARK_CK(idx, n) (idx)
#define ARK_CK_IN(v, lo, hi) (true)
#endif

} // namespace ark
