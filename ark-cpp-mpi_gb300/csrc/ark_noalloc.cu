// ark_conservation_sums_noalloc: the conservation sums of ark_conservation_sums over device
// arrays the caller owns, with no device allocation at all.
//
// Who needs it: a caller whose device memory is already owned by something else -- a grid
// that fills the GPU, or arrays handed out by another framework's caching allocator -- and
// who wants the mass / momentum / energy check inside its own loop.  ark_conservation_sums
// needs an ark_ctx, and ark_create allocates the whole solver state; a cudaMalloc/cudaFree
// pair per call would synchronize the device and can fail when the pool holds all memory.
//
// Scratch: one file-scope __device__ array of (kMaxBlocks + 1) x kCols 64-bit integers
// (65,600 bytes), which every GPU that loads the library keeps until the process exits.
// Each block writes one row of partial sums; a second kernel adds the rows into the last
// row.  Nothing in it has to start at zero: a call writes every row it reads.  All calls
// share the array, so calls that overlap on the GPU (different streams or host threads at
// the same time) race and must be serialized by the caller.
//
// The device address of the array is looked up with cudaGetSymbolAddress once per device, on
// the first call made while that device is current, and kept; make that first call before any
// stream capture on the device.  A cudaDeviceReset of that device after the first call is not
// supported: the module can load again at another address, which the kept one would miss.
// Errors are reported through the status and ark_last_error(), like every other entry point.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/ark_gpu.h"
#include "ark_kernels.cuh"

namespace {

constexpr int kMaxBlocks = 1024;                                    // rows of partial sums
constexpr int kCellsPerBlock = 65536;                               // interior cells per row
constexpr long long kMaxCells = (long long)kMaxBlocks * kCellsPerBlock; // 67,108,864 cells
constexpr int kCols = 8;                                            // 6 used: 5 sums + cell count
constexpr int kThreads = 256;

static __device__ __align__(256) long long g_sums_scratch[(kMaxBlocks + 1) * kCols];
static_assert(sizeof(g_sums_scratch) == 65600, "scratch size stated in ark_gpu.h");

constexpr int kMaxDevices = 128;
std::mutex g_mu;
long long *g_scratch_addr[kMaxDevices]; // the array's device address, per device once looked up

// Per-block partial sums of the same fixed-point terms k_sums accumulates.
__global__ void __launch_bounds__(kThreads)
k_sums_rows(const double *ro, const double *u1, const double *u2, const double *u3, const double *cond,
            ark::Geom g, long long n, long long *scratch) {
    __shared__ long long red[kThreads / 32][6];
    long long a[6] = {0, 0, 0, 0, 0, 0};
    const long long lo = (long long)blockIdx.x * kCellsPerBlock;
    const long long hi = lo + kCellsPerBlock < n ? lo + kCellsPerBlock : n;
    for (long long t = lo + threadIdx.x; t < hi; t += kThreads) {
        const int i = (int)(t % g.C1) + 1;
        const long long r = t / g.C1;
        const int j = (int)(r % g.C2) + 1;
        const int k = (int)(r / g.C2) + 1;
        const int64_t c = g.cell(i, j, k);
        if (cond[c] != 0) continue;
        const double r0 = ro[c], v1 = u1[c], v2 = u2[c], v3 = u3[c];
        a[0] += ark::fixed32(r0);
        a[1] += ark::fixed32(r0 * v1);
        a[2] += ark::fixed32(r0 * v2);
        a[3] += ark::fixed32(r0 * v3);
        a[4] += ark::fixed32((v1 * v1 + v2 * v2 + v3 * v3) / 2);
        a[5] += 1;
    }
    for (int q = 0; q < 6; ++q) a[q] = ark::warp_sum_i64(a[q]);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 6; ++q) red[w][q] = a[q];
    __syncthreads();
    if (threadIdx.x < 6) {
        long long s = 0;
        for (int v = 0; v < kThreads / 32; ++v) s += red[v][threadIdx.x];
        scratch[(long long)blockIdx.x * kCols + threadIdx.x] = s;
    }
}

// One block: add rows 0..nrows-1 column by column into row kMaxBlocks.
__global__ void __launch_bounds__(kThreads) k_sums_total(long long *scratch, int nrows) {
    __shared__ long long red[kThreads / 32];
    for (int q = 0; q < 6; ++q) {
        long long s = 0;
        for (int r = threadIdx.x; r < nrows; r += kThreads) s += scratch[(long long)r * kCols + q];
        s = ark::warp_sum_i64(s);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            long long t = 0;
            for (int v = 0; v < kThreads / 32; ++v) t += red[v];
            scratch[(long long)kMaxBlocks * kCols + q] = t;
        }
        __syncthreads();
    }
}

} // namespace

namespace {
int cuda_fail(const char *what, cudaError_t e) {
    return ark::api_fail(ARK_ERR_CUDA, std::string("ark_conservation_sums_noalloc: ") + what + ": " +
                                           cudaGetErrorString(e));
}
} // namespace

extern "C" int ark_conservation_sums_noalloc(const ark_params *p, const double *ro, const double *u1,
                                             const double *u2, const double *u3, const double *condition,
                                             ark_sums *out) {
    if (!p || !ro || !u1 || !u2 || !u3 || !condition || !out)
        return ark::api_fail(ARK_ERR_PARAM, "ark_conservation_sums_noalloc: NULL argument");
    if (p->n1_cells < 1 || p->n2_cells < 1 || p->n3_cells < 1)
        return ark::api_fail(ARK_ERR_PARAM, "ark_conservation_sums_noalloc: need at least one cell per axis");
    const long long n = (long long)p->n1_cells * p->n2_cells * p->n3_cells;
    if (n > kMaxCells)
        return ark::api_fail(ARK_ERR_PARAM, "ark_conservation_sums_noalloc: " + std::to_string(n) +
                                                " interior cells exceed the static scratch's limit of 67,108,864");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail("cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices)
        return ark::api_fail(ARK_ERR_UNSUPPORTED, "ark_conservation_sums_noalloc: device ordinal beyond 127");
    long long *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch_addr[dev]) {
            void *addr = nullptr;
            e = cudaGetSymbolAddress(&addr, g_sums_scratch);
            if (e != cudaSuccess || !addr)
                return cuda_fail("cudaGetSymbolAddress", e != cudaSuccess ? e : cudaErrorInvalidSymbol);
            g_scratch_addr[dev] = (long long *)addr;
        }
        scratch = g_scratch_addr[dev];
    }
    ark::Geom g = ark::host_geom(p->n1_cells, p->n2_cells, p->n3_cells);
    int rows = (int)((n + kCellsPerBlock - 1) / kCellsPerBlock);
    // launched through cudaLaunchKernel, whose return value is this launch's own error (an
    // earlier error of the caller's stays where it is)
    void *a1[] = {(void *)&ro, (void *)&u1, (void *)&u2, (void *)&u3, (void *)&condition, (void *)&g, (void *)&n,
                  (void *)&scratch};
    e = cudaLaunchKernel((const void *)k_sums_rows, dim3(rows), dim3(kThreads), a1, 0, 0);
    if (e != cudaSuccess) return cuda_fail("row sums launch", e);
    void *a2[] = {(void *)&scratch, (void *)&rows};
    e = cudaLaunchKernel((const void *)k_sums_total, dim3(1), dim3(kThreads), a2, 0, 0);
    if (e != cudaSuccess) return cuda_fail("total launch", e);
    long long v[6];
    e = cudaMemcpy(v, scratch + (long long)kMaxBlocks * kCols, sizeof(v), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail("result copy", e);
    const double q = 1.0 / 4294967296.0;
    out->mass = (double)v[0] * q;
    out->momentum1 = (double)v[1] * q;
    out->momentum2 = (double)v[2] * q;
    out->momentum3 = (double)v[3] * q;
    out->kinetic = (double)v[4] * q;
    out->cells = v[5];
    return ARK_OK;
}
