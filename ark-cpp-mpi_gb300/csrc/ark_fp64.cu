// FP64 instantiation of the step kernels.  Built with --fmad=false: no a*b+c is fused, so
// every operation rounds as the reference's does when built with -ffp-contract=off.
#include "ark_kernels.cuh"

namespace ark {
template struct Launch<double>;
template void rows_from_double<double>(double *, const double *, int, int64_t, int, double, cudaStream_t);
template void rows_to_double<double>(double *, const double *, int, int64_t, int, double, cudaStream_t);
template void rows_face_density<double>(double *, const double *, int, int64_t, int, double, double, cudaStream_t);

// Self-check of div_rn against the hardware IEEE division: n operand pairs from splitmix64
// (random signs and mantissas; numerator exponents over the whole range, subnormals and
// zeros included, divisor exponents in [-120, 120]); divisors are reused 8 times so the
// reciprocal is a "run constant" like dx or dt.  Where the divisor's reciprocal is within a
// quarter ulp (recip_tight, about 70% of random divisors) the one-correction form is checked
// too.  Also the small exact cases the step meets.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double rnd_double(unsigned long long z, int emin, int emax) {
    const unsigned long long mant = z & 0x000FFFFFFFFFFFFFull;
    const long long e = (long long)((z >> 52) % (unsigned long long)(emax - emin + 1)) + emin + 1023;
    const unsigned long long sign = (z >> 63) << 63;
    if (e <= 0) return __longlong_as_double((long long)(sign | (mant >> (1 - e)))); // subnormal / zero
    return __longlong_as_double((long long)(sign | ((unsigned long long)e << 52) | mant));
}
__global__ void k_selftest_division(long long n, unsigned long long seed, unsigned long long *bad) {
    unsigned long long local = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const unsigned long long za = mix64(seed + 2 * (unsigned long long)t);
        const double a = (t & 3) == 0 ? rnd_double(za, -1075, 1000) : rnd_double(za, -60, 60);
        const double b = rnd_double(mix64(seed + 2 * (unsigned long long)(t / 8) + 1), -120, 120);
        const double rb = 1.0 / b;
        const double want = a / b, got = div_rn(a, b, rb);
        if (__double_as_longlong(want) != __double_as_longlong(got)) ++local;
        if (recip_tight(b, rb) && __double_as_longlong(want) != __double_as_longlong(div_rn(a, b, rb, true))) ++local;
        const double a2 = (double)(long long)(t % 2001 - 1000) * 0.5, b2 = 10.0;
        if (__double_as_longlong(a2 / b2) != __double_as_longlong(div_rn(a2, b2, 1.0 / b2))) ++local;
    }
    if (local) atomicAdd(bad, local);
}

void selftest_division(long long n, unsigned long long seed, unsigned long long *bad, cudaStream_t st) {
    k_selftest_division<<<152 * 4, 256, 0, st>>>(n, seed, bad);
}
} // namespace ark
