// FP64 instantiation of the step kernels.  Built with --fmad=false: no a*b+c is fused, so
// every operation rounds as the reference's does when built with -ffp-contract=off.
#include "ark_kernels.cuh"

#include <cstring>
#include <vector>

namespace ark {
template struct Launch<double>;
template void rows_from_double<double>(double *, const double *, int, int64_t, int, double, cudaStream_t);
template void rows_to_double<double>(double *, const double *, int, int64_t, int, double, cudaStream_t);
template void flat_from_host<double>(double *, const double *, int, int64_t, int, double, cudaStream_t);
template void flat_to_host<double>(double *, const double *, int, int64_t, int, double, cudaStream_t);
template void rows_face_density<double>(double *, const double *, int, int64_t, int, double, double, cudaStream_t);

// Self-check of div_rn against the hardware IEEE division: n operand pairs from splitmix64
// (random signs and mantissas; numerator exponents over the whole range, subnormals and
// zeros included, divisor exponents in [-120, 120]); divisors are reused 8 times so the
// reciprocal is a "run constant" like dx or dt.  Also the small exact cases the step meets.
// qdiv is checked on the same pairs, and on a table of divisors prepared by make_qrecip on the
// host (powers of two, the significands 2^52 + 1 and 2^53 - 1, the channel's constants, random
// values), where the device's own make_qrecip must also agree with the host's, and qrecip_var
// (the per-cell divisor's reciprocal) with make_qrecip; qdiv2 against the division of 2a, and
// dhalf against a / 2, and the integer fixed-point image (fixed32) against its FP64 form.
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
struct QCase {
    double b;
    QRecip q;
};
__device__ __forceinline__ bool same(double x, double y) { return __double_as_longlong(x) == __double_as_longlong(y); }
__global__ void k_selftest_division(long long n, unsigned long long seed, const QCase *qc, int nqc,
                                    unsigned long long *bad) {
    unsigned long long local = 0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const unsigned long long za = mix64(seed + 2 * (unsigned long long)t);
        const double a = (t & 3) == 0 ? rnd_double(za, -1075, 1000) : rnd_double(za, -60, 60);
        const double b = rnd_double(mix64(seed + 2 * (unsigned long long)(t / 8) + 1), -120, 120);
        const double rb = 1.0 / b;
        const double want = a / b, got = div_rn(a, b, rb);
        if (__double_as_longlong(want) != __double_as_longlong(got)) ++local;
        const double a2 = (double)(long long)(t % 2001 - 1000) * 0.5, b2 = 10.0;
        if (__double_as_longlong(a2 / b2) != __double_as_longlong(div_rn(a2, b2, 1.0 / b2))) ++local;
        const QRecip qm = make_qrecip(b), qv = qrecip_var(b);
        if (!same(want, qdiv(a, b, rb, qm))) ++local;
        if (qv.r0 != qm.r0 || qv.r1 != qm.r1 || qv.k != qm.k || qv.sgn != qm.sgn) ++local;
        if (!same(want, qdiv_v(a, b, qv))) ++local;
        if (!same((2.0 * a) / b, qdiv2(a, b, rb, qm))) ++local;
        if (!same(a / 2.0, dhalf(a))) ++local;
        // the fixed-point image, over the whole range and near ties (values of 2^-33 multiples)
        const double v1 = (t & 1) ? a : (double)(long long)(za >> 20) * 0x1p-33 * ((t & 2) ? -1.0 : 1.0);
        if (fixed32(v1) != fixed32_fp64(v1)) ++local;
        // the FP32 path's image from the FP32 bits: every bit pattern (NaN, infinities and
        // subnormals included) and values near ties, against the image of the widened value
        const float f1 = (t & 8) ? __uint_as_float((unsigned)(za >> 32))
                                 : (float)((double)(long long)(za >> 40) * 0x1p-33 * ((t & 16) ? -1.0 : 1.0));
        if (fixed32(f1) != fixed32((double)f1)) ++local;
        const QCase &c = qc[t % nqc];
        if (t < nqc) {
            const QRecip d = make_qrecip(c.b);
            if (d.r0 != c.q.r0 || d.r1 != c.q.r1 || d.k != c.q.k || d.sgn != c.q.sgn) ++local;
        }
        if (!same(a / c.b, qdiv(a, c.b, 1.0 / c.b, c.q))) ++local;
        const QRecip cv = qrecip_var(c.b);
        if (cv.r0 != c.q.r0 || cv.r1 != c.q.r1 || cv.k != c.q.k || cv.sgn != c.q.sgn) ++local;
        if (!same(a / c.b, qdiv_v(a, c.b, cv))) ++local;
        if (!same(a2 / c.b, qdiv(a2, c.b, 1.0 / c.b, c.q))) ++local;
        // a numerator with the divisor's significand bits: exact and near-exact quotients
        const double a3 = c.b * (double)(long long)(t % 4097 - 2048) * ((t & 4) ? 0.75 : 1.0);
        if (!same(a3 / c.b, qdiv(a3, c.b, 1.0 / c.b, c.q))) ++local;
    }
    if (local) atomicAdd(bad, local);
}

int selftest_division(long long n, unsigned long long seed, unsigned long long *bad, cudaStream_t st) {
    std::vector<double> bs = {1.0, 0.5, 2.0, -4.0, 0x1p-100, 0x1p100, 10.0, 100.0, 1.0 / 3.0, -7.0,
                              0x1.0000000000001p0, 0x1.fffffffffffffp0, -0x1.0000000000001p-7, 0x1.fffffffffffffp9,
                              6.283185307179586 / 256, 2.0 / 128, 3.141592653589793 / 128,
                              6.283185307179586 / 512, 3.141592653589793 / 256};
    unsigned long long z = seed ^ 0x5DEECE66Dull;
    while (bs.size() < 256) { // random significands, exponents in [-60, 60], both signs
        z = z * 6364136223846793005ull + 1442695040888963407ull;
        const unsigned long long m = (z >> 11) & 0x000FFFFFFFFFFFFFull;
        const unsigned long long e = (unsigned long long)(1023 - 60 + (int)((z >> 1) % 121));
        const unsigned long long bits = ((z & 1ull) << 63) | (e << 52) | m;
        double b;
        std::memcpy(&b, &bits, sizeof b);
        bs.push_back(b);
    }
    std::vector<QCase> h(bs.size());
    for (size_t i = 0; i < bs.size(); ++i) h[i] = {bs[i], make_qrecip(bs[i])};
    QCase *d = nullptr;
    if (cudaMalloc(&d, sizeof(QCase) * h.size()) != cudaSuccess) return 1;
    cudaMemcpy(d, h.data(), sizeof(QCase) * h.size(), cudaMemcpyHostToDevice);
    k_selftest_division<<<152 * 4, 256, 0, st>>>(n, seed, d, (int)h.size(), bad);
    cudaStreamSynchronize(st);
    cudaFree(d);
    return 0;
}
} // namespace ark
