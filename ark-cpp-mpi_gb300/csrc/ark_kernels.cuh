// CUDA kernels of the CABARET step, templated on the storage/arithmetic type T.
//
// ark_fp64.cu instantiates T = double in a translation unit compiled with --fmad=false:
// every FP64 expression below keeps the reference's operand order (source/main.cpp), so the
// FP64 path rounds exactly like the reference built with -ffp-contract=off.  Its quotients are
// the correctly rounded IEEE ones, taken on the integer pipes where they can be (qdiv,
// qrecip_var), with the Markstein form (div_rn) and the IEEE division for the rest.
// ark_fp32.cu instantiates T = float (also without FMA contraction) with the density stored as
// the deviation rho - ro0 and face density derived from face pressure (Storage<T>).
//
// Kernels and the reference code they restate:
//   k_reduce_start / k_finalize_dt   TimeStepSize (main.cpp:374-415) + bulk-flow sum
//   k_wrap                           the single-rank halo exchange (main.cpp:603-801,
//                                    1049-1631) as a periodic ghost copy
//   k_phase1<MODE>                   Phase1 (main.cpp:417-575), optionally fused with
//                                    StressTensor's force (main.cpp:856-1023) and
//                                    UseForces (main.cpp:1026-1045)
//   k_stress_faces / k_stress_force  StressTensor alone (main.cpp:856-1023)
//   k_use_forces                     UseForces alone
//   k_sweep_x, k_sweep_col<AX>       Phase2 sweeps (main.cpp:1726-2011, 2023-2255, 2261-2494)
//   k_boundary_fill                  BoundaryConditions (source/BoundaryConditions.cpp:22-83)
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda.h> // CUtensorMap and its enums (types only: the encoder comes through the runtime)
#include <cuda_runtime.h>

#include <type_traits>

#include "ark_check.cuh"
#include "ark_state.h"

namespace ark {

// ---------------------------------------------------------------------------------------
// scalar helpers
// ---------------------------------------------------------------------------------------

// Ordered comparisons.  FP64 ones run on the integer pipe (GB300 issues FP64 instructions at a
// small fraction of the integer rate): dkey maps a double to an int64 whose order is the IEEE
// order, with -0 and +0 equal, so every comparison of non-NaN values gives the IEEE answer.
// Only NaN orders differently (above everything); a NaN velocity has already raised the
// non-finite status by then.
__device__ __forceinline__ long long dkey(double x) {
    const long long s = __double_as_longlong(x);
    return s < 0 ? (s ^ 0x7FFFFFFFFFFFFFFFll) + 1 : s;
}
template <class T> __device__ __forceinline__ bool lt(T a, T b) { return a < b; }
template <> __device__ __forceinline__ bool lt<double>(double a, double b) { return dkey(a) < dkey(b); }
template <class T> __device__ __forceinline__ bool gt(T a, T b) { return lt(b, a); }
template <class T> __device__ __forceinline__ bool ge0(T a) { return !lt(a, (T)0); }
template <class T> __device__ __forceinline__ bool le0(T a) { return !lt((T)0, a); }

// min3d / max3d of main.cpp:2963-2973: the same ternaries.
template <class T> __device__ __forceinline__ T min3d(T x1, T x2, T x3) {
    x1 = gt(x1, x2) ? x2 : x1;
    x1 = gt(x1, x3) ? x3 : x1;
    return x1;
}
template <class T> __device__ __forceinline__ T max3d(T x1, T x2, T x3) {
    x1 = lt(x1, x2) ? x2 : x1;
    x1 = lt(x1, x3) ? x3 : x1;
    return x1;
}

// a / b correctly rounded, given rb = RN(1/b) (the IEEE reciprocal).  Markstein's theorem
// (P. Markstein, "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990): if rb is within half an ulp of 1/b and q is
// within one ulp of a/b, then with the exact residual r = a - b*q (one FMA),
// RN(q + r*rb) = RN(a/b), provided nothing underflows or overflows.  q = RN(a*rb) may be up
// to 1.5 ulp off, so one correction makes it faithful and a second one makes it correctly
// rounded: 1 multiply + 4 FMA.  Operands outside 2^-895 <= |a| < 2^897 and
// 2^-100 <= |b| < 2^101 (where the residual could leave the normal range), zeros included, take
// the IEEE division instead; the exponent test is integer work.  The FP64 parity tests check
// every quotient of the step against the reference bit for bit, and ark_selftest_division
// compares it with the hardware division, tiny and subnormal operands included.
__device__ __forceinline__ double div_rn(double a, double b, double rb) {
    const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7FFu;
    const unsigned eb = ((unsigned)__double2hiint(b) >> 20) & 0x7FFu;
    if (ea - 128u > 1792u || eb - 923u > 200u) return a / b;
    double q = a * rb;
    double r = __fma_rn(-q, b, a);
    q = __fma_rn(r, rb, q);
    r = __fma_rn(-q, b, a);
    return __fma_rn(r, rb, q);
}

// RN(a / b) on the integer pipes, for a divisor b prepared by make_qrecip.  GB300 runs FP64 at
// 1/64 of its FP32 rate, so one warp-wide FP64 instruction holds the FP64 pipe for about 64
// cycles while integer instructions issue one per cycle: the step's FP64 kernels are bound by
// that pipe, and a quotient taken here (about 30 integer instructions) frees the three FP64
// operations of div_rn's one-correction form.
// With a = Ma 2^(ea-1075), Ma in [2^52, 2^53), and r = ceil(2^116 / Mb) = 2^116 / Mb + e,
// 0 <= e < 1: the product Ma r = Ma 2^116 / Mb + Ma e with Ma e < 2^53, so T = floor(Ma r / 2^53)
// and X = (Ma / Mb) 2^63 (the exact quotient's significand, in (2^62, 2^64)) satisfy
// T - 1 < X < T + 1.  The significand is RN(X / 2^(10+s)), s = 1 when T >= 2^63.  A quotient of
// two 53-bit significands is never a midpoint of 53-bit values (that would make an odd number
// of 54 or more bits a product of the divisor's significand and a 53-bit integer), so X lies on
// the same side of the rounding midpoint as T unless T's low 10+s bits are exactly the
// midpoint pattern; that case (about 1 in 2048), a zero, subnormal or non-finite a, and a
// result outside the normal range take div_rn.  For Mb = 2^52, r = 2^64 - 1 gives
// T = Ma 2^11 - 1, which rounds up to the exact quotient Ma 2^11.  ark_selftest_division
// compares this with the hardware division.  qdiv_try returns ok = false where the quotient
// needs another path.  TWICE: the quotient of 2a (exact for a below 2^1023), which is twice
// that of a wherever both are normal: the exponent takes the factor.
template <bool TWICE = false> __device__ __forceinline__ double qdiv_try(double a, const QRecip &Q, bool &ok) {
    const unsigned ha = (unsigned)__double2hiint(a), la = (unsigned)__double2loint(a);
    const unsigned ea = (ha >> 20) & 0x7FFu;
    const unsigned a1 = (ha & 0xFFFFFu) | 0x100000u; // significand high word with the hidden bit
    // w3:w2:w1 = bits 32..127 of (a1:la) * (r1:r0); bits 0..31 do not carry into them
    unsigned w1, w2, w3;
    asm("mul.hi.u32 %0, %3, %5;\n\t"
        "mad.lo.cc.u32 %0, %3, %6, %0;\n\t"
        "madc.hi.u32 %1, %3, %6, 0;\n\t"
        "mad.lo.cc.u32 %0, %4, %5, %0;\n\t"
        "madc.hi.cc.u32 %1, %4, %5, %1;\n\t"
        "addc.u32 %2, 0, 0;\n\t"
        "mad.lo.cc.u32 %1, %4, %6, %1;\n\t"
        "madc.hi.u32 %2, %4, %6, %2;"
        : "=&r"(w1), "=&r"(w2), "=&r"(w3)
        : "r"(la), "r"(a1), "r"(Q.r0), "r"(Q.r1));
    const unsigned thi = __funnelshift_l(w2, w3, 11), tlo = __funnelshift_l(w1, w2, 11); // T = P >> 53
    const unsigned s = thi >> 31, sh = 10u + s;
    const unsigned below = tlo << (32u - sh); // T's low sh bits, at the top of the word
    const int E = (int)ea + (int)s + Q.k + (TWICE ? 1 : 0); // the quotient's biased exponent
    ok = ea - 1u < (TWICE ? 2045u : 2046u) && (unsigned)(E - 1) < 2046u && below != 0x80000000u;
    const unsigned long long sig =
        (((unsigned long long)(thi >> sh) << 32) | __funnelshift_r(tlo, thi, sh)) + (below > 0x80000000u ? 1ull : 0ull);
    // the significand's hidden bit (bit 52) adds one to the exponent field E - 1; a carry out of
    // the rounding (sig = 2^53) adds another, and at E = 2046 gives the infinity RN gives
    const unsigned long long bits = sig + ((unsigned long long)(unsigned)(E - 1) << 52);
    return __hiloint2double((int)((unsigned)(bits >> 32) | ((ha & 0x80000000u) ^ Q.sgn)), (int)(unsigned)bits);
}
// The fallbacks as calls of their own, so that a rarely taken one is not evaluated ahead of the
// branch (a division has no side effects, so the compiler may otherwise compute it for every
// quotient and select).
static __device__ __noinline__ double ieee_div(double a, double b) { return a / b; }
static __device__ __noinline__ double div_rn_call(double a, double b, double rb) { return div_rn(a, b, rb); }
// b a run constant or dt (rb = RN(1/b)): the other path is div_rn
__device__ __forceinline__ double qdiv(double a, double b, double rb, const QRecip &Q) {
    bool ok;
    const double q = qdiv_try(a, Q, ok);
    return ok ? q : div_rn_call(a, b, rb);
}
// RN(2a / b), b as for qdiv
__device__ __forceinline__ double qdiv2(double a, double b, double rb, const QRecip &Q) {
    bool ok;
    const double q = qdiv_try<true>(a, Q, ok);
    return ok ? q : div_rn_call(2.0 * a, b, rb);
}
// x / 2: FP64 subtracts one from the exponent field when that is at least 2 (exact, as the
// multiply by 0.5 is); a zero, tiny or non-finite x takes the multiply.
static __device__ __noinline__ double halve_call(double x) { return x * 0.5; }
__device__ __forceinline__ double dhalf(double x) {
    const unsigned h = (unsigned)__double2hiint(x);
    if (((h >> 20) & 0x7FFu) - 2u < 2045u) return __hiloint2double((int)(h - 0x100000u), __double2loint(x));
    return halve_call(x);
}
__device__ __forceinline__ float dhalf(float x) { return x / 2.f; }
// b that changes from cell to cell (Q from qrecip_var): the other path is the IEEE division
__device__ __forceinline__ double qdiv_v(double a, double b, const QRecip &Q) {
    bool ok;
    const double q = qdiv_try(a, Q, ok);
    return ok ? q : ieee_div(a, b);
}

// make_qrecip on the integer pipes, for a divisor that changes from cell to cell.  Seed: the FP32
// reciprocal approximation of f = M / 2^52 (its top 24 bits), absolute error below 2^-23 on
// (1/2, 1], so R0 = RN32(1/f) 2^64 has relative error below 2^-21.4.  Two Newton steps
// R <- R + R (2^116 - M R) / 2^116 in 64-bit fixed point (Newton's iteration for the
// reciprocal; R. Brent, P. Zimmermann, "Modern Computer Arithmetic", 2010, sec. 4.2.2)
// square the relative error twice (2^-42.8, then 2^-85.6).  An exact Newton step never lands
// above 2^116 / M (the new error is -(2^116 / M) e^2); the products here are rounded down, and
// (2^116 - M R) / 2^32 is rounded up by at most 2^-32, so after the second step R lies within
// 1 + 2^-20 below 2^116 / M and at most 2^-20 above it.  The exact remainder 2^116 - M R then
// counts the steps (one or two) to ceil(2^116 / M); for M = 2^52, where that is 2^64, R is
// 2^64 - 1 as make_qrecip sets it.  A zero, subnormal or non-finite divisor
// gets k = -100000 (every quotient takes the IEEE division).
__device__ __forceinline__ QRecip qrecip_var(double b) {
    const unsigned hb = (unsigned)__double2hiint(b), m0 = (unsigned)__double2loint(b);
    const unsigned eb = (hb >> 20) & 0x7FFu;
    const unsigned m1 = (hb & 0xFFFFFu) | 0x100000u; // M = m1:m0
    QRecip q;
    q.sgn = hb & 0x80000000u;
    q.k = eb - 1u < 2046u ? 1022 - (int)eb : -100000;
    const float f = __uint_as_float(0x3F800000u | ((hb & 0xFFFFFu) << 3) | (m0 >> 29));
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(f));
    unsigned long long R = (unsigned long long)__float2uint_rz(rf * 0x1p32f) << 32; // saturates at 1/f = 1
    const unsigned long long M = ((unsigned long long)m1 << 32) | m0;
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        // w2:w1 = bits 32..95 of M R; (2^116 - M R) / 2^32 lies within 2^63 of zero, so its low
        // 64 bits, -(w2:w1), hold it
        unsigned w1, w2;
        asm("mul.hi.u32 %0, %2, %4;\n\t"
            "mad.lo.cc.u32 %0, %2, %5, %0;\n\t"
            "madc.hi.u32 %1, %2, %5, 0;\n\t"
            "mad.lo.cc.u32 %0, %3, %4, %0;\n\t"
            "madc.hi.u32 %1, %3, %4, %1;\n\t"
            "mad.lo.u32 %1, %3, %5, %1;"
            : "=&r"(w1), "=&r"(w2)
            : "r"(m0), "r"(m1), "r"((unsigned)R), "r"((unsigned)(R >> 32)));
        const long long D = (long long)(0ull - (((unsigned long long)w2 << 32) | w1));
        // floor(R D / 2^84): the signed high word of R * D (R is unsigned), shifted
        long long hi = (long long)__umul64hi(R, (unsigned long long)D);
        if (D < 0) hi -= (long long)R;
        R += (unsigned long long)(hi >> 20);
    }
    long long rem = (long long)(0ull - M * R); // 2^116 - M R, exact: |rem| < 2^63
#pragma unroll
    for (int it = 0; it < 3; ++it) {
        const bool up = rem > 0;
        R += up ? 1ull : 0ull;
        rem -= up ? (long long)M : 0ll;
    }
    if (M == (1ull << 52)) R = ~0ull; // 2^116 / M = 2^64: make_qrecip's 2^64 - 1 (see qdiv)
    q.r0 = (unsigned)R;
    q.r1 = (unsigned)(R >> 32);
    return q;
}

// Division by a run constant or by dt, with the divisor's reciprocals: FP64 on the integer pipes
// (qdiv, correctly rounded), FP32 multiplication by the reciprocal.
__device__ __forceinline__ double divq(double a, double b, double rb, const QRecip &Q) { return qdiv(a, b, rb, Q); }
__device__ __forceinline__ float divq(float a, float b, float rb, const QRecip &) {
    (void)b;
    return a * rb;
}

// Division by a cell-dependent value.
__device__ __forceinline__ double divv(double a, double b) { return a / b; }
__device__ __forceinline__ float divv(float a, float b) { return __fdiv_rn(a, b); }

// Reciprocal of a cell-dependent value for divr below: IEEE 1/b (FP64), or 1/b (FP32).
__device__ __forceinline__ double recip(double b) { return __drcp_rn(b); }
__device__ __forceinline__ float recip(float b) { return __frcp_rn(b); }
// a / b with rb = recip(b): correctly rounded in FP64, a*rb in FP32.
__device__ __forceinline__ double divr(double a, double b, double rb) { return div_rn(a, b, rb); }
__device__ __forceinline__ float divr(float a, float b, float rb) {
    (void)b;
    return a * rb;
}

// Run constants rounded to T (filled on the host).
template <class T> using K = KT<T>;

// a*b + c.  FP64: the product and the sum rounded separately, as the reference computes them
// (the FP64 code is built with --fmad=false).  FP32: one fused multiply-add.  Every FP32 kernel
// shape calls the same helpers, so all of them keep identical bits.
__device__ __forceinline__ double mad(double a, double b, double c) { return a * b + c; }
__device__ __forceinline__ float mad(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// ---------------------------------------------------------------------------------------
// TimeStepSize + bulk flow rate
// ---------------------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ unsigned long long abs_bits(float v) {
    // widen to double so the accumulator compares like FP64 values
    return (unsigned long long)__double_as_longlong((double)fabsf(v));
}

// Fixed-point image of a value: round(v * 2^32) (to nearest, ties to even), NaN -> 0, v clamped
// to +-2^30.  The FP64 form (fixed32_fp64) costs five FP64-pipe instructions; this one takes the
// same integer from the bits: v = M 2^(e-1075), so v 2^32 = M 2^(e-1043), a left shift for
// e >= 1043 and a rounded right shift below.  ark_selftest_division compares the two.
__device__ __forceinline__ long long fixed32_fp64(double v) {
    if (v != v) v = 0.0;
    v = fmin(fmax(v, -1073741824.0), 1073741824.0);
    return __double2ll_rn(v * 4294967296.0);
}
__device__ __forceinline__ long long fixed32(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FF);
    const unsigned long long M = (b & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
    unsigned long long m;
    if (e >= 1053) { // |v| >= 2^30, infinities and NaN
        if (e == 0x7FF && (b & 0x000FFFFFFFFFFFFFull)) return 0;
        m = 1ull << 62;
    } else if (e >= 1043) {
        m = M << (e - 1043);
    } else if (e >= 1043 - 54) { // shifts of 1..54: round to nearest, ties to even
        const int k = 1043 - e;
        const unsigned long long q = M >> k, r = M & ((1ull << k) - 1), half = 1ull << (k - 1);
        m = q + ((r > half || (r == half && (q & 1))) ? 1ull : 0ull);
    } else {
        m = 0; // below 2^-33: rounds to zero (zeros and subnormals included)
    }
    return (b >> 63) ? -(long long)m : (long long)m;
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}
__device__ __forceinline__ long long warp_sum_i64(long long v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Fixed-point image of an FP32 value for the FP32 path's bulk-flow sum: the same integer
// round(v * 2^32) (ties to even, NaN -> 0, |v| clamped to 2^30) that fixed32 gives for the value
// widened to FP64, taken from the FP32 bits with integer instructions only (the FP64 pipe runs
// at 1/64 of the FP32 rate on this part): v = M 2^(e-150), so v 2^32 = M 2^(e-118), a left
// shift for e >= 118 and a rounded right shift below.  Every |v| >= 2^-9 is represented
// exactly, smaller ones to 2^-33.
__device__ __forceinline__ long long fixed32(float v) {
    const unsigned b = __float_as_uint(v);
    const int e = (int)((b >> 23) & 0xFFu);
    const unsigned M = (b & 0x7FFFFFu) | 0x800000u;
    unsigned long long m;
    if (e >= 157) { // |v| >= 2^30, infinities and NaN
        if (e == 0xFF && (b & 0x7FFFFFu)) return 0;
        m = 1ull << 62;
    } else if (e >= 118) {
        m = (unsigned long long)M << (e - 118);
    } else if (e >= 118 - 25) { // shifts of 1..25: round to nearest, ties to even
        const int k = 118 - e;
        const unsigned q = M >> k, r = M & ((1u << k) - 1u), half = 1u << (k - 1);
        m = q + ((r > half || (r == half && (q & 1u))) ? 1u : 0u);
    } else {
        m = 0; // below 2^-33: rounds to zero (zeros and subnormals included)
    }
    return (b >> 31) ? -(long long)m : (long long)m;
}
__device__ __forceinline__ long long fixed_sum_term(double v) { return fixed32(v); }
__device__ __forceinline__ long long fixed_sum_term(float v) { return fixed32(v); }
// both precisions sum in units of 2^-32
template <class T> struct FixedScale { static constexpr double inv = 1.0 / 4294967296.0; };

// |v| as an order-preserving integer: FP64 bit pattern, or FP32 bit pattern (widened to an
// FP64 bit pattern once per tile, see tile_store).
__device__ __forceinline__ unsigned long long abs_key(double v) { return abs_bits(v); }
__device__ __forceinline__ unsigned long long abs_key(float v) { return (unsigned long long)__float_as_uint(fabsf(v)); }
__device__ __forceinline__ unsigned long long key_to_double_bits(unsigned long long m, double) { return m; }
__device__ __forceinline__ unsigned long long key_to_double_bits(unsigned long long m, float) {
    return (unsigned long long)__double_as_longlong((double)__uint_as_float((unsigned)m));
}

// Block coordinates of one unit of work.  A single-grid launch takes them from blockIdx; a
// batched (ensemble) launch decodes them from its work list, so both run the same bodies.
struct BIx {
    int x, y, z, gx, gy;
    __device__ __forceinline__ int linear() const { return x + gx * (y + gy * z); }
};
__device__ __forceinline__ BIx bix_here() {
    BIx b = {(int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z, (int)gridDim.x, (int)gridDim.y};
    return b;
}

// Block-wide combination of the per-thread partials into the block's slot.  Every thread of
// the block (NT threads) must call it.
template <class T, int NT = kTileX * kTileY>
__device__ __forceinline__ void tile_store(const DevState<T> &S, const BIx &bx, bool do_max, bool do_sum,
                                           unsigned long long m0, unsigned long long m1, unsigned long long m2,
                                           long long s) {
    __shared__ unsigned long long smax[3][NT / 32];
    __shared__ long long ssum[NT / 32];
    m0 = warp_max_u64(m0);
    m1 = warp_max_u64(m1);
    m2 = warp_max_u64(m2);
    s = warp_sum_i64(s);
    const int t = threadIdx.y * blockDim.x + threadIdx.x, w = t >> 5;
    if ((t & 31) == 0) {
        smax[0][w] = m0;
        smax[1][w] = m1;
        smax[2][w] = m2;
        ssum[w] = s;
    }
    __syncthreads();
    const int slot = bx.linear() % kBuckets;
    if (t < 3 && do_max) {
        unsigned long long m = 0;
        for (int v = 0; v < NT / 32; ++v) m = smax[t][v] > m ? smax[t][v] : m;
        if (m) atomicMax(&S.part_max[3 * slot + t], key_to_double_bits(m, T()));
    } else if (t == 3 && do_sum) {
        long long z = 0;
        for (int v = 0; v < NT / 32; ++v) z += ssum[v];
        if (z) atomicAdd((unsigned long long *)&S.part_sum[slot], (unsigned long long)z);
    }
}

// Standalone partials of the step start (used after an upload or the reference-order calls;
// the fused step takes the same partials inside its Phase1 kernels): max |u_d| of level
// `con` and the fixed-point sum of u1 over fluid cells of level `con^1`.  The slots must be
// clear.
// dt is monotone in max |u|: min over cells of CFL*dx/(c + |u|) is CFL*dx/(c + max|u|)
// exactly, since IEEE + and / are monotone.  Max and integer sums are order independent.
template <class T> __device__ __forceinline__ void reduce_start_body(const DevState<T> &S, int con, const BIx &bx) {
    const Geom g = S.g;
    const int i = bx.x * kTileX + threadIdx.x + 1;
    const int j = bx.y * kTileY + threadIdx.y + 1;
    const int k0 = bx.z * kTileK + 1;
    const int k1 = k0 + kTileK - 1 < g.C3 ? k0 + kTileK - 1 : g.C3;
    const T *__restrict__ cu1 = S.lv[con].u1;
    const T *__restrict__ cu2 = S.lv[con].u2;
    const T *__restrict__ cu3 = S.lv[con].u3;
    const T *__restrict__ nu1 = S.lv[con ^ 1].u1;
    const uint8_t *__restrict__ fl = S.flags;
    unsigned long long m0 = 0, m1 = 0, m2 = 0;
    long long s = 0;
    if (i <= g.C1 && j <= g.C2 && ARK_CK_IN(k0, 1, g.C3)) {
        const int cs2 = (int)g.cs2;
        int c = g.ci(i, j, k0);
#pragma unroll 4
        for (int k = k0; k <= k1; ++k, c += cs2) {
            const unsigned long long b0 = abs_key(cu1[c]), b1 = abs_key(cu2[c]), b2 = abs_key(cu3[c]);
            m0 = b0 > m0 ? b0 : m0;
            m1 = b1 > m1 ? b1 : m1;
            m2 = b2 > m2 ? b2 : m2;
            if (fl[c] & FL_EQ0) s += fixed_sum_term(nu1[c]);
        }
    }
    tile_store(S, bx, true, true, m0, m1, m2, s);
}
template <class T>
__global__ void __launch_bounds__(kTileX *kTileY) k_reduce_start(const __grid_constant__ DevState<T> S, int con) {
    reduce_start_body(S, con, bix_here());
}

// One block: combine (and clear) the partial slots, form dt as TimeStepSize does, then the
// bulk force.
template <class T> __device__ __forceinline__ void finalize_dt_body(const DevState<T> &S, int advance_time) {
    __shared__ unsigned long long smax[3][32];
    __shared__ long long ssum[32];
    unsigned long long m0 = 0, m1 = 0, m2 = 0;
    long long s = 0;
    for (int q = threadIdx.x; q < kBuckets; q += blockDim.x) {
        const unsigned long long a = S.part_max[3 * q], b = S.part_max[3 * q + 1], c = S.part_max[3 * q + 2];
        m0 = a > m0 ? a : m0;
        m1 = b > m1 ? b : m1;
        m2 = c > m2 ? c : m2;
        s += S.part_sum[q];
        S.part_max[3 * q] = S.part_max[3 * q + 1] = S.part_max[3 * q + 2] = 0;
        S.part_sum[q] = 0;
    }
    m0 = warp_max_u64(m0);
    m1 = warp_max_u64(m1);
    m2 = warp_max_u64(m2);
    s = warp_sum_i64(s);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        smax[0][w] = m0;
        smax[1][w] = m1;
        smax[2][w] = m2;
        ssum[w] = s;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const int nw = (blockDim.x + 31) / 32;
    for (int v = 1; v < nw; ++v) {
        m0 = smax[0][v] > m0 ? smax[0][v] : m0;
        m1 = smax[1][v] > m1 ? smax[1][v] : m1;
        m2 = smax[2][v] > m2 ? smax[2][v] : m2;
    }
    m0 = smax[0][0] > m0 ? smax[0][0] : m0;
    m1 = smax[1][0] > m1 ? smax[1][0] : m1;
    m2 = smax[2][0] > m2 ? smax[2][0] : m2;
    s = 0;
    for (int v = 0; v < nw; ++v) s += ssum[v];
    DevScalars *sc = S.sc;
    const Consts &k = S.k;
    const unsigned long long inf_bits = 0x7FF0000000000000ull;
    if (m0 >= inf_bits || m1 >= inf_bits || m2 >= inf_bits) sc->status |= STATUS_NONFINITE;
    const double M0 = __longlong_as_double((long long)m0);
    const double M1 = __longlong_as_double((long long)m1);
    const double M2 = __longlong_as_double((long long)m2);
    const double dtu1 = k.cfl_dx[0] / (k.sound + M0);
    const double dtu2 = k.cfl_dx[1] / (k.sound + M1);
    const double dtu3 = k.cfl_dx[2] / (k.sound + M2);
    const double dtu = min3d(dtu1, dtu2, dtu3);
    const double dt = min3d(1e8, dtu, k.dtv);
    sc->dt = dt;
    sc->rdt = 1.0 / dt;
    sc->dtf = (float)dt;
    sc->rdtf = (float)(1.0 / dt);
    sc->qdt = make_qrecip(dt);
    if (k.forcing) {
        const double ub = sc->nfluid > 0 ? ((double)s * FixedScale<T>::inv) / (double)sc->nfluid : 0.0;
        sc->ub = ub;
        sc->G = (k.u_target - ub) / dt;
        sc->Gf = (float)sc->G;
    }
    if (advance_time) {
        sc->nstep += 1;
        sc->time += 0.5 * dt;
        sc->time += 0.5 * dt;
    }
}
template <class T>
__global__ void __launch_bounds__(1024) k_finalize_dt(const __grid_constant__ DevState<T> S, int advance_time) {
    finalize_dt_body(S, advance_time);
}

// ---------------------------------------------------------------------------------------
// ghost fill (periodic x and z)
// ---------------------------------------------------------------------------------------

enum : uint8_t { GH_NONE = 0, GH_WRAP = 1, GH_COPY = 2 };

struct WrapJob {
    void *a[16];
    uint8_t face[16];
    uint8_t mode[16][2]; // per array, for x and for z: GH_NONE, GH_WRAP or GH_COPY
    int n;
};

// The halo exchange of one rank with itself, per axis and array:
//   GH_WRAP (periodic axis): ghost 0 <- cell C, ghost C+1 <- cell 1; faces: halo 0 <- face C,
//           halo C+2 <- face 2 (main.cpp:603-801, 1049-1631 with self-neighbours);
//   GH_COPY (bounded axis): zero-gradient ghost 0 <- cell 1, ghost C+1 <- cell C; faces:
//           halo 0 <- face 1, halo C+2 <- face C+1 (main.cpp:803-845, 1633-1698);
// over the interior of the other two axes.
// Ghost line r: first the (j, k) lines of x, then the (i, j) lines of z.  Its position is found
// once per line, in 32-bit arithmetic (line counts stay below 2^31), and serves every array.
struct WrapLine {
    int a, b; // (j, k) of an x line, (i, j) of a z line
    bool z;
};
__device__ __forceinline__ WrapLine wrap_line(const Geom &g, int r) {
    const int nx = g.C2 * g.C3;
    WrapLine L;
    L.z = r >= nx;
    const int u = L.z ? r - nx : r, w = L.z ? g.C1 : g.C2;
    const int hi = u / w;
    L.a = u - hi * w + 1;
    L.b = hi + 1;
    return L;
}
__host__ __device__ inline int wrap_lines(const Geom &g) { return g.C2 * g.C3 + g.C1 * g.C2; }
// The two ghosts of line L of array q.
template <class T> __device__ __forceinline__ void wrap_copy(const Geom &g, const WrapJob &J, int q, const WrapLine &L) {
    T *a = (T *)J.a[q];
    const int64_t n = J.face[q] ? g.nface() : g.ncell();
    auto cp = [&](int64_t dst, int64_t src) { a[ARK_CK(dst, n)] = a[ARK_CK(src, n)]; };
    if (!L.z) {
        const uint8_t m = J.mode[q][0];
        if (m == GH_NONE) return;
        const int j = L.a, k = L.b;
        if (J.face[q]) {
            cp(g.face(0, j, k), g.face(m == GH_WRAP ? g.C1 : 1, j, k));
            cp(g.face(g.C1 + 2, j, k), g.face(m == GH_WRAP ? 2 : g.C1 + 1, j, k));
        } else {
            cp(g.cell(0, j, k), g.cell(m == GH_WRAP ? g.C1 : 1, j, k));
            cp(g.cell(g.C1 + 1, j, k), g.cell(m == GH_WRAP ? 1 : g.C1, j, k));
        }
    } else {
        const uint8_t m = J.mode[q][1];
        if (m == GH_NONE) return;
        const int i = L.a, j = L.b;
        if (J.face[q]) {
            cp(g.face(i, j, 0), g.face(i, j, m == GH_WRAP ? g.C3 : 1));
            cp(g.face(i, j, g.C3 + 2), g.face(i, j, m == GH_WRAP ? 2 : g.C3 + 1));
        } else {
            cp(g.cell(i, j, 0), g.cell(i, j, m == GH_WRAP ? g.C3 : 1));
            cp(g.cell(i, j, g.C3 + 1), g.cell(i, j, m == GH_WRAP ? 1 : g.C3));
        }
    }
}

// One thread per line looping over the arrays (the ensemble's batched ghost fill, whose
// parallelism comes from the members).
template <class T> __device__ __forceinline__ void wrap_body_lines(const Geom &g, const WrapJob &J, int t) {
    if (t >= wrap_lines(g)) return;
    const WrapLine L = wrap_line(g, t);
    for (int q = 0; q < J.n; ++q) wrap_copy<T>(g, J, q, L);
}

// Thread x copies line x of array blockIdx.y.
template <class T> __global__ void k_wrap(Geom g, const __grid_constant__ WrapJob J) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= wrap_lines(g)) return;
    wrap_copy<T>(g, J, blockIdx.y, wrap_line(g, t));
}

// BoundaryConditions::alongX1/2/3 (source/BoundaryConditions.cpp:22-83) on one cell level,
// without the temperature.  axis 1: zero-gradient; axes 2, 3: periodic copy or no-slip
// (u = 0, density zero-gradient).  Copies are the same for rho and for rho - ro0.
template <class T> __global__ void k_boundary_fill(Geom g, Level<T> L, int axis, int periodic) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    T *a[4] = {L.u1, L.u2, L.u3, L.ro};
    const int64_t n = g.ncell();
    auto at = [&](int q, int64_t c) -> T & { return a[q][ARK_CK(c, n)]; };
    if (axis == 1) {
        if (t >= (int64_t)g.C2 * g.C3) return;
        const int j = (int)(t % g.C2) + 1, k = (int)(t / g.C2) + 1;
        for (int q = 0; q < 4; ++q) {
            at(q, g.cell(g.C1 + 1, j, k)) = at(q, g.cell(g.C1, j, k));
            at(q, g.cell(0, j, k)) = at(q, g.cell(1, j, k));
        }
    } else if (axis == 2) {
        if (t >= (int64_t)g.C1 * g.C3) return;
        const int i = (int)(t % g.C1) + 1, k = (int)(t / g.C1) + 1;
        const int64_t top = g.cell(i, g.C2 + 1, k), bot = g.cell(i, 0, k);
        for (int q = 0; q < 3; ++q) {
            at(q, top) = periodic ? at(q, g.cell(i, 1, k)) : (T)0;
            at(q, bot) = periodic ? at(q, g.cell(i, g.C2, k)) : (T)0;
        }
        at(3, top) = periodic ? at(3, g.cell(i, 1, k)) : at(3, g.cell(i, g.C2, k));
        at(3, bot) = periodic ? at(3, g.cell(i, g.C2, k)) : at(3, g.cell(i, 1, k));
    } else {
        if (t >= (int64_t)g.C1 * g.C2) return;
        const int i = (int)(t % g.C1) + 1, j = (int)(t / g.C1) + 1;
        const int64_t top = g.cell(i, j, g.C3 + 1), bot = g.cell(i, j, 0);
        for (int q = 0; q < 3; ++q) {
            at(q, top) = periodic ? at(q, g.cell(i, j, 1)) : (T)0;
            at(q, bot) = periodic ? at(q, g.cell(i, j, g.C3)) : (T)0;
        }
        at(3, top) = periodic ? at(3, g.cell(i, j, 1)) : at(3, g.cell(i, j, g.C3));
        at(3, bot) = periodic ? at(3, g.cell(i, j, g.C3)) : at(3, g.cell(i, j, 1));
    }
}

constexpr int kCellBX = 64, kCellBY = 2; // block shape of the one-cell-per-thread kernels

// ---------------------------------------------------------------------------------------
// viscous stress on one face (main.cpp:856-982), component by component
// ---------------------------------------------------------------------------------------

// one: the kernel was built for grid steps whose reciprocals are within a quarter ulp (div_rn)
template <class T>
__device__ __forceinline__ T sigma(uint8_t fw, uint8_t fc, T u_cw, T u_c, const K<T> &kk, int d) {
    if ((fw & FL_LT) && (fc & FL_LT)) return divq(kk.vis * (u_c - u_cw), kk.dx[d], kk.rdx[d], kk.q_dx[d]);
    if ((fw & FL_LT) && (fc & FL_GT)) return divq(kk.two_vis * (-u_cw), kk.dx[d], kk.rdx[d], kk.q_dx[d]);
    if ((fw & FL_GT) && (fc & FL_LT)) return divq(kk.two_vis * u_c, kk.dx[d], kk.rdx[d], kk.q_dx[d]);
    return (T)0;
}

// The stress force of one cell (main.cpp:995-1023): f_m = sum_d (sigma_md(+) - sigma_md(-))
// * ds_d * ro_c.  fln/un: flags and velocities of the six neighbours in the order
// (i-1, i+1, j-1, j+1, k-1, k+1).  FP64 evaluates every face stress exactly as the reference
// does; FP32 uses the equivalent coefficient form sigma = a_c u_c - a_w u_w per face.
// nuf (FP32 only; nullptr: none): eddy viscosity per face in the same order, added to vis.
template <class T>
__device__ __forceinline__ void stress_force(const uint8_t fln[6], const T un[6][3], uint8_t fl, const T uc[3],
                                             T ro_c, const K<T> &kk, T f[3], const T *nuf = nullptr) {
    if constexpr (!Storage<T>::deviation) {
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            T sw[3], se[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                sw[d] = sigma(fln[2 * d], fl, un[2 * d][m], uc[m], kk, d);
                se[d] = sigma(fl, fln[2 * d + 1], uc[m], un[2 * d + 1][m], kk, d);
            }
            f[m] = ((se[0] - sw[0]) * kk.ds[0] + (se[1] - sw[1]) * kk.ds[1] + (se[2] - sw[2]) * kk.ds[2]) * ro_c;
        }
    } else {
        if (!nuf && (fl & fln[0] & fln[1] & fln[2] & fln[3] & fln[4] & fln[5] & FL_LT)) {
            // a fluid cell among fluid neighbours: every coefficient is VIS / dx_d, the values the
            // general form below selects for such faces, in the same arithmetic
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                T acc = (T)0;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const T v = kk.vrdx[d];
                    const T sw = mad(v, uc[m], -(v * un[2 * d][m]));
                    const T se = mad(v, un[2 * d + 1][m], -(v * uc[m]));
                    acc = mad(se - sw, kk.ds[d], acc);
                }
                f[m] = acc * ro_c;
            }
            return;
        }
        T aw[6], ac[6]; // per face: coefficient on the cell behind (w) and ahead (c)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const T v = kk.vrdx[d];
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const uint8_t fw = side ? fl : fln[2 * d], fc = side ? fln[2 * d + 1] : fl;
                const bool wl = fw & FL_LT, wg = fw & FL_GT, cl = fc & FL_LT, cg = fc & FL_GT;
                const int q = 2 * d + side;
                const T vq = nuf ? mad(nuf[q], kk.rdx[d], v) : v;
                aw[q] = (wl && cl) ? vq : (wl && cg) ? (T)2 * vq : (T)0;
                ac[q] = (wl && cl) ? vq : (wg && cl) ? (T)2 * vq : (T)0;
            }
        }
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            T acc = (T)0;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const T sw = mad(ac[2 * d], uc[m], -(aw[2 * d] * un[2 * d][m]));
                const T se = mad(ac[2 * d + 1], un[2 * d + 1][m], -(aw[2 * d + 1] * uc[m]));
                acc = mad(se - sw, kk.ds[d], acc);
            }
            f[m] = acc * ro_c;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Phase1 (+ stress force, bulk force, UseForces, dt / bulk-flow partials)
// ---------------------------------------------------------------------------------------

// One face's values: pressure, density, velocity components.
template <class T> struct FaceVal { T p, ro, u[3]; };

// FP32 face density from face pressure: ro0 + p / c^2
__device__ __forceinline__ float face_ro(float p, const K<float> &kk) { return __fmaf_rn(p, kk.rc2, kk.ro0); }

// The bulk force on a cell's x1 momentum: f1 + (ro dvc) G (main.cpp:1013-1015 with the
// forcing term); FP32 fused.
__device__ __forceinline__ double bulk_force(double f1, double ro, const K<double> &kk, double G) {
    return f1 + (ro * kk.dvc) * G;
}
__device__ __forceinline__ float bulk_force(float f1, float ro, const K<float> &kk, float G) {
    return __fmaf_rn(ro * kk.dvc, G, f1);
}

// UseForces (main.cpp:1035-1041) in the FP32 form: u += (dt/2) f / (dvc ro) with rden = 1/ro
// already formed, one fused multiply-add per component.
__device__ __forceinline__ void use_forces_f32(float u[3], const float f[3], float dt, const K<float> &kk, float rden) {
    const float g2 = 0.5f * dt * kk.rdvc * rden;
#pragma unroll
    for (int m = 0; m < 3; ++m) u[m] = __fmaf_rn(g2, f[m], u[m]);
}

template <class T>
__device__ __forceinline__ FaceVal<T> load_face(const FaceSet<T> &F, int f, const K<T> &kk) {
    FaceVal<T> v;
    v.p = __ldg(F.p + f);
    if constexpr (Storage<T>::deviation) v.ro = face_ro(v.p, kk);
    else v.ro = __ldg(F.ro + f);
    v.u[0] = __ldg(F.u[0] + f);
    v.u[1] = __ldg(F.u[1] + f);
    v.u[2] = __ldg(F.u[2] + f);
    return v;
}

// The conservative half step of one fluid cell (main.cpp:530-551) from its six faces
// lo[d] (west/south/bottom) and hi[d] (east/north/top).  ro_c: density (FP64) or deviation.
template <class T>
__device__ __forceinline__ void half_step(const FaceVal<T> lo[3], const FaceVal<T> hi[3], T ro_c, const T uc[3],
                                          T dt, const K<T> &kk, T &ro_cn, T ucn[3], T &rden_out) {
    if constexpr (!Storage<T>::deviation) {
        // new density (main.cpp:530-533)
        ro_cn = divq(ro_c * kk.dvc - (T)0.5 * dt * ((hi[0].ro * hi[0].u[0] - lo[0].ro * lo[0].u[0]) * kk.ds[0] +
                                                    (hi[1].ro * hi[1].u[1] - lo[1].ro * lo[1].u[1]) * kk.ds[1] +
                                                    (hi[2].ro * hi[2].u[2] - lo[2].ro * lo[2].u[2]) * kk.ds[2]),
                     kk.dvc, kk.rdvc, kk.q_dvc);
        // momentum (main.cpp:536-551): the flux of u_m through faces normal to d is
        // (ro*u_m)*u_d, plus p when m == d
        // one reciprocal serves the three momentum quotients (and UseForces, whose divisor
        // dvc*ro_cn is the same product)
        const T den = ro_cn * kk.dvc;
        const T rden = recip(den);
        rden_out = rden;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            T fx[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (m == d)
                    fx[d] = (hi[d].ro * hi[d].u[m] * hi[d].u[d] + hi[d].p) - (lo[d].ro * lo[d].u[m] * lo[d].u[d] + lo[d].p);
                else
                    fx[d] = hi[d].ro * hi[d].u[m] * hi[d].u[d] - lo[d].ro * lo[d].u[m] * lo[d].u[d];
            }
            ucn[m] = divr(ro_c * uc[m] * kk.dvc - (T)0.5 * dt * (fx[0] * kk.ds[0] + fx[1] * kk.ds[1] + fx[2] * kk.ds[2]),
                          den, rden);
        }
    } else {
        // the same balance with the volume divided out and the density as a deviation:
        // ro'_new = ro'_c - (dt/2/dvc) sum_d (rho u_d)|_faces ds_d.  The momentum flux of u_m
        // through a face is the face's mass flux times u_m; products fused with the sums.
        const T h = (T)0.5 * dt * kk.rdvc;
        T mh[3], ml[3]; // mass flux through the hi and lo face of each direction
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            mh[d] = hi[d].ro * hi[d].u[d];
            ml[d] = lo[d].ro * lo[d].u[d];
        }
        T sm = (mh[0] - ml[0]) * kk.ds[0];
        sm = mad(mh[1] - ml[1], kk.ds[1], sm);
        sm = mad(mh[2] - ml[2], kk.ds[2], sm);
        ro_cn = mad(-h, sm, ro_c);
        const T rden = (T)1 / (kk.ro0 + ro_cn);
        rden_out = rden;
        const T ro_cf = kk.ro0 + ro_c;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            T fx[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                fx[d] = mad(mh[d], hi[d].u[m], -(ml[d] * lo[d].u[m]));
                if (m == d) fx[d] += hi[d].p - lo[d].p;
            }
            T sx = fx[0] * kk.ds[0];
            sx = mad(fx[1], kk.ds[1], sx);
            sx = mad(fx[2], kk.ds[2], sx);
            ucn[m] = mad(-h, sx, ro_cf * uc[m]) * rden;
        }
    }
}

// Phase1 over one tile (kTileX x kTileY cells, kTileK planes), marching up in k: the face
// below a cell is the face above the previous one, and the stress's lower neighbour is the
// previous centre, so both stay in registers.  src: the level read as "Con" (the previous
// "nCon"); dst: the level written as "nCon"; faces of generation fcur.  MODE adds the
// stress force (+ bulk force) of the src level, UseForces, and the partials of the next
// step's dt (max |u| of dst) or bulk flow (sum of u1 of dst).
template <class T, int MODE>
__device__ __forceinline__ void phase1_march_body(const DevState<T> &S, int src, int dst, int fcur, const BIx &bx) {
    constexpr bool DEV = Storage<T>::deviation;
    constexpr bool STRESS = MODE & P1_STRESS;
    const Geom g = S.g;
    const int i = bx.x * kTileX + threadIdx.x + 1;
    const int j = bx.y * kTileY + threadIdx.y + 1;
    const int k0 = bx.z * kTileK + 1;
    const int k1 = k0 + kTileK - 1 < g.C3 ? k0 + kTileK - 1 : g.C3;
    unsigned long long m0 = 0, m1 = 0, m2 = 0;
    long long rsum = 0;
    if (i <= g.C1 && j <= g.C2 && ARK_CK_IN(k0, 1, g.C3)) {
        const K<T> &kk = kconst<T>(S.k);
        const T dt = sc_dt<T>(S.sc);
        const T *__restrict__ sro = S.lv[src].ro;
        const T *__restrict__ su1 = S.lv[src].u1;
        const T *__restrict__ su2 = S.lv[src].u2;
        const T *__restrict__ su3 = S.lv[src].u3;
        T *__restrict__ dro = S.lv[dst].ro;
        T *__restrict__ du1 = S.lv[dst].u1;
        T *__restrict__ du2 = S.lv[dst].u2;
        T *__restrict__ du3 = S.lv[dst].u3;
        const uint8_t *__restrict__ flags = S.flags;
        const int cs1 = (int)g.cs1, cs2 = (int)g.cs2, fs1 = (int)g.fs1, fs2 = (int)g.fs2;
        const T G = (MODE & P1_BULK) ? sc_G<T>(S.sc) : (T)0;
        int c = g.ci(i, j, k0), fw = g.fi(i, j, k0);
        FaceVal<T> bot = load_face(S.fc[fcur][2], fw, kk);
        // stress state carried up the column: the cell below and the current cell
        uint8_t fdn = 0, fcen = 0;
        T udn[3] = {(T)0, (T)0, (T)0}, ucen[3] = {(T)0, (T)0, (T)0}, rocen = (T)0;
        if (STRESS) {
            fdn = flags[c - cs2];
            udn[0] = su1[c - cs2];
            udn[1] = su2[c - cs2];
            udn[2] = su3[c - cs2];
            fcen = flags[c];
            ucen[0] = su1[c];
            ucen[1] = su2[c];
            ucen[2] = su3[c];
            rocen = sro[c];
        }
        for (int k = k0; k <= k1; ++k, c += cs2, fw += fs2) {
            uint8_t fl;
            T ro_c, uc[3];
            if (STRESS) {
                fl = fcen;
                ro_c = rocen;
                uc[0] = ucen[0];
                uc[1] = ucen[1];
                uc[2] = ucen[2];
            } else {
                fl = flags[c];
                ro_c = sro[c];
                uc[0] = su1[c];
                uc[1] = su2[c];
                uc[2] = su3[c];
            }
            const FaceVal<T> top = load_face(S.fc[fcur][2], fw + fs2, kk);
            T ro_cn, ucn[3], rden = (T)0;
            if (fl & FL_LT) {
                FaceVal<T> lo[3], hi[3];
                lo[0] = load_face(S.fc[fcur][0], fw, kk);
                hi[0] = load_face(S.fc[fcur][0], fw + 1, kk);
                lo[1] = load_face(S.fc[fcur][1], fw, kk);
                hi[1] = load_face(S.fc[fcur][1], fw + fs1, kk);
                lo[2] = bot;
                hi[2] = top;
                half_step(lo, hi, ro_c, uc, dt, kk, ro_cn, ucn, rden);
            } else {
                ucn[0] = ucn[1] = ucn[2] = (T)0;
                ro_cn = DEV ? (T)0 : kk.ro0;
            }
            T f[3] = {(T)0, (T)0, (T)0};
            if (STRESS) {
                // the cell above: next iteration's centre
                const uint8_t fup = flags[c + cs2];
                const T uup[3] = {su1[c + cs2], su2[c + cs2], su3[c + cs2]};
                if (fl & FL_EQ0) {
                    const int nb[4] = {c - 1, c + 1, c - cs1, c + cs1};
                    uint8_t fln[6];
                    T un[6][3];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        fln[q] = flags[nb[q]];
                        un[q][0] = su1[nb[q]];
                        un[q][1] = su2[nb[q]];
                        un[q][2] = su3[nb[q]];
                    }
                    fln[4] = fdn;
                    fln[5] = fup;
#pragma unroll
                    for (int m = 0; m < 3; ++m) {
                        un[4][m] = udn[m];
                        un[5][m] = uup[m];
                    }
                    const T ro_cf = DEV ? kk.ro0 + ro_c : ro_c;
                    stress_force(fln, un, fl, uc, ro_cf, kk, f);
                    if (MODE & P1_BULK) f[0] = bulk_force(f[0], ro_cf, kk, G);
                }
                S.f[0][c] = f[0];
                S.f[1][c] = f[1];
                S.f[2][c] = f[2];
                fdn = fl;
                udn[0] = uc[0];
                udn[1] = uc[1];
                udn[2] = uc[2];
                fcen = fup;
                ucen[0] = uup[0];
                ucen[1] = uup[1];
                ucen[2] = uup[2];
                if (k < k1) rocen = sro[c + cs2];
            } else if (MODE & P1_FORCES) {
                f[0] = __ldg(S.f[0] + c);
                f[1] = __ldg(S.f[1] + c);
                f[2] = __ldg(S.f[2] + c);
            }
            if ((MODE & P1_FORCES) && (fl & FL_EQ0)) {
                // UseForces (main.cpp:1035-1041); a fluid cell always went through half_step,
                // so rden is 1/(dvc*ro_cn) (FP64) or 1/(ro0 + ro'_cn) (FP32)
                if constexpr (!DEV) {
                    const T den = kk.dvc * ro_cn;
#pragma unroll
                    for (int m = 0; m < 3; ++m) ucn[m] = divr(ro_cn * kk.dvc * ucn[m] + (T)0.5 * dt * f[m], den, rden);
                } else {
                    use_forces_f32(ucn, f, dt, kk, rden);
                }
            }
            dro[c] = ro_cn;
            du1[c] = ucn[0];
            du2[c] = ucn[1];
            du3[c] = ucn[2];
            if (MODE & P1_RMAX) {
                const unsigned long long b0 = abs_key(ucn[0]), b1 = abs_key(ucn[1]), b2 = abs_key(ucn[2]);
                m0 = b0 > m0 ? b0 : m0;
                m1 = b1 > m1 ? b1 : m1;
                m2 = b2 > m2 ? b2 : m2;
            }
            if ((MODE & P1_RSUM) && (fl & FL_EQ0)) rsum += fixed_sum_term(ucn[0]);
            bot = top;
        }
    }
    if (MODE & (P1_RMAX | P1_RSUM)) tile_store(S, bx, (MODE & P1_RMAX) != 0, (MODE & P1_RSUM) != 0, m0, m1, m2, rsum);
}
template <class T, int MODE>
__global__ void __launch_bounds__(kTileX *kTileY)
    k_phase1(const __grid_constant__ DevState<T> S, int src, int dst, int fcur) {
    phase1_march_body<T, MODE>(S, src, dst, fcur, bix_here());
}

// Phase1 with one cell per thread (grid z over all planes): fewer registers than the marching
// kernel, so more warps in flight.  Same arithmetic and outputs as k_phase1.
template <class T, int MODE>
__device__ __forceinline__ void phase1_cell_body(const DevState<T> &S, int src, int dst, int fcur, const BIx &bx) {
    constexpr bool DEV = Storage<T>::deviation;
    const Geom g = S.g;
    const int i = bx.x * kTileX + threadIdx.x + 1;
    const int j = bx.y * kTileY + threadIdx.y + 1;
    const int k = bx.z + 1;
    unsigned long long m0 = 0, m1 = 0, m2 = 0;
    long long rsum = 0;
    if (i <= g.C1 && j <= g.C2 && ARK_CK_IN(k, 1, g.C3)) {
        const K<T> &kk = kconst<T>(S.k);
        const T dt = sc_dt<T>(S.sc);
        const T *__restrict__ sro = S.lv[src].ro;
        const T *__restrict__ su1 = S.lv[src].u1;
        const T *__restrict__ su2 = S.lv[src].u2;
        const T *__restrict__ su3 = S.lv[src].u3;
        const uint8_t *__restrict__ flags = S.flags;
        const int cs1 = (int)g.cs1, cs2 = (int)g.cs2, fs1 = (int)g.fs1, fs2 = (int)g.fs2;
        const int c = g.ci(i, j, k), fw = g.fi(i, j, k);
        const uint8_t fl = flags[c];
        const T ro_c = sro[c];
        const T uc[3] = {su1[c], su2[c], su3[c]};
        T ro_cn, ucn[3], rden = (T)0;
        if (fl & FL_LT) {
            FaceVal<T> lo[3], hi[3];
            lo[0] = load_face(S.fc[fcur][0], fw, kk);
            hi[0] = load_face(S.fc[fcur][0], fw + 1, kk);
            lo[1] = load_face(S.fc[fcur][1], fw, kk);
            hi[1] = load_face(S.fc[fcur][1], fw + fs1, kk);
            lo[2] = load_face(S.fc[fcur][2], fw, kk);
            hi[2] = load_face(S.fc[fcur][2], fw + fs2, kk);
            half_step(lo, hi, ro_c, uc, dt, kk, ro_cn, ucn, rden);
        } else {
            ucn[0] = ucn[1] = ucn[2] = (T)0;
            ro_cn = DEV ? (T)0 : kk.ro0;
        }
        T f[3] = {(T)0, (T)0, (T)0};
        if (MODE & P1_STRESS) {
            if (fl & FL_EQ0) {
                const int nb[6] = {c - 1, c + 1, c - cs1, c + cs1, c - cs2, c + cs2};
                uint8_t fln[6];
                T un[6][3];
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    fln[q] = flags[nb[q]];
                    un[q][0] = su1[nb[q]];
                    un[q][1] = su2[nb[q]];
                    un[q][2] = su3[nb[q]];
                }
                const T ro_cf = DEV ? kk.ro0 + ro_c : ro_c;
                if (MODE & P1_NUT) {
                    // eddy viscosity on each face: the mean of the two cells' nu_t
                    const T nc = S.nut[c];
                    T nuf[6];
#pragma unroll
                    for (int q = 0; q < 6; ++q) nuf[q] = (T)0.5 * (nc + S.nut[nb[q]]);
                    stress_force(fln, un, fl, uc, ro_cf, kk, f, nuf);
                } else {
                    stress_force(fln, un, fl, uc, ro_cf, kk, f);
                }
                if (MODE & P1_BULK) f[0] = bulk_force(f[0], ro_cf, kk, sc_G<T>(S.sc));
            }
            S.f[0][c] = f[0];
            S.f[1][c] = f[1];
            S.f[2][c] = f[2];
        } else if (MODE & P1_FORCES) {
            f[0] = __ldg(S.f[0] + c);
            f[1] = __ldg(S.f[1] + c);
            f[2] = __ldg(S.f[2] + c);
        }
        if ((MODE & P1_FORCES) && (fl & FL_EQ0)) {
            // UseForces (main.cpp:1035-1041), with the reciprocal half_step formed
            if constexpr (!DEV) {
                const T den = kk.dvc * ro_cn;
#pragma unroll
                for (int m = 0; m < 3; ++m) ucn[m] = divr(ro_cn * kk.dvc * ucn[m] + (T)0.5 * dt * f[m], den, rden);
            } else {
                use_forces_f32(ucn, f, dt, kk, rden);
            }
        }
        S.lv[dst].ro[c] = ro_cn;
        S.lv[dst].u1[c] = ucn[0];
        S.lv[dst].u2[c] = ucn[1];
        S.lv[dst].u3[c] = ucn[2];
        if (MODE & P1_RMAX) {
            m0 = abs_key(ucn[0]);
            m1 = abs_key(ucn[1]);
            m2 = abs_key(ucn[2]);
        }
        if ((MODE & P1_RSUM) && (fl & FL_EQ0)) rsum = fixed_sum_term(ucn[0]);
    }
    if (MODE & (P1_RMAX | P1_RSUM)) tile_store(S, bx, (MODE & P1_RMAX) != 0, (MODE & P1_RSUM) != 0, m0, m1, m2, rsum);
}
template <class T, int MODE>
__global__ void __launch_bounds__(kTileX *kTileY)
    k_phase1_cell(const __grid_constant__ DevState<T> S, int src, int dst, int fcur) {
    phase1_cell_body<T, MODE>(S, src, dst, fcur, bix_here());
}

// ---------------------------------------------------------------------------------------
// Phase1 with each face's quantities computed once (FP64 contexts, bound by the FP64 pipe).
// The one-cell kernel evaluates the mass flux, the three momentum fluxes and (with the
// stress) the three face stresses of every face twice, once for each cell beside it.  Here a
// block owns a 64 x 4 tile of columns and marches up a chunk of planes: per plane, each thread
// evaluates the x and y faces below its cell (the last column and row of the tile also the
// faces above) into shared memory and the z face above its cell in registers (the face below
// is the previous plane's face above).  Every face value is the expression the one-cell kernel
// evaluates, in the same operation order, and every cell combines them in the same order, so
// the results are bit-identical (tested).
// ---------------------------------------------------------------------------------------
namespace fcs {
constexpr int SX = 64, SY = 4;
template <class T> struct FaceQ {
    T mf, mom[3], sig[3];
};
// dynamic shared memory of k_phase1_faces: two generations of SY x (SX + 1) x faces and
// (SY + 1) x SX y faces
template <class T> constexpr int face_smem() { return 2 * (SY * (SX + 1) + (SY + 1) * SX) * (int)sizeof(FaceQ<T>); }

// The quantities of the face normal to d with values V: the mass flux ro u_d, the momentum
// fluxes (ro u_m) u_d (+ p when m == d) of half_step, and StressTensor's sigma_md between the
// cell below (flags flo, velocity ulo) and the cell above (fhi, uhi).
template <class T, bool STRESS>
__device__ __forceinline__ FaceQ<T> face_q(const FaceVal<T> &V, int d, uint8_t flo, uint8_t fhi, const T ulo[3],
                                           const T uhi[3], const K<T> &kk) {
    FaceQ<T> q;
    q.mf = V.ro * V.u[d];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        q.mom[m] = (m == d) ? V.ro * V.u[m] * V.u[d] + V.p : V.ro * V.u[m] * V.u[d];
        q.sig[m] = STRESS ? sigma(flo, fhi, ulo[m], uhi[m], kk, d) : (T)0;
    }
    return q;
}

template <class T, int MODE>
__global__ void __launch_bounds__(SX *SY, 3) k_phase1_faces(const __grid_constant__ DevState<T> S, int src, int dst, int fcur, int kch) {
    static_assert(!Storage<T>::deviation, "face-centric Phase1: FP64 storage form");
    constexpr bool STRESS = (MODE & P1_STRESS) != 0;
    // two generations of a plane's x and y face quantities (face_smem bytes), alternating by
    // plane: a thread may write plane k+1's while others still read plane k's, and the barrier
    // of plane k+1 keeps plane k+2's writes behind every read of plane k, so one barrier per
    // plane suffices
    extern __shared__ __align__(16) unsigned char fcs_sm[];
    typedef FaceQ<T> RowX[SX + 1];
    typedef FaceQ<T> RowY[SX];
    RowX *const FxAll = reinterpret_cast<RowX *>(fcs_sm);
    RowY *const FyAll = reinterpret_cast<RowY *>(fcs_sm + 2 * SY * sizeof(RowX));
    const Geom g = S.g;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i = blockIdx.x * SX + tx + 1, j = blockIdx.y * SY + ty + 1;
    const int k0 = blockIdx.z * kch + 1;
    const int k1 = k0 + kch - 1 < g.C3 ? k0 + kch - 1 : g.C3;
    const bool valid = i <= g.C1 && j <= g.C2 && ARK_CK_IN(k0, 1, g.C3);
    const int ilast = blockIdx.x * SX + SX < g.C1 ? blockIdx.x * SX + SX : g.C1;
    const int jlast = blockIdx.y * SY + SY < g.C2 ? blockIdx.y * SY + SY : g.C2;
    const K<T> &kk = kconst<T>(S.k);
    const T dt = sc_dt<T>(S.sc);
    const T G = (MODE & P1_BULK) ? sc_G<T>(S.sc) : (T)0;
    const Level<T> L = S.lv[src];
    const uint8_t *__restrict__ flags = S.flags;
    const int cs1 = (int)g.cs1, cs2 = (int)g.cs2, fs1 = (int)g.fs1, fs2 = (int)g.fs2;
    const T zero3[3] = {(T)0, (T)0, (T)0};
    auto cellu = [&](int c, T u[3]) {
        u[0] = L.u1[c];
        u[1] = L.u2[c];
        u[2] = L.u3[c];
    };
    unsigned long long m0 = 0, m1 = 0, m2 = 0;
    long long rsum = 0;
    FaceQ<T> zlo = {};
    uint8_t fl = 0;
    T uc[3] = {(T)0, (T)0, (T)0};
    if (valid) {
        const int c = g.ci(i, j, k0), f = g.fi(i, j, k0);
        fl = flags[c];
        cellu(c, uc);
        T ud[3];
        if (STRESS) cellu(c - cs2, ud);
        zlo = face_q<T, STRESS>(load_face(S.fc[fcur][2], f, kk), 2, STRESS ? flags[c - cs2] : 0, fl, STRESS ? ud : zero3,
                                uc, kk);
    }
    for (int k = k0; k <= k1; ++k) {
        RowX *const Fx = FxAll + ((k - k0) & 1) * SY;
        RowY *const Fy = FyAll + ((k - k0) & 1) * (SY + 1);
        FaceQ<T> zhi = {};
        uint8_t flu = 0;
        T uu[3] = {(T)0, (T)0, (T)0};
        const int c = valid ? g.ci(i, j, k) : 0, f = valid ? g.fi(i, j, k) : 0;
        if (valid) {
            T un[3] = {(T)0, (T)0, (T)0};
            uint8_t fn = 0;
            if (STRESS) {
                fn = flags[c - 1];
                cellu(c - 1, un);
            }
            Fx[ty][tx] = face_q<T, STRESS>(load_face(S.fc[fcur][0], f, kk), 0, fn, fl, un, uc, kk);
            if (i == ilast) {
                if (STRESS) {
                    fn = flags[c + 1];
                    cellu(c + 1, un);
                }
                Fx[ty][tx + 1] = face_q<T, STRESS>(load_face(S.fc[fcur][0], f + 1, kk), 0, fl, fn, uc, un, kk);
            }
            if (STRESS) {
                fn = flags[c - cs1];
                cellu(c - cs1, un);
            }
            Fy[ty][tx] = face_q<T, STRESS>(load_face(S.fc[fcur][1], f, kk), 1, fn, fl, un, uc, kk);
            if (j == jlast) {
                if (STRESS) {
                    fn = flags[c + cs1];
                    cellu(c + cs1, un);
                }
                Fy[ty + 1][tx] = face_q<T, STRESS>(load_face(S.fc[fcur][1], f + fs1, kk), 1, fl, fn, uc, un, kk);
            }
            flu = flags[c + cs2];
            cellu(c + cs2, uu);
            zhi = face_q<T, STRESS>(load_face(S.fc[fcur][2], f + fs2, kk), 2, fl, flu, uc, uu, kk);
        }
        __syncthreads();
        if (valid) {
            const FaceQ<T> &Lx = Fx[ty][tx], &Hx = Fx[ty][tx + 1], &Ly = Fy[ty][tx], &Hy = Fy[ty + 1][tx];
            const T ro_c = L.ro[c];
            T ro_cn, ucn[3];
            QRecip qden = {0u, 0u, -100000, 0u};
            if (fl & FL_LT) {
                // half_step (main.cpp:530-551) over the face quantities
                ro_cn = divq(ro_c * kk.dvc - (T)0.5 * dt * ((Hx.mf - Lx.mf) * kk.ds[0] + (Hy.mf - Ly.mf) * kk.ds[1] +
                                                            (zhi.mf - zlo.mf) * kk.ds[2]),
                             kk.dvc, kk.rdvc, kk.q_dvc);
                // one reciprocal of the divisor ro_cn dvc serves the three momentum quotients and
                // UseForces' three, whose divisor dvc ro_cn is the same product
                const T den = ro_cn * kk.dvc;
                qden = qrecip_var(den);
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    const T fx0 = Hx.mom[m] - Lx.mom[m], fx1 = Hy.mom[m] - Ly.mom[m], fx2 = zhi.mom[m] - zlo.mom[m];
                    ucn[m] = qdiv_v(ro_c * uc[m] * kk.dvc - (T)0.5 * dt * (fx0 * kk.ds[0] + fx1 * kk.ds[1] + fx2 * kk.ds[2]),
                                    den, qden);
                }
            } else {
                ucn[0] = ucn[1] = ucn[2] = (T)0;
                ro_cn = kk.ro0;
            }
            T fv[3] = {(T)0, (T)0, (T)0};
            if (STRESS) {
                if (fl & FL_EQ0) {
#pragma unroll
                    for (int m = 0; m < 3; ++m)
                        fv[m] = ((Hx.sig[m] - Lx.sig[m]) * kk.ds[0] + (Hy.sig[m] - Ly.sig[m]) * kk.ds[1] +
                                 (zhi.sig[m] - zlo.sig[m]) * kk.ds[2]) *
                                ro_c;
                    if (MODE & P1_BULK) fv[0] = bulk_force(fv[0], ro_c, kk, G);
                }
                S.f[0][c] = fv[0];
                S.f[1][c] = fv[1];
                S.f[2][c] = fv[2];
            } else if (MODE & P1_FORCES) {
                fv[0] = __ldg(S.f[0] + c);
                fv[1] = __ldg(S.f[1] + c);
                fv[2] = __ldg(S.f[2] + c);
            }
            if ((MODE & P1_FORCES) && (fl & FL_EQ0)) {
                // UseForces (main.cpp:1035-1041)
                const T den = kk.dvc * ro_cn;
#pragma unroll
                for (int m = 0; m < 3; ++m) ucn[m] = qdiv_v(ro_cn * kk.dvc * ucn[m] + (T)0.5 * dt * fv[m], den, qden);
            }
            S.lv[dst].ro[c] = ro_cn;
            S.lv[dst].u1[c] = ucn[0];
            S.lv[dst].u2[c] = ucn[1];
            S.lv[dst].u3[c] = ucn[2];
            if (MODE & P1_RMAX) {
                const unsigned long long b0 = abs_key(ucn[0]), b1 = abs_key(ucn[1]), b2 = abs_key(ucn[2]);
                m0 = b0 > m0 ? b0 : m0;
                m1 = b1 > m1 ? b1 : m1;
                m2 = b2 > m2 ? b2 : m2;
            }
            if ((MODE & P1_RSUM) && (fl & FL_EQ0)) rsum += fixed_sum_term(ucn[0]);
        }
        zlo = zhi;
        fl = flu;
        uc[0] = uu[0];
        uc[1] = uu[1];
        uc[2] = uu[2];
    }
    if (MODE & (P1_RMAX | P1_RSUM)) {
        const BIx bx = {(int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z, (int)gridDim.x, (int)gridDim.y};
        tile_store<T, SX * SY>(S, bx, (MODE & P1_RMAX) != 0, (MODE & P1_RSUM) != 0, m0, m1, m2, rsum);
    }
}
} // namespace fcs

// StressTensor's face stresses into the sigm arrays (kept only on request), faces normal
// to d with index 1..C_d+1 along d (main.cpp:856-982).
template <class T> __global__ void k_stress_faces(DevState<T> S, int con, int d) {
    const Geom g = S.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    const int hi0 = g.C1 + (d == 0), hi1 = g.C2 + (d == 1), hi2 = g.C3 + (d == 2);
    if (i > hi0 || j > hi1 || k > hi2) return;
    const K<T> &kk = kconst<T>(S.k);
    const Level<T> L = S.lv[con];
    const int64_t c = g.cell(i, j, k);
    const int64_t cw = c - (d == 0 ? 1 : d == 1 ? g.cs1 : g.cs2);
    const uint8_t fc = S.flags[c], fw = S.flags[cw];
    const int64_t fi = g.face(i, j, k);
    T *s0 = d == 0 ? S.sig[0][0] : d == 1 ? S.sig[1][0] : S.sig[2][0];
    T *s1 = d == 0 ? S.sig[0][1] : d == 1 ? S.sig[1][1] : S.sig[2][1];
    T *s2 = d == 0 ? S.sig[0][2] : d == 1 ? S.sig[1][2] : S.sig[2][2];
    s0[fi] = sigma(fw, fc, L.u1[cw], L.u1[c], kk, d);
    s1[fi] = sigma(fw, fc, L.u2[cw], L.u2[c], kk, d);
    s2[fi] = sigma(fw, fc, L.u3[cw], L.u3[c], kk, d);
}

// StressTensor's force alone (the same device code the fused Phase1 uses).
template <class T> __global__ void k_stress_force(DevState<T> S, int con, int bulk) {
    constexpr bool DEV = Storage<T>::deviation;
    const Geom g = S.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.C1 || j > g.C2) return;
    const K<T> &kk = kconst<T>(S.k);
    const Level<T> L = S.lv[con];
    const int64_t c = g.cell(i, j, k);
    const uint8_t fl = S.flags[c];
    T f[3] = {(T)0, (T)0, (T)0};
    if (fl & FL_EQ0) {
        const T ro_c = DEV ? kk.ro0 + L.ro[c] : L.ro[c];
        const T uc[3] = {L.u1[c], L.u2[c], L.u3[c]};
        const int64_t nb[6] = {c - 1, c + 1, c - g.cs1, c + g.cs1, c - g.cs2, c + g.cs2};
        uint8_t fln[6];
        T un[6][3];
        for (int q = 0; q < 6; ++q) {
            fln[q] = S.flags[nb[q]];
            un[q][0] = L.u1[nb[q]];
            un[q][1] = L.u2[nb[q]];
            un[q][2] = L.u3[nb[q]];
        }
        stress_force(fln, un, fl, uc, ro_c, kk, f);
        if (bulk) f[0] = bulk_force(f[0], ro_c, kk, sc_G<T>(S.sc));
    }
    S.f[0][c] = f[0];
    S.f[1][c] = f[1];
    S.f[2][c] = f[2];
}

// UseForces alone (main.cpp:1026-1045) on level ncon.
template <class T> __global__ void k_use_forces(DevState<T> S, int ncon) {
    constexpr bool DEV = Storage<T>::deviation;
    const Geom g = S.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.C1 || j > g.C2) return;
    const int64_t c = g.cell(i, j, k);
    if (!(S.flags[c] & FL_EQ0)) return;
    const K<T> &kk = kconst<T>(S.k);
    const T dt = sc_dt<T>(S.sc);
    const Level<T> L = S.lv[ncon];
    if constexpr (!DEV) {
        const T ro_cn = L.ro[c];
        const T den = kk.dvc * ro_cn;
        const T rden = recip(den);
        L.u1[c] = divr(ro_cn * kk.dvc * L.u1[c] + (T)0.5 * dt * S.f[0][c], den, rden);
        L.u2[c] = divr(ro_cn * kk.dvc * L.u2[c] + (T)0.5 * dt * S.f[1][c], den, rden);
        L.u3[c] = divr(ro_cn * kk.dvc * L.u3[c] + (T)0.5 * dt * S.f[2][c], den, rden);
    } else {
        T u[3] = {L.u1[c], L.u2[c], L.u3[c]};
        const T f[3] = {S.f[0][c], S.f[1][c], S.f[2][c]};
        use_forces_f32(u, f, dt, kk, recip(kk.ro0 + L.ro[c]));
        L.u1[c] = u[0];
        L.u2[c] = u[1];
        L.u3[c] = u[2];
    }
}

// ---------------------------------------------------------------------------------------
// Phase2: characteristic extrapolation, limiter, face update
// ---------------------------------------------------------------------------------------

// What one cell hands to its two faces: forward values (to face s+1) and backward values
// (to face s) of the invariant and the two tangential velocities.
template <class T> struct Ext { T rf, qb, af, ab, bf, bb; };

template <class T> struct SweepK {
    T sound, ro0, c2, rc2, roc, rroc, dt, rdt, dx, rdx;
    QRecip qc2, qroc, qdt, qdx; // FP64: the divisors for qdiv
};

// The gradient term of a limiter bound, (2 d) / dt + b / dx.  FP64: the two correctly rounded
// quotients summed, as the reference evaluates it, the first one with the factor 2 taken by its
// exponent (qdiv2); FP32: (2 d) * (1/dt) + b * (1/dx), fused.
__device__ __forceinline__ double grad_sum(double d, double b, const SweepK<double> &q) {
    return qdiv2(d, q.dt, q.rdt, q.qdt) + divq(b, q.dx, q.rdx, q.qdx);
}
__device__ __forceinline__ float grad_sum(float d, float b, const SweepK<float> &q) {
    return __fmaf_rn(2.f * d, q.rdt, b * q.rdx);
}

// One cell of a sweep (main.cpp:1756-1873 for x1; the x2 and x3 sweeps are the same with
// the axes permuted).  u1: the velocity component normal to the sweep, u2/u3: tangential.
// ro_cn/ro_c: density (FP64) or density deviation (FP32).  Q_USES_R selects the x1/x3 form
// of the Q-limiter source, 2*(r_cn - r_c)/dt (main.cpp:1804, 2321); the x2 sweep uses
// 2*(q_cn - q_c)/dt (main.cpp:2083).
// 2x - y.  The product 2x is exact, so one fused multiply-add rounds it exactly as the
// reference's separate multiply and subtract do (both precisions).
__device__ __forceinline__ double twice_minus(double x, double y) { return __fma_rn(2.0, x, -y); }
__device__ __forceinline__ float twice_minus(float x, float y) { return __fmaf_rn(2.f, x, -y); }

// The Riemann invariants of a face, R = u_n + p/(ro0 c) and Q = u_n - p/(ro0 c)
// (main.cpp:1790-1797).  The sweeps compute them once per face and hand them to the cell ahead.
template <class T> struct RQ { T r, q; };
template <class T> __device__ __forceinline__ RQ<T> face_rq(T u_n, T p, const SweepK<T> &q) {
    const T pf = divq(p, q.roc, q.rroc, q.qroc);
    RQ<T> v;
    v.r = u_n + pf;
    v.q = u_n - pf;
    return v;
}

// The extrapolation with the invariants of the forward (f) and backward (b) face given.
template <class T, bool Q_USES_R>
__device__ __forceinline__ Ext<T> extrapolate_rq(RQ<T> f, RQ<T> b, T u1_cn, T u1_c, T u2_f, T u2_b, T u2_cn, T u2_c,
                                                 T u3_f, T u3_b, T u3_cn, T u3_c, T ro_cn, T ro_c, const SweepK<T> &q) {
    constexpr bool DEV = Storage<T>::deviation;
    const T p_cn = DEV ? q.c2 * ro_cn : q.c2 * (ro_cn - q.ro0);
    const T p_c = DEV ? q.c2 * ro_c : q.c2 * (ro_c - q.ro0);
    const T pcn = divq(p_cn, q.roc, q.rroc, q.qroc), pc = divq(p_c, q.roc, q.rroc, q.qroc);

    // max + dt*g: mad rounds it exactly as written in FP64, fused in FP32
    const T r_f = f.r, r_b = b.r, r_cn = u1_cn + pcn, r_c = u1_c + pc;
    T r_fn = twice_minus(r_cn, r_b);
    const T q_f = f.q, q_b = b.q, q_cn = u1_cn - pcn, q_c = u1_c - pc;
    T q_bn = twice_minus(q_cn, q_f);

    T u2_fn = twice_minus(u2_cn, u2_b);
    T u2_bn = twice_minus(u2_cn, u2_f);
    T u3_fn = twice_minus(u3_cn, u3_b);
    T u3_bn = twice_minus(u3_cn, u3_f);

    const T gr = grad_sum(r_cn - r_c, (u1_cn + q.sound) * (r_f - r_b), q);
    const T gq = grad_sum(Q_USES_R ? (r_cn - r_c) : (q_cn - q_c), (u1_cn - q.sound) * (q_f - q_b), q);
    const T gu2 = grad_sum(u2_cn - u2_c, u1_cn * (u2_f - u2_b), q);
    const T gu3 = grad_sum(u3_cn - u3_c, u1_cn * (u3_f - u3_b), q);

    const T rmax = mad(q.dt, gr, max3d(r_f, r_c, r_b));
    const T rmin = mad(q.dt, gr, min3d(r_f, r_c, r_b));
    const T qmax = mad(q.dt, gq, max3d(q_f, q_c, q_b));
    const T qmin = mad(q.dt, gq, min3d(q_f, q_c, q_b));
    const T u2_max = mad(q.dt, gu2, max3d(u2_f, u2_c, u2_b));
    const T u2_min = mad(q.dt, gu2, min3d(u2_f, u2_c, u2_b));
    const T u3_max = mad(q.dt, gu3, max3d(u3_f, u3_c, u3_b));
    const T u3_min = mad(q.dt, gu3, min3d(u3_f, u3_c, u3_b));

    if (gt(r_fn, rmax)) r_fn = rmax;
    if (lt(r_fn, rmin)) r_fn = rmin;
    if (gt(q_bn, qmax)) q_bn = qmax;
    if (lt(q_bn, qmin)) q_bn = qmin;
    if (gt(u2_fn, u2_max)) u2_fn = u2_max;
    if (lt(u2_fn, u2_min)) u2_fn = u2_min;
    if (gt(u2_bn, u2_max)) u2_bn = u2_max;
    if (lt(u2_bn, u2_min)) u2_bn = u2_min;
    if (gt(u3_fn, u3_max)) u3_fn = u3_max;
    if (lt(u3_fn, u3_min)) u3_fn = u3_min;
    if (gt(u3_bn, u3_max)) u3_bn = u3_max;
    if (lt(u3_bn, u3_min)) u3_bn = u3_min;
    Ext<T> e;
    e.rf = r_fn;
    e.qb = q_bn;
    e.af = u2_fn;
    e.ab = u2_bn;
    e.bf = u3_fn;
    e.bb = u3_bn;
    return e;
}

// The same from the faces' normal velocities and pressures.
template <class T, bool Q_USES_R>
__device__ __forceinline__ Ext<T> extrapolate(T u1_f, T u1_b, T u1_cn, T u1_c, T u2_f, T u2_b, T u2_cn,
                                              T u2_c, T u3_f, T u3_b, T u3_cn, T u3_c, T ro_cn, T ro_c,
                                              T p_f, T p_b, const SweepK<T> &q) {
    return extrapolate_rq<T, Q_USES_R>(face_rq(u1_f, p_f, q), face_rq(u1_b, p_b, q), u1_cn, u1_c, u2_f, u2_b, u2_cn,
                                       u2_c, u3_f, u3_b, u3_cn, u3_c, ro_cn, ro_c, q);
}

// Half-step cell values a face update may need in its rarer branches (loaded on demand).
template <class T> struct NCell {
    const T *__restrict__ nN;
    const T *__restrict__ nA;
    const T *__restrict__ nB;
    const T *__restrict__ ro;
    int nc; // elements of a cell array (bounds-checked builds)
};

// The new face generation of one sweep direction.
template <class T> struct FaceOut {
    T *__restrict__ p;
    T *__restrict__ ro;
    T *__restrict__ n;
    T *__restrict__ a;
    T *__restrict__ b;
    int nf; // elements of a face array (bounds-checked builds)
};

// The new values of one face: pressure, density, normal and tangential velocities.
template <class T> struct FaceNew { T p, ro, n, a, b; };

// The half-step values (tangential velocities nA / nB, density ro) of the cell behind (0) and
// ahead (1) of a face that the rarer branches of a face update read: from the level in memory
// (the sweeps, loaded only in those branches) or from registers (NVals).
template <class T> struct NAt {
    const NCell<T> &N;
    int cb, cf;
    __device__ __forceinline__ T nA(int ahead) const { return N.nA[ahead ? cf : cb]; }
    __device__ __forceinline__ T nB(int ahead) const { return N.nB[ahead ? cf : cb]; }
    __device__ __forceinline__ T ro(int ahead) const { return N.ro[ahead ? cf : cb]; }
};
template <class T> struct NVals {
    T a[2], b[2], r[2];
    __device__ __forceinline__ T nA(int ahead) const { return a[ahead]; }
    __device__ __forceinline__ T nB(int ahead) const { return b[ahead]; }
    __device__ __forceinline__ T ro(int ahead) const { return r[ahead]; }
};

// Face update (main.cpp:1920-2008).  prev = the cell behind the face (index f-1), cur = the
// cell ahead (index f); V gives those cells' half-step values for the rarer branches; flb/flf
// their flags and ucb/ucf their half-step normal velocities.  uA_old/uB_old: the face's
// previous tangential velocities.  WALL_A_FROM_N: the x2 sweep takes the tangential u1 from
// u2nCon in its wall branches (main.cpp:2219, 2238).
template <class T, bool WALL_A_FROM_N, class NV>
__device__ __forceinline__ FaceNew<T> face_values_v(const NV &V, uint8_t flb, uint8_t flf, T ucb, T ucf, const Ext<T> &prev,
                                                    const Ext<T> &cur, T uA_old, T uB_old, const SweepK<T> &q) {
    constexpr bool DEV = Storage<T>::deviation;
    T un, pn, ro_n, ua, ub;
    if ((flb & FL_LT) && (flf & FL_LT)) {
        const T rn = prev.rf, qn = cur.qb;
        un = dhalf(rn + qn);
        pn = dhalf((rn - qn) * q.sound * q.ro0);
        ro_n = q.ro0 + divq(pn, q.c2, q.rc2, q.qc2);
        if (ge0(ucf) && ge0(ucb)) {
            ua = prev.af;
            ub = prev.bf;
        } else if (le0(ucf) && le0(ucb)) {
            ua = cur.ab;
            ub = cur.bb;
        } else if (ge0(ucb) && le0(ucf)) {
            if (gt(ucb, -ucf)) {
                ua = prev.af;
                ub = prev.bf;
            } else {
                ua = cur.ab;
                ub = cur.bb;
            }
        } else {
            ua = V.nA(1) + V.nA(0) - uA_old;
            ub = V.nB(1) + V.nB(0) - uB_old;
        }
    } else {
        un = (T)0;
        if ((flb & FL_GT) && (flf & FL_LT)) {
            if (le0(ucf)) {
                const T qn = cur.qb;
                pn = -qn * q.sound * q.ro0;
                ro_n = q.ro0 + divq(pn, q.c2, q.rc2, q.qc2);
                ua = cur.ab;
                ub = cur.bb;
            } else {
                ro_n = V.ro(1);
                pn = DEV ? ro_n * q.c2 : (ro_n - q.ro0) * q.c2;
                ua = WALL_A_FROM_N ? ucf : V.nA(1);
                ub = V.nB(1);
            }
        } else if ((flb & FL_LT) && (flf & FL_GT)) {
            if (ge0(ucb)) {
                const T rn = prev.rf;
                pn = rn * q.sound * q.ro0;
                ro_n = q.ro0 + divq(pn, q.c2, q.rc2, q.qc2);
                ua = prev.af;
                ub = prev.bf;
            } else {
                ro_n = V.ro(0);
                pn = DEV ? ro_n * q.c2 : (ro_n - q.ro0) * q.c2;
                ua = WALL_A_FROM_N ? ucb : V.nA(0);
                ub = V.nB(0);
            }
        } else {
            pn = (T)0;
            ro_n = q.ro0;
            ua = (T)0;
            ub = (T)0;
        }
    }
    FaceNew<T> v;
    v.p = pn;
    v.ro = ro_n;
    v.n = un;
    v.a = ua;
    v.b = ub;
    return v;
}
// cb / cf index the cells behind and ahead in the half-step level N
template <class T, bool WALL_A_FROM_N>
__device__ __forceinline__ FaceNew<T> face_values(const NCell<T> &N, int cb, int cf, uint8_t flb, uint8_t flf, T ucb,
                                                  T ucf, const Ext<T> &prev, const Ext<T> &cur, T uA_old, T uB_old,
                                                  const SweepK<T> &q) {
    return face_values_v<T, WALL_A_FROM_N>(NAt<T>{N, cb, cf}, flb, flf, ucb, ucf, prev, cur, uA_old, uB_old, q);
}

template <class T> __device__ __forceinline__ void face_store(const FaceOut<T> &W, int fc, const FaceNew<T> &v) {
    W.p[fc] = v.p;
    W.n[fc] = v.n;
    if (!Storage<T>::deviation) W.ro[fc] = v.ro;
    W.a[fc] = v.a;
    W.b[fc] = v.b;
}

// face_values stored into the new face generation at face fc
template <class T, bool WALL_A_FROM_N>
__device__ __forceinline__ void face_update(const NCell<T> &N, const FaceOut<T> &W, int cb, int cf, int fc,
                                            uint8_t flb, uint8_t flf, T ucb, T ucf, const Ext<T> &prev,
                                            const Ext<T> &cur, T uA_old, T uB_old, const SweepK<T> &q) {
    cb = ARK_CK(cb, N.nc);
    cf = ARK_CK(cf, N.nc);
    fc = ARK_CK(fc, W.nf);
    face_store(W, fc, face_values<T, WALL_A_FROM_N>(N, cb, cf, flb, flf, ucb, ucf, prev, cur, uA_old, uB_old, q));
}

template <class T>
__device__ __forceinline__ SweepK<T> sweep_consts(const DevState<T> &S, int d) {
    const KT<T> &k = kconst<T>(S.k);
    SweepK<T> q;
    q.sound = k.sound;
    q.ro0 = k.ro0;
    q.c2 = k.c2;
    q.rc2 = k.rc2;
    q.roc = k.roc;
    q.rroc = k.rroc;
    q.dt = sc_dt<T>(S.sc);
    q.rdt = sc_rdt<T>(S.sc);
    q.dx = k.dx[d];
    q.rdx = k.rdx[d];
    q.qc2 = k.q_c2;
    q.qroc = k.q_roc;
    q.qdx = k.q_dx[d];
    q.qdt = sc_qdt(S.sc);
    return q;
}

// Everything one cell of a sweep reads: its forward face (s+1), the half-step ("n") and
// old ("c") values of the cell, and its flags.  The backward face is the previous cell's
// forward face.
template <class T> struct SweepIn {
    T uN_f, uA_f, uB_f, p_f, nN, cN, nA, cA, nB, cB, nR, cR;
    uint8_t fl;
};

// The pointers of one sweep: old faces F*, cell levels c* ("Con") and n* ("nCon").
template <class T> struct SweepSrc {
    const T *__restrict__ FN;
    const T *__restrict__ FA;
    const T *__restrict__ FB;
    const T *__restrict__ FP;
    const T *__restrict__ cN;
    const T *__restrict__ nN;
    const T *__restrict__ cA;
    const T *__restrict__ nA;
    const T *__restrict__ cB;
    const T *__restrict__ nB;
    const T *__restrict__ cR;
    const T *__restrict__ nR;
    const uint8_t *__restrict__ fl;
    int nc, nf; // elements of a cell and of a face array (bounds-checked builds)
};

template <class T>
__device__ __forceinline__ SweepSrc<T> sweep_src(const DevState<T> &S, int con, int fcur, int ax) {
    const Level<T> Lc = S.lv[con], Ln = S.lv[con ^ 1];
    const FaceSet<T> F = S.fc[fcur][ax];
    const int a = ax == 0 ? 1 : 0, b = ax == 2 ? 1 : 2;
    const T *cu[3] = {Lc.u1, Lc.u2, Lc.u3}, *nu[3] = {Ln.u1, Ln.u2, Ln.u3};
    SweepSrc<T> r = {F.u[ax], F.u[a], F.u[b], F.p, cu[ax], nu[ax], cu[a], nu[a], cu[b], nu[b], Lc.ro, Ln.ro, S.flags,
                     (int)S.g.ncell(), (int)S.g.nface()};
    return r;
}

template <class T> __device__ __forceinline__ FaceOut<T> sweep_out(const DevState<T> &S, int fcur, int ax) {
    const FaceSet<T> W = S.fc[fcur ^ 1][ax];
    const int a = ax == 0 ? 1 : 0, b = ax == 2 ? 1 : 2;
    FaceOut<T> o = {W.p, W.ro, W.u[ax], W.u[a], W.u[b], (int)S.g.nface()};
    return o;
}

// cf: the flag index of the cell, when its values come from another cell (the x1 sweep's ghost
// positions, see xcell); -1: c itself
template <class T>
__device__ __forceinline__ void sweep_load(const SweepSrc<T> &R, int c, int ff, SweepIn<T> &x, int cf = -1) {
    cf = ARK_CK(cf < 0 ? c : cf, R.nc);
    c = ARK_CK(c, R.nc);
    ff = ARK_CK(ff, R.nf);
    x.uN_f = R.FN[ff];
    x.uA_f = R.FA[ff];
    x.uB_f = R.FB[ff];
    x.p_f = R.FP[ff];
    x.nN = R.nN[c];
    x.cN = R.cN[c];
    x.nA = R.nA[c];
    x.cA = R.cA[c];
    x.nB = R.nB[c];
    x.cB = R.cB[c];
    x.nR = R.nR[c];
    x.cR = R.cR[c];
    x.fl = R.fl[cf];
}

// The x1 sweep reads its line's ghost positions from the cells and faces whose images the ghost
// fill would copy there (k_wrap), so no ghost cell or halo face of x is read: position 0 is cell C1
// (periodic) or 1 (bounded, zero-gradient), position C1+1 cell 1 or C1; face 0 is face C1 and face
// C1+2 face 2 (periodic; a bounded x sweep overrides what it reads there).  The flags stay the
// ghost cells' own (the ghost fill never copies them).
__device__ __forceinline__ int xcell(int s, int C1, bool periodic) {
    return s == 0 ? (periodic ? C1 : 1) : s == C1 + 1 ? (periodic ? 1 : C1) : s;
}
__device__ __forceinline__ int xface(int s, int C1, bool periodic) {
    return !periodic ? s : s == 0 ? C1 : s == C1 + 2 ? 2 : s;
}
// The x3 sweep does the same along z (unless the z ghosts are a slab's halo): cell 0 is cell C3
// (periodic) or 1 (bounded), cell C3+1 cell 1 or C3; face 0 is face C3 or 1, face C3+2 face 2 or
// C3+1 (the ghost fill copies the adjacent face on a bounded z).
__device__ __forceinline__ int zcell(int s, int C3, bool periodic) { return xcell(s, C3, periodic); }
__device__ __forceinline__ int zface(int s, int C3, bool periodic) {
    return s == 0 ? (periodic ? C3 : 1) : s == C3 + 2 ? (periodic ? 2 : C3 + 1) : s;
}

// x1 sweep: one warp per (j,k) line, lanes on consecutive cells (coalesced), marching along
// i in chunks of 32 with the next chunk's loads issued before the current chunk is
// computed.  A face needs the forward values of the cell behind it: a shuffle from the
// neighbouring lane, or the carry from the previous chunk's last lane.  Old faces come from
// generation fcur, new faces go to fcur^1.

template <class T>
__device__ __forceinline__ void sweep_x_body(const DevState<T> &S, int con, int fcur, int glines, const BIx &bx) {
    const Geom g = S.g;
    const int lane = threadIdx.x & 31;
    const int nlines = g.C2 * g.C3;
    const int first = (bx.x * 4 + (threadIdx.x >> 5)) * glines; // the warp's first line
    if (first >= nlines) return;
    const int nl = nlines - first < glines ? nlines - first : glines;
    const int nd = g.C1 + 1, npos = g.C1 + 2; // cells 0..C1+1 of a line
    const int total = nl * npos;              // positions of the warp's stream
    const SweepSrc<T> R = sweep_src(S, con, fcur, 0);
    const FaceOut<T> W = sweep_out(S, fcur, 0);
    const NCell<T> N = {R.nN, R.nA, R.nB, R.nR, R.nc};
    const SweepK<T> q = sweep_consts(S, 0);
    const bool bounded = !S.k.periodic_x;
    // a lane's position: line li of the group, cell s, and the line's cell / face 0 indices
    // dc / db / df / dp: what the ghost positions add to the indices of the cell's values, its
    // backward and forward faces and the cell behind (xcell, xface), nonzero only at s = 0, 1, C1+1
    struct Pos {
        int li, s, c0, f0, dc, db, df, dp;
    };
    const bool px = S.k.periodic_x;
    const int x0 = xcell(0, g.C1, px), x1 = xcell(g.C1 + 1, g.C1, px) - (g.C1 + 1);
    auto deltas = [&](Pos &P) {
        const bool e0 = P.s == 0, e1 = P.s == g.C1 + 1;
        P.dc = e0 ? x0 : e1 ? x1 : 0;
        P.db = e0 && px ? g.C1 : 0;
        P.df = e1 && px ? -g.C1 : 0;
        P.dp = P.s == 1 ? x0 : 0;
    };
    auto locate = [&](Pos &P) {
        const int L = first + P.li;
        const int j = L % g.C2 + 1, k = L / g.C2 + 1;
        P.c0 = g.ci(0, j, k);
        P.f0 = g.fi(0, j, k);
    };
    auto advance = [&](Pos &P) { // 32 positions on
        P.s += 32;
        bool moved = false;
        while (P.s >= npos) {
            P.s -= npos;
            ++P.li;
            moved = true;
        }
        if (moved && P.li < nl) locate(P);
        deltas(P);
    };
    Pos cp;
    cp.li = lane / npos;
    cp.s = lane - cp.li * npos;
    cp.c0 = cp.f0 = 0;
    if (cp.li < nl) locate(cp);
    deltas(cp);
    Ext<T> carry = {};
    T carry_u = 0;
    uint8_t carry_fl = 0;
    SweepIn<T> cur = {}, nxt = {};
    T uA_b = 0, uB_b = 0, nuA_b = 0, nuB_b = 0;
    // the invariants of a cell's backward face are those the cell behind computed for its
    // forward face: a shuffle from the neighbouring lane, across chunks the carry from the last
    // lane, and for cell 0 of a line the face 0 itself
    RQ<T> carry_rq = {(T)0, (T)0};
    if (cp.li < nl) {
        sweep_load(R, cp.c0 + cp.s + cp.dc, cp.f0 + cp.s + 1 + cp.df, cur, cp.c0 + cp.s);
        uA_b = R.FA[ARK_CK(cp.f0 + cp.s + cp.db, R.nf)];
        uB_b = R.FB[ARK_CK(cp.f0 + cp.s + cp.db, R.nf)];
    }
    for (int p0 = 0; p0 < total; p0 += 32) {
        const bool act = cp.li < nl;
        const int s = cp.s, c0 = cp.c0, f0 = cp.f0, dc = cp.dc, db = cp.db, dp = cp.dp;
        Pos np = cp;
        advance(np);
        if (np.li < nl) {
            sweep_load(R, np.c0 + np.s + np.dc, np.f0 + np.s + 1 + np.df, nxt, np.c0 + np.s);
            nuA_b = R.FA[ARK_CK(np.f0 + np.s + np.db, R.nf)];
            nuB_b = R.FB[ARK_CK(np.f0 + np.s + np.db, R.nf)];
        }
        RQ<T> rqf = {(T)0, (T)0};
        if (act) rqf = face_rq(cur.uN_f, cur.p_f, q);
        RQ<T> rqb;
        rqb.r = __shfl_up_sync(0xffffffffu, rqf.r, 1);
        rqb.q = __shfl_up_sync(0xffffffffu, rqf.q, 1);
        if (lane == 0) rqb = carry_rq;
        if (act && s == 0) rqb = face_rq(R.FN[ARK_CK(f0 + db, R.nf)], R.FP[ARK_CK(f0 + db, R.nf)], q);
        carry_rq.r = __shfl_sync(0xffffffffu, rqf.r, 31);
        carry_rq.q = __shfl_sync(0xffffffffu, rqf.q, 31);
        Ext<T> e = {};
        if (act)
            e = extrapolate_rq<T, true>(rqf, rqb, cur.nN, cur.cN, cur.uA_f, uA_b, cur.nA, cur.cA, cur.uB_f, uB_b, cur.nB,
                                        cur.cB, cur.nR, cur.cR, q);
        if (bounded && act) {
            // a bounded x axis sweeps cells 1..C1 only; the edge faces take the reference's
            // inflow invariant R = 1 (0 behind a solid first cell) and outflow Q = 5/6 with
            // zero tangential velocity (main.cpp:1731-1745)
            if (s == 0) {
                e.rf = (R.fl[ARK_CK(c0 + 1, R.nc)] & FL_LT) ? (T)1 : (T)0;
                e.af = (T)0;
                e.bf = (T)0;
            }
            if (s == nd) {
                e.qb = (T)(5. / 6.);
                e.ab = (T)0;
                e.bb = (T)0;
            }
        }
        Ext<T> prev;
        prev.rf = __shfl_up_sync(0xffffffffu, e.rf, 1);
        prev.af = __shfl_up_sync(0xffffffffu, e.af, 1);
        prev.bf = __shfl_up_sync(0xffffffffu, e.bf, 1);
        T ucb = __shfl_up_sync(0xffffffffu, cur.nN, 1);
        uint8_t flb = (uint8_t)__shfl_up_sync(0xffffffffu, (int)cur.fl, 1);
        if (lane == 0) {
            prev.rf = carry.rf;
            prev.af = carry.af;
            prev.bf = carry.bf;
            ucb = carry_u;
            flb = carry_fl;
        }
        carry.rf = __shfl_sync(0xffffffffu, e.rf, 31);
        carry.af = __shfl_sync(0xffffffffu, e.af, 31);
        carry.bf = __shfl_sync(0xffffffffu, e.bf, 31);
        carry_u = __shfl_sync(0xffffffffu, cur.nN, 31);
        carry_fl = (uint8_t)__shfl_sync(0xffffffffu, (int)cur.fl, 31);
        if (act && s >= 1)
            face_update<T, false>(N, W, c0 + s - 1 + dp, c0 + s + dc, f0 + s, flb, cur.fl, ucb, cur.nN, prev, e, uA_b,
                                  uB_b, q);
        cur = nxt;
        uA_b = nuA_b;
        uB_b = nuB_b;
        cp = np;
    }
}

template <class T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 6 : 3)
    k_sweep_x(const __grid_constant__ DevState<T> S, int con, int fcur, int glines) {
    sweep_x_body<T>(S, con, fcur, glines, bix_here());
}

// The x faces that Phase1 + stress with the x1 sweep folded in leaves (stg::phase1_tma_body
// with XS): per line (j, k), face b * tw + 1 of every tile seam b < nb = ceil(C1 / tw), between
// the last cell of tile b - 1 and the first of tile b, and face C1 + 1.  Everything comes from
// the seam arrays the tiles wrote.  On a periodic x axis the ghost positions stand for cells C1
// (behind face 1) and 1 (ahead of face C1 + 1): their values are those cells' (slots nb and 0),
// and so are their extrapolations when the old faces 1 and C1 + 1 agree bit for bit (as every
// step leaves them: the two faces are one, updated from the same values); otherwise the ghost
// position's extrapolation is computed here as k_sweep_x computes it, from the cell and the
// faces it stands for (xcell, xface).  One thread per face (id < seam_slots(g, tw)), the seams of
// a line side by side.
template <class T>
__device__ __forceinline__ void sweep_x_seams_body(const DevState<T> &S, int con, int fcur, const XSeams &X, int id) {
    const Geom g = S.g;
    const int rows = g.C2 * g.C3, nb = (g.C1 + X.tw - 1) / X.tw;
    if (id >= rows * (nb + 1)) return;
    const int row = id / (nb + 1), b = id - row * (nb + 1);
    const int j = row % g.C2 + 1, k = row / g.C2 + 1;
    const int s = b == nb ? g.C1 + 1 : b * X.tw + 1; // the face, between positions s - 1 and s
    const bool px = S.k.periodic_x;
    const int w = ARK_CK(seam_slot(g, X.tw, b, j, k), X.n);
    // the slots of the cells behind and ahead (the cells the periodic ghost positions stand for)
    const int wb = ARK_CK(px && b == 0 ? w + nb : w, X.n), wa = ARK_CK(px && b == nb ? w - nb : w, X.n);
    Ext<T> prev = {}, cur = {};
    prev.rf = X.b[0][wb];
    prev.af = X.b[1][wb];
    prev.bf = X.b[2][wb];
    cur.qb = X.a[0][wa];
    cur.ab = X.a[1][wa];
    cur.bb = X.a[2][wa];
    const SweepK<T> q = sweep_consts(S, 0);
    if (px && (b == 0 || b == nb)) {
        // faces 1 and C1 + 1 (u2, u3, u1, p) as the tiles holding cells 1 and C1 left them in
        // slots 0 and nb
        const int w0 = ARK_CK(w - b, X.n), we = ARK_CK(w - b + nb, X.n);
        auto same = [&](int a) { return __float_as_int(X.a[a][w0]) == __float_as_int(X.a[a][we]); };
        if (!(same(8) && same(9) && same(10) && same(11))) {
            const SweepSrc<T> R = sweep_src(S, con, fcur, 0);
            const int c0 = g.ci(0, j, k), f0 = g.fi(0, j, k);
            const bool lo = b == 0; // ghost position 0 (cell C1; faces 1 ahead, C1 behind) or C1 + 1
            const int c = ARK_CK(c0 + (lo ? g.C1 : 1), R.nc);
            const int ff = ARK_CK(f0 + (lo ? 1 : 2), R.nf), fb = ARK_CK(f0 + (lo ? g.C1 : g.C1 + 1), R.nf);
            const Ext<T> e = extrapolate_rq<T, true>(face_rq(R.FN[ff], R.FP[ff], q), face_rq(R.FN[fb], R.FP[fb], q), R.nN[c],
                                                     R.cN[c], R.FA[ff], R.FA[fb], R.nA[c], R.cA[c], R.FB[ff], R.FB[fb], R.nB[c],
                                                     R.cB[c], R.nR[c], R.cR[c], q);
            if (lo) {
                prev.rf = e.rf;
                prev.af = e.af;
                prev.bf = e.bf;
            } else {
                cur.qb = e.qb;
                cur.ab = e.ab;
                cur.bb = e.bb;
            }
        }
    }
    NVals<T> V;
    V.a[0] = X.b[4][wb];
    V.b[0] = X.b[5][wb];
    V.r[0] = X.b[6][wb];
    V.a[1] = X.a[4][wa];
    V.b[1] = X.a[5][wa];
    V.r[1] = X.a[6][wa];
    // the positions' own flags and the face's old tangential velocities: slot w's
    const uint8_t flb = (uint8_t)__float_as_int(X.b[7][w]), flf = (uint8_t)__float_as_int(X.a[7][w]);
    const FaceOut<T> W = sweep_out(S, fcur, 0);
    face_store(W, ARK_CK(g.fi(s, j, k), W.nf),
               face_values_v<T, false>(V, flb, flf, X.b[3][wb], X.a[3][wa], prev, cur, X.a[8][w], X.a[9][w], q));
}
template <class T>
__global__ void __launch_bounds__(256) k_sweep_x_seams(const __grid_constant__ DevState<T> S, int con, int fcur,
                                                       const __grid_constant__ XSeams X) {
    sweep_x_seams_body<T>(S, con, fcur, X, blockIdx.x * blockDim.x + threadIdx.x);
}

// x2 (AX = 1) and x3 (AX = 2) sweeps: one thread per segment of `seg` faces of a line,
// threads on consecutive i (coalesced), marching along the sweep axis with the next cell's
// loads issued before the current cell is computed.  A segment of faces s0+1..s1 needs
// cells s0..s1 (cell s0 is the one overlap with the previous segment); the face behind
// the current cell is carried in registers.  Old faces come from generation fcur, new
// faces go to fcur^1, so segments are independent.  Each warp takes 32 consecutive i of one
// line row o: warp q of the grid covers chunk q % ceil(C1/32) of row q / ceil(C1/32), so rows
// narrower than a block (an ensemble's 32- and 64-cell members) still fill every lane.
__host__ __device__ inline int col_sweep_blocks(const Geom &g, int axis) {
    return (((g.C1 + 31) >> 5) * (axis == 1 ? g.C3 : g.C2) + 3) >> 2;
}
template <class T, int AX>
__device__ __forceinline__ void sweep_col_body(const DevState<T> &S, int con, int fcur, int seg, const BIx &bx) {
    const Geom g = S.g;
    const int nic = (g.C1 + 31) >> 5;
    const int wq = bx.x * 4 + (threadIdx.x >> 5); // this warp's (chunk, row)
    const int i = (wq % nic) * 32 + (threadIdx.x & 31) + 1;
    const int o = wq / nic + 1;
    const int nd = (AX == 1 ? g.C2 : g.C3) + 1;
    const int s0 = bx.z * seg;
    if (i > g.C1 || o > (AX == 1 ? g.C3 : g.C2) || s0 >= nd) return;
    const int s1 = s0 + seg < nd ? s0 + seg : nd;
    const SweepSrc<T> R = sweep_src(S, con, fcur, AX);
    const FaceOut<T> W = sweep_out(S, fcur, AX);
    const NCell<T> N = {R.nN, R.nA, R.nB, R.nR, R.nc};
    const SweepK<T> q = sweep_consts(S, AX);
    const int cst = AX == 1 ? (int)g.cs1 : (int)g.cs2, fst = AX == 1 ? (int)g.fs1 : (int)g.fs2;
    // z: the ghost positions read from the cells and faces they stand for (zcell, zface), the
    // flags from the ghost cells themselves: c0 / f0 shift cell 0 / face 0, c1 / f1 cell nd =
    // C3+1 / face nd+1 (zero along y, or when the z ghosts are a slab's halo)
    const bool fold = AX == 2 && !S.k.ext_z, pz = S.k.periodic_z;
    const int c0 = fold ? zcell(0, g.C3, pz) * cst : 0, f0 = fold ? zface(0, g.C3, pz) * fst : 0;
    const int c1 = fold ? (zcell(nd, g.C3, pz) - nd) * cst : 0, f1 = fold ? (zface(nd + 1, g.C3, pz) - nd - 1) * fst : 0;
    int c = (AX == 1 ? g.ci(i, 0, o) : g.ci(i, o, 0)) + s0 * cst;
    int fb = (AX == 1 ? g.fi(i, 0, o) : g.fi(i, o, 0)) + s0 * fst;
    const int fb0 = fb + (s0 == 0 ? f0 : 0);
    T uA_b = R.FA[ARK_CK(fb0, R.nf)], uB_b = R.FB[ARK_CK(fb0, R.nf)];
    RQ<T> rqb = face_rq(R.FN[ARK_CK(fb0, R.nf)], R.FP[ARK_CK(fb0, R.nf)], q); // then the forward face's, carried
    SweepIn<T> cur, nxt = {};
    sweep_load(R, c + (s0 == 0 ? c0 : 0), fb + fst, cur, c); // (s0 < nd: its forward face is inside)
    Ext<T> prev = {};
    T uprev = 0;
    uint8_t flprev = 0;
    for (int s = s0; s <= s1; ++s, c += cst, fb += fst) {
        const bool last = s + 1 == nd; // the next position is the ghost C3+1, its forward face C3+2
        if (s < s1) sweep_load(R, c + cst + (last ? c1 : 0), fb + 2 * fst + (last ? f1 : 0), nxt, c + cst);
        const RQ<T> rqf = face_rq(cur.uN_f, cur.p_f, q);
        const Ext<T> e = extrapolate_rq<T, AX == 2>(rqf, rqb, cur.nN, cur.cN, cur.uA_f, uA_b, cur.nA, cur.cA, cur.uB_f,
                                                    uB_b, cur.nB, cur.cB, cur.nR, cur.cR, q);
        if (s > s0)
            face_update<T, AX == 1>(N, W, c - cst + (s == 1 ? c0 : 0), c + (s == nd ? c1 : 0), fb, flprev, cur.fl, uprev,
                                    cur.nN, prev, e, uA_b, uB_b, q);
        prev = e;
        uprev = cur.nN;
        flprev = cur.fl;
        rqb = rqf;
        uA_b = cur.uA_f;
        uB_b = cur.uB_f;
        cur = nxt;
    }
}

template <class T, int AX>
__global__ void __launch_bounds__(128) k_sweep_col(const __grid_constant__ DevState<T> S, int con, int fcur, int seg) {
    sweep_col_body<T, AX>(S, con, fcur, seg, bix_here());
}

// The z faces that Phase1 + stress with the x3 sweep folded in leaves (stg::phase1_tma_body with
// XS & 2): per column, the face below the first plane of each chunk of kch planes (c * kch + 1,
// blockIdx.z = c < nch) and face C3 + 1 (blockIdx.z = nch), each the x3 sweep's own segment of
// one face (positions s0 and s0 + 1, ghost positions read where they stand for).
template <class T>
__global__ void __launch_bounds__(128) k_sweep_z_seams(const __grid_constant__ DevState<T> S, int con, int fcur, int kch) {
    BIx bx = bix_here();
    const int nch = (S.g.C3 + kch - 1) / kch;
    bx.z = (int)blockIdx.z < nch ? (int)blockIdx.z * kch : S.g.C3;
    sweep_col_body<T, 2>(S, con, fcur, 1, bx);
}

// ---------------------------------------------------------------------------------------
// Phase2 with the three sweeps fused.  The sweeps are independent (each reads its own face
// set and the two cell levels, and writes its own new face generation), so one kernel can do
// all three: a block owns a 64 x 4 tile of columns and marches up a chunk of planes.  Per
// plane every thread computes its cell's x, y and z extrapolations (the same extrapolate
// calls, with the same inputs, as the separate sweeps), plus the halo cells the tile's faces
// need (column i0-1, row j0-1, and the ghost cells C+1 of the tiles at the domain's end).  The
// x and y results meet in shared memory, the z result is carried to the next plane; then every
// thread updates the faces below its cell in the three directions with the same face_update
// calls.  Cell levels and flags are read once per cell instead of three times.  Results are
// bit-identical to the separate sweeps (tested).
// ---------------------------------------------------------------------------------------
namespace p2f {
constexpr int SX = 64, SY = 4;

// What a face update needs from the cell behind or ahead: the extrapolated values, the
// half-step normal velocity and the flags.
template <class T> struct CellExt {
    Ext<T> e;
    T un;
    uint8_t fl;
};

// The extrapolation of cell c along axis AX: its faces lo (index f) and hi (f + stride).
template <class T, int AX>
__device__ __forceinline__ CellExt<T> cell_ext(const SweepSrc<T> &R, const SweepK<T> &q, int c, int f, int fst) {
    SweepIn<T> x;
    sweep_load(R, c, f + fst, x);
    CellExt<T> r;
    r.e = extrapolate<T, AX != 1>(x.uN_f, R.FN[f], x.nN, x.cN, x.uA_f, R.FA[f], x.nA, x.cA, x.uB_f, R.FB[f], x.nB, x.cB,
                                  x.nR, x.cR, x.p_f, R.FP[f], q);
    r.un = x.nN;
    r.fl = x.fl;
    return r;
}

template <class T>
__global__ void __launch_bounds__(SX *SY, 2) k_phase2_fused(const __grid_constant__ DevState<T> S, int con, int fcur, int kch) {
    __shared__ CellExt<T> EX[SY][SX + 2], EY[SY + 2][SX];
    const Geom g = S.g;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.x * SX + 1, j0 = blockIdx.y * SY + 1;
    const int i = i0 + tx, j = j0 + ty;
    const int k0 = blockIdx.z * kch + 1;
    const int k1 = k0 + kch - 1 < g.C3 ? k0 + kch - 1 : g.C3;
    const bool valid = i <= g.C1 && j <= g.C2;
    const SweepSrc<T> RX = sweep_src(S, con, fcur, 0), RY = sweep_src(S, con, fcur, 1), RZ = sweep_src(S, con, fcur, 2);
    const FaceOut<T> WX = sweep_out(S, fcur, 0), WY = sweep_out(S, fcur, 1), WZ = sweep_out(S, fcur, 2);
    const NCell<T> NX = {RX.nN, RX.nA, RX.nB, RX.nR, RX.nc}, NY = {RY.nN, RY.nA, RY.nB, RY.nR, RY.nc},
                   NZ = {RZ.nN, RZ.nA, RZ.nB, RZ.nR, RZ.nc};
    const SweepK<T> qx = sweep_consts(S, 0), qy = sweep_consts(S, 1), qz = sweep_consts(S, 2);
    const int cs1 = (int)g.cs1, cs2 = (int)g.cs2, fs1 = (int)g.fs1, fs2 = (int)g.fs2;
    const bool bounded_x = !S.k.periodic_x;
    // the bounded x axis's edge invariants (main.cpp:1731-1745), as the x1 sweep applies them
    auto x_edges = [&](CellExt<T> &ce, int ic, int jc, int kc) {
        if (!bounded_x) return;
        if (ic == 0) {
            ce.e.rf = (S.flags[g.ci(1, jc, kc)] & FL_LT) ? (T)1 : (T)0;
            ce.e.af = (T)0;
            ce.e.bf = (T)0;
        } else if (ic == g.C1 + 1) {
            ce.e.qb = (T)(5. / 6.);
            ce.e.ab = (T)0;
            ce.e.bb = (T)0;
        }
    };
    CellExt<T> zlo = {};
    if (valid) zlo = cell_ext<T, 2>(RZ, qz, g.ci(i, j, k0 - 1), g.fi(i, j, k0 - 1), fs2);
    for (int k = k0; k <= k1; ++k) {
        CellExt<T> zc = {};
        if (valid) {
            const int c = g.ci(i, j, k), f = g.fi(i, j, k);
            CellExt<T> ex = cell_ext<T, 0>(RX, qx, c, f, 1);
            x_edges(ex, i, j, k);
            EX[ty][tx + 1] = ex;
            if (tx == 0) {
                CellExt<T> eh = cell_ext<T, 0>(RX, qx, c - 1, f - 1, 1);
                x_edges(eh, i - 1, j, k);
                EX[ty][0] = eh;
            }
            if (i == g.C1) {
                CellExt<T> eh = cell_ext<T, 0>(RX, qx, c + 1, f + 1, 1);
                x_edges(eh, i + 1, j, k);
                EX[ty][tx + 2] = eh;
            }
            EY[ty + 1][tx] = cell_ext<T, 1>(RY, qy, c, f, fs1);
            if (ty == 0) EY[0][tx] = cell_ext<T, 1>(RY, qy, c - cs1, f - fs1, fs1);
            if (j == g.C2) EY[ty + 2][tx] = cell_ext<T, 1>(RY, qy, c + cs1, f + fs1, fs1);
            zc = cell_ext<T, 2>(RZ, qz, c, f, fs2);
        }
        __syncthreads();
        if (valid) {
            const int c = g.ci(i, j, k), f = g.fi(i, j, k);
            {   // x faces i (and C1 + 1)
                const CellExt<T> &b = EX[ty][tx], &a = EX[ty][tx + 1];
                face_update<T, false>(NX, WX, c - 1, c, f, b.fl, a.fl, b.un, a.un, b.e, a.e, RX.FA[f], RX.FB[f], qx);
                if (i == g.C1) {
                    const CellExt<T> &z = EX[ty][tx + 2];
                    face_update<T, false>(NX, WX, c, c + 1, f + 1, a.fl, z.fl, a.un, z.un, a.e, z.e, RX.FA[f + 1],
                                          RX.FB[f + 1], qx);
                }
            }
            {   // y faces j (and C2 + 1)
                const CellExt<T> &b = EY[ty][tx], &a = EY[ty + 1][tx];
                face_update<T, true>(NY, WY, c - cs1, c, f, b.fl, a.fl, b.un, a.un, b.e, a.e, RY.FA[f], RY.FB[f], qy);
                if (j == g.C2) {
                    const CellExt<T> &z = EY[ty + 2][tx];
                    face_update<T, true>(NY, WY, c, c + cs1, f + fs1, a.fl, z.fl, a.un, z.un, a.e, z.e, RY.FA[f + fs1],
                                         RY.FB[f + fs1], qy);
                }
            }
            // z faces k (and C3 + 1)
            face_update<T, false>(NZ, WZ, c - cs2, c, f, zlo.fl, zc.fl, zlo.un, zc.un, zlo.e, zc.e, RZ.FA[f], RZ.FB[f], qz);
            if (k == g.C3) {
                const CellExt<T> zg = cell_ext<T, 2>(RZ, qz, c + cs2, f + fs2, fs2);
                face_update<T, false>(NZ, WZ, c, c + cs2, f + fs2, zc.fl, zg.fl, zc.un, zg.un, zc.e, zg.e, RZ.FA[f + fs2],
                                      RZ.FB[f + fs2], qz);
            }
        }
        __syncthreads();
        zlo = zc;
    }
}
} // namespace p2f

// ---------------------------------------------------------------------------------------
// conservation sums of one level (fixed point: identical for any grid)
// ---------------------------------------------------------------------------------------

template <class T> __global__ void __launch_bounds__(kTileX *kTileY) k_sums(DevState<T> S, int ncon) {
    constexpr bool DEV = Storage<T>::deviation;
    __shared__ long long red[6][kTileX * kTileY / 32];
    const Geom g = S.g;
    const Level<T> L = S.lv[ncon];
    const int i = blockIdx.x * kTileX + threadIdx.x + 1;
    const int j = blockIdx.y * kTileY + threadIdx.y + 1;
    long long a[6] = {0, 0, 0, 0, 0, 0};
    if (i <= g.C1 && j <= g.C2) {
        int64_t c = g.cell(i, j, 1);
        for (int k = 1; k <= g.C3; ++k, c += g.cs2) {
            if (!(S.flags[c] & FL_EQ0)) continue;
            const double ro = DEV ? S.k.ro0 + (double)L.ro[c] : (double)L.ro[c];
            const double u1 = L.u1[c], u2 = L.u2[c], u3 = L.u3[c];
            a[0] += fixed32(ro);
            a[1] += fixed32(ro * u1);
            a[2] += fixed32(ro * u2);
            a[3] += fixed32(ro * u3);
            a[4] += fixed32((u1 * u1 + u2 * u2 + u3 * u3) / 2);
            a[5] += 1;
        }
    }
    for (int q = 0; q < 6; ++q) a[q] = warp_sum_i64(a[q]);
    const int t = threadIdx.y * kTileX + threadIdx.x, w = t >> 5;
    if ((t & 31) == 0)
        for (int q = 0; q < 6; ++q) red[q][w] = a[q];
    __syncthreads();
    if (t < 6) {
        long long z = 0;
        for (int v = 0; v < kTileX * kTileY / 32; ++v) z += red[t][v];
        if (z != 0)
            atomicAdd((unsigned long long *)(t < 5 ? &S.sc->sums[t] : &S.sc->sum_cells), (unsigned long long)z);
    }
}

// Mean of u1 over the fluid cells of each y plane (one block per plane), summed in exact
// 2^-32 fixed point: acc[2*(j-1)] = sum, acc[2*(j-1)+1] = cells.  The plane mean profile
// U(y) and, from its first and last entries, the wall shear 2*VIS*U/dx2 in the one-sided
// wall form of StressTensor (main.cpp:924-927).
template <class T> __global__ void __launch_bounds__(256) k_mean_profile(DevState<T> S, int ncon, long long *acc) {
    __shared__ long long red[2][8];
    const Geom g = S.g;
    const int j = blockIdx.x + 1;
    const T *__restrict__ u1 = S.lv[ncon].u1;
    long long s = 0, n = 0;
    const int plane = g.C1 * g.C3;
    for (int t = threadIdx.x; t < plane; t += blockDim.x) {
        const int i = t % g.C1 + 1, k = t / g.C1 + 1;
        const int64_t c = g.cell(i, j, k);
        if (!(S.flags[c] & FL_EQ0)) continue;
        s += fixed32((double)u1[c]);
        n += 1;
    }
    s = warp_sum_i64(s);
    n = warp_sum_i64(n);
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = s;
        red[1][threadIdx.x >> 5] = n;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long a = 0, b = 0;
        for (int w = 0; w < 8; ++w) {
            a += red[0][w];
            b += red[1][w];
        }
        acc[2 * (j - 1)] = a;
        acc[2 * (j - 1) + 1] = b;
    }
}

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------

inline int grid_for(int64_t n, int block, int cap) {
    int64_t b = (n + block - 1) / block;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

inline dim3 cell_grid(const Geom &g) {
    return dim3((g.C1 + kCellBX - 1) / kCellBX, (g.C2 + kCellBY - 1) / kCellBY, g.C3);
}

inline dim3 tile_grid(const Geom &g) { return dim3(tiles_x(g), tiles_y(g), tiles_k(g)); }

template <class T> void Launch<T>::reduce_start(const DevState<T> &S, int con, cudaStream_t st) {
    k_reduce_start<T><<<tile_grid(S.g), dim3(kTileX, kTileY), 0, st>>>(S, con);
}

template <class T> void Launch<T>::finalize_dt(const DevState<T> &S, int advance_time, cudaStream_t st) {
    k_finalize_dt<T><<<1, 1024, 0, st>>>(S, advance_time);
}

inline void wrap_add(WrapJob &J, void *a, int face, uint8_t mx, uint8_t mz) {
    if (!a || (mx == GH_NONE && mz == GH_NONE)) return;
    J.a[J.n] = a;
    J.face[J.n] = (uint8_t)face;
    J.mode[J.n][0] = mx;
    J.mode[J.n][1] = mz;
    ++J.n;
}

template <class T> inline void wrap_launch(const DevState<T> &S, const WrapJob &J, cudaStream_t st) {
    if (J.n == 0) return;
    k_wrap<T><<<dim3((wrap_lines(S.g) + 255) / 256, J.n), 256, 0, st>>>(S.g, J);
}

// StressTensor's exchange of u1Con, u2Con, u3Con (main.cpp:603-845): periodic axes wrap,
// bounded x and z take the zero-gradient copy.  with_ro also fills roCon's ghosts as Phase2's
// exchange does (main.cpp:1049-1698): copied or wrapped on z, for the fused step, which reads
// that level before Phase2; on x only for the one-kernel Phase2 forms (with_ro = 2), as the x1
// sweep kernel reads x ghost positions from the cells they stand for (xcell).
// A slab of a z split (ext_z) leaves its z ghosts to the slab group's halo exchange.
template <class T> void Launch<T>::wrap_con(const DevState<T> &S, int con, int with_ro, cudaStream_t st) {
    const uint8_t ux = S.k.periodic_x ? GH_WRAP : GH_COPY;
    const uint8_t uz = S.k.ext_z ? GH_NONE : S.k.periodic_z ? GH_WRAP : GH_COPY;
    WrapJob J = {};
    const Level<T> L = S.lv[con];
    wrap_add(J, L.u1, 0, ux, uz);
    wrap_add(J, L.u2, 0, ux, uz);
    wrap_add(J, L.u3, 0, ux, uz);
    if (with_ro) wrap_add(J, L.ro, 0, with_ro == 2 && S.k.periodic_x ? GH_WRAP : GH_NONE, uz);
    wrap_launch(S, J, st);
}

// The halo exchange before Phase2 (main.cpp:1049-1698): u?nCon and ronCon wrap or copy on
// both axes; roCon wraps, or is copied on a bounded z only; faces normal to x1 wrap in x (a
// bounded x sweep never reads their halo); faces normal to x3 wrap or copy in z.  The x ghosts
// only for the one-kernel Phase2 forms (xlines): the x1 sweep kernel reads its x ghost
// positions from the cells and faces they stand for (xcell, xface), and no other Phase2 kernel
// reads x ghosts.
template <class T> void Launch<T>::wrap_phase2(const DevState<T> &S, int con, int fcur, cudaStream_t st, int xlines) {
    const bool px = S.k.periodic_x, pz = S.k.periodic_z;
    const uint8_t cx = !xlines ? GH_NONE : px ? GH_WRAP : GH_COPY;
    const uint8_t cz = S.k.ext_z ? GH_NONE : pz ? GH_WRAP : GH_COPY;
    WrapJob J = {};
    const Level<T> Ln = S.lv[con ^ 1], Lc = S.lv[con];
    wrap_add(J, Ln.u1, 0, cx, cz);
    wrap_add(J, Ln.u2, 0, cx, cz);
    wrap_add(J, Ln.u3, 0, cx, cz);
    wrap_add(J, Ln.ro, 0, cx, cz);
    wrap_add(J, Lc.ro, 0, xlines && px ? GH_WRAP : GH_NONE, cz);
    const FaceSet<T> &X = S.fc[fcur][0], &Z = S.fc[fcur][2];
    T *fx[5] = {X.p, X.u[0], X.u[1], X.u[2], X.ro};
    T *fz[5] = {Z.p, Z.u[0], Z.u[1], Z.u[2], Z.ro};
    for (int q = 0; q < 5; ++q) wrap_add(J, fx[q], 1, xlines && px ? GH_WRAP : GH_NONE, GH_NONE);
    for (int q = 0; q < 5; ++q) wrap_add(J, fz[q], 1, GH_NONE, cz);
    wrap_launch(S, J, st);
}

// A slab group's halo exchange: thread (x, job) copies interior element x of one plane.  The
// sources are interior planes of the slabs, the destinations ghost planes, so the copies of one
// exchange are independent.
template <class T> __global__ void k_halo(Geom g, const HaloJob *__restrict__ jobs) {
    const HaloJob J = jobs[blockIdx.y];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.C1 * g.C2) return;
    const int i = t % g.C1 + 1, j = t / g.C1 + 1;
    const int64_t row = (int64_t)j * (J.face ? g.fs1 : g.cs1) + i;
    const int64_t plane = J.face ? g.fs2 : g.cs2;
    ((T *)J.dst)[ARK_CK((int64_t)J.dst_plane * plane + row, (int64_t)J.dst_planes * plane)] =
        ((const T *)J.src)[ARK_CK((int64_t)J.src_plane * plane + row, (int64_t)J.src_planes * plane)];
}
template <class T> void Launch<T>::halo_exchange(const Geom &g, const HaloJob *jobs, int njobs, cudaStream_t st) {
    if (njobs <= 0) return;
    k_halo<T><<<dim3((g.C1 * g.C2 + 255) / 256, njobs), 256, 0, st>>>(g, jobs);
}

template <class T, template <class, int> class KERNEL>
void launch_phase1(const DevState<T> &S, int src, int dst, int fcur, int mode, dim3 grid, cudaStream_t st) {
    const dim3 block(kTileX, kTileY);
    switch (mode) {
    case P1_PLAIN: KERNEL<T, P1_PLAIN>::launch(grid, block, st, S, src, dst, fcur); break;
    case P1_STRESS | P1_FORCES | P1_RMAX:
        KERNEL<T, P1_STRESS | P1_FORCES | P1_RMAX>::launch(grid, block, st, S, src, dst, fcur);
        break;
    case P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX:
        KERNEL<T, P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>::launch(grid, block, st, S, src, dst, fcur);
        break;
    case P1_FORCES | P1_RSUM: KERNEL<T, P1_FORCES | P1_RSUM>::launch(grid, block, st, S, src, dst, fcur); break;
    default: break;
    }
}
// the learned-closure modes exist for the one-cell kernel only
template <class T>
void launch_phase1_nut(const DevState<T> &S, int src, int dst, int fcur, int mode, dim3 grid, cudaStream_t st) {
    const dim3 block(kTileX, kTileY);
    switch (mode) {
    case P1_STRESS | P1_FORCES | P1_RMAX | P1_NUT:
        k_phase1_cell<T, P1_STRESS | P1_FORCES | P1_RMAX | P1_NUT><<<grid, block, 0, st>>>(S, src, dst, fcur);
        break;
    case P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX | P1_NUT:
        k_phase1_cell<T, P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX | P1_NUT><<<grid, block, 0, st>>>(S, src, dst, fcur);
        break;
    default: break;
    }
}
template <class T, int MODE> struct MarchK {
    static void launch(dim3 g, dim3 b, cudaStream_t st, const DevState<T> &S, int src, int dst, int fcur) {
        k_phase1<T, MODE><<<g, b, 0, st>>>(S, src, dst, fcur);
    }
};
template <class T, int MODE> struct CellK {
    static void launch(dim3 g, dim3 b, cudaStream_t st, const DevState<T> &S, int src, int dst, int fcur) {
        k_phase1_cell<T, MODE><<<g, b, 0, st>>>(S, src, dst, fcur);
    }
};

#include "ark_staged.cuh"
#include "ark_fused.cuh"

// march = 3: fcs::k_phase1_faces (FP64, face quantities computed once); 2: k_phase1_staged
// (FP32); both for the two Phase1 modes of a step, other modes fall back to the one-cell
// kernel; 1: k_phase1 (a block marches kTileK planes); 0: k_phase1_cell
template <class T>
void Launch<T>::phase1(const DevState<T> &S, int src, int dst, int fcur, int mode, int march, cudaStream_t st, int kch_in) {
    if (mode & P1_NUT) {
        launch_phase1_nut<T>(S, src, dst, fcur, mode, dim3(tiles_x(S.g), tiles_y(S.g), S.g.C3), st);
        return;
    }
    if constexpr (std::is_same<T, double>::value) {
        if (march == 3) {
            // default planes per block: about nine waves of three blocks per SM (at 256x128x128:
            // 4 planes, Phase1 + stress 1.208 -> 1.178 ms and second Phase1 0.758 -> 0.739 ms
            // against 8; 2, 3, 6 and 12 planes measured between)
            const long long cols = (long long)((S.g.C1 + fcs::SX - 1) / fcs::SX) * ((S.g.C2 + fcs::SY - 1) / fcs::SY);
            const int kdef = (int)std::max(2LL, std::min(64LL, (long long)S.g.C3 * cols / (152 * 3 * 9)));
            const int kch = kch_in > 0 ? std::min(kch_in, S.g.C3) : kdef;
            const dim3 grid((S.g.C1 + fcs::SX - 1) / fcs::SX, (S.g.C2 + fcs::SY - 1) / fcs::SY, (S.g.C3 + kch - 1) / kch);
            const dim3 block(fcs::SX, fcs::SY);
            switch (mode) {
            case P1_STRESS | P1_FORCES | P1_RMAX:
                fcs::k_phase1_faces<T, P1_STRESS | P1_FORCES | P1_RMAX><<<grid, block, fcs::face_smem<T>(), st>>>(S, src, dst, fcur, kch);
                return;
            case P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX:
                fcs::k_phase1_faces<T, P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX><<<grid, block, fcs::face_smem<T>(), st>>>(S, src, dst, fcur,
                                                                                                      kch);
                return;
            case P1_FORCES | P1_RSUM:
                fcs::k_phase1_faces<T, P1_FORCES | P1_RSUM><<<grid, block, fcs::face_smem<T>(), st>>>(S, src, dst, fcur, kch);
                return;
            default: march = 0; break;
            }
        }
    }
    if constexpr (std::is_same<T, float>::value) {
        if (march == 2) {
            switch (mode) {
            case P1_STRESS | P1_FORCES | P1_RMAX:
                stg::launch_staged<P1_STRESS | P1_FORCES | P1_RMAX>(S, src, dst, fcur, st, kch_in);
                return;
            case P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX:
                stg::launch_staged<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>(S, src, dst, fcur, st, kch_in);
                return;
            case P1_FORCES | P1_RSUM: stg::launch_staged<P1_FORCES | P1_RSUM>(S, src, dst, fcur, st, kch_in); return;
            default: march = 0; break;
            }
        } else if (march >= 4 && march <= 6) { // TMA copies, 64 x 4, 32 x 8 or 128 x 2 tiles
            constexpr int A = P1_STRESS | P1_FORCES | P1_RMAX, B = A | P1_BULK, C = P1_FORCES | P1_RSUM;
            auto shape = [&](auto m) {
                constexpr int M = decltype(m)::value;
                if (march == 4) stg::launch_staged_tma<M, 64, 4>(S, src, dst, fcur, st, kch_in);
                else if (march == 5) stg::launch_staged_tma<M, 32, 8>(S, src, dst, fcur, st, kch_in);
                else stg::launch_staged_tma<M, 128, 2>(S, src, dst, fcur, st, kch_in);
            };
            switch (mode) {
            case A: shape(std::integral_constant<int, A>()); return;
            case B: shape(std::integral_constant<int, B>()); return;
            case C: shape(std::integral_constant<int, C>()); return;
            default: march = 0; break;
            }
        }
    }
    if (march == 1)
        launch_phase1<T, MarchK>(S, src, dst, fcur, mode, tile_grid(S.g), st);
    else
        launch_phase1<T, CellK>(S, src, dst, fcur, mode, dim3(tiles_x(S.g), tiles_y(S.g), S.g.C3), st);
}

template <class T> void Launch<T>::sweep_x_seams(const DevState<T> &S, int con, int fcur, const XSeams &X, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        const long long n = seam_slots(S.g, X.tw);
        k_sweep_x_seams<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(S, con, fcur, X);
    }
}

template <class T>
bool Launch<T>::phase1_sweep_x(const DevState<T> &S, int src, int dst, int fcur, int mode, int march, cudaStream_t st, int kch,
                               XSeams &X, int fold) {
    if constexpr (std::is_same<T, float>::value) {
        constexpr int A = P1_STRESS | P1_FORCES | P1_RMAX, B = A | P1_BULK;
        if (mode != A && mode != B) return false;
        auto go = [&](auto m, auto xs) {
            constexpr int M = decltype(m)::value, XS = decltype(xs)::value;
            if (march == 4) return stg::launch_staged_tma_xs<M, 64, 4, XS>(S, src, dst, fcur, X, st, kch);
            if (march == 5) return stg::launch_staged_tma_xs<M, 32, 8, XS>(S, src, dst, fcur, X, st, kch);
            if (march == 6) return stg::launch_staged_tma_xs<M, 128, 2, XS>(S, src, dst, fcur, X, st, kch);
            return false;
        };
        using I1 = std::integral_constant<int, 1>;
        using I3 = std::integral_constant<int, 3>;
        if (mode == A) return fold == 3 ? go(std::integral_constant<int, A>(), I3()) : go(std::integral_constant<int, A>(), I1());
        return fold == 3 ? go(std::integral_constant<int, B>(), I3()) : go(std::integral_constant<int, B>(), I1());
    }
    return false;
}

template <class T> void Launch<T>::sweep_z_seams(const DevState<T> &S, int con, int fcur, int kch, cudaStream_t st) {
    const int nch = (S.g.C3 + kch - 1) / kch;
    k_sweep_z_seams<T><<<dim3(col_sweep_blocks(S.g, 2), 1, nch + 1), 128, 0, st>>>(S, con, fcur, kch);
}


template <class T> void Launch<T>::prepare() {
    if constexpr (std::is_same<T, double>::value) {
        constexpr int fb = fcs::face_smem<double>();
        cudaFuncSetAttribute(fcs::k_phase1_faces<double, P1_STRESS | P1_FORCES | P1_RMAX>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, fb);
        cudaFuncSetAttribute(fcs::k_phase1_faces<double, P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, fb);
        cudaFuncSetAttribute(fcs::k_phase1_faces<double, P1_FORCES | P1_RSUM>, cudaFuncAttributeMaxDynamicSharedMemorySize, fb);
    }
    if constexpr (std::is_same<T, float>::value) {
        stg::prepare_staged<P1_STRESS | P1_FORCES | P1_RMAX>();
        stg::prepare_staged<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>();
        stg::prepare_staged<P1_FORCES | P1_RSUM>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_RMAX, 64, 4>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 64, 4>();
        stg::prepare_staged_tma<P1_FORCES | P1_RSUM, 64, 4>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_RMAX, 32, 8>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 32, 8>();
        stg::prepare_staged_tma<P1_FORCES | P1_RSUM, 32, 8>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_RMAX, 128, 2>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 128, 2>();
        stg::prepare_staged_tma<P1_FORCES | P1_RSUM, 128, 2>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_RMAX, 128, 2, 1>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 128, 2, 1>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_RMAX, 64, 4, 1>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 64, 4, 1>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_RMAX, 32, 8, 1>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 32, 8, 1>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_RMAX, 128, 2, 3>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 128, 2, 3>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_RMAX, 64, 4, 3>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 64, 4, 3>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_RMAX, 32, 8, 3>();
        stg::prepare_staged_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 32, 8, 3>();
        s2::prepare<float>();
    }
}

template <class T> int Launch<T>::staging_unmet(const DevState<T> &S, int src, int dst, int fcur, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value)
        return stg::launch_staged_tma_unmet<P1_STRESS | P1_FORCES | P1_RMAX>(S, src, dst, fcur, 16, st) ? 1 : 0;
    return 0;
}

template <class T> void Launch<T>::stress(const DevState<T> &S, int con, int bulk, cudaStream_t st) {
    const dim3 block(kCellBX, kCellBY);
    k_stress_force<T><<<cell_grid(S.g), block, 0, st>>>(S, con, bulk);
    if (S.sig[0][0]) {
        for (int d = 0; d < 3; ++d) {
            dim3 gd((S.g.C1 + (d == 0) + kCellBX - 1) / kCellBX, (S.g.C2 + (d == 1) + kCellBY - 1) / kCellBY,
                    S.g.C3 + (d == 2));
            k_stress_faces<T><<<gd, block, 0, st>>>(S, con, d);
        }
    }
}

template <class T> void Launch<T>::use_forces(const DevState<T> &S, int ncon, cudaStream_t st) {
    k_use_forces<T><<<cell_grid(S.g), dim3(kCellBX, kCellBY), 0, st>>>(S, ncon);
}

// Segments of at most 32 faces, balanced so no thread gets a short tail.
// segments of at most `target` faces, balanced
inline int sweep_segment(int nd, int target, int *nseg) {
    const int n = (nd + target - 1) / target;
    *nseg = n;
    return (nd + n - 1) / n;
}

template <class T>
void Launch<T>::sweep(const DevState<T> &S, int con, int fcur, int axis, cudaStream_t st, int target, int xlines) {
    if (axis == 0) {
        const int lines_x = S.g.C2 * S.g.C3, gl = xlines > 0 ? xlines : x_lines_per_warp(S.g, sizeof(T) == 8);
        const dim3 grid((lines_x + 4 * gl - 1) / (4 * gl)); // 4 warps of gl lines
        k_sweep_x<T><<<grid, 128, 0, st>>>(S, con, fcur, gl);
    } else if (axis == 1) {
        int nseg;
        const int seg = sweep_segment(S.g.C2 + 1, target, &nseg);
        const dim3 grid(col_sweep_blocks(S.g, 1), 1, nseg);
        k_sweep_col<T, 1><<<grid, 128, 0, st>>>(S, con, fcur, seg);
    } else {
        int nseg;
        const int seg = sweep_segment(S.g.C3 + 1, target, &nseg);
        const dim3 grid(col_sweep_blocks(S.g, 2), 1, nseg);
        k_sweep_col<T, 2><<<grid, 128, 0, st>>>(S, con, fcur, seg);
    }
}

template <class T>
void Launch<T>::phase2_phase1(const DevState<T> &S, int con, int fcur, const Level<T> &out, cudaStream_t st, bool tma) {
    if constexpr (std::is_same<T, float>::value) s2::launch<float>(S, con, fcur, out, st, tma);
}
template <class T> void Launch<T>::phase2_fused(const DevState<T> &S, int con, int fcur, cudaStream_t st) {
    const int kch = stg::staged_chunk(S.g);
    const dim3 grid((S.g.C1 + p2f::SX - 1) / p2f::SX, (S.g.C2 + p2f::SY - 1) / p2f::SY, (S.g.C3 + kch - 1) / kch);
    p2f::k_phase2_fused<T><<<grid, dim3(p2f::SX, p2f::SY), 0, st>>>(S, con, fcur, kch);
}

template <class T>
void Launch<T>::boundary_fill(const DevState<T> &S, int ncon, int axis, int periodic, cudaStream_t st) {
    const int64_t n = axis == 1 ? (int64_t)S.g.C2 * S.g.C3 : axis == 2 ? (int64_t)S.g.C1 * S.g.C3
                                                                       : (int64_t)S.g.C1 * S.g.C2;
    k_boundary_fill<T><<<grid_for(n, 256, 1 << 30), 256, 0, st>>>(S.g, S.lv[ncon], axis, periodic);
}

template <class T> void Launch<T>::mean_profile(const DevState<T> &S, int ncon, long long *acc, cudaStream_t st) {
    k_mean_profile<T><<<S.g.C2, 256, 0, st>>>(S, ncon, acc);
}

template <class T> void Launch<T>::sums(const DevState<T> &S, int ncon, cudaStream_t st) {
    dim3 grid(tiles_x(S.g), tiles_y(S.g));
    k_sums<T><<<grid, dim3(kTileX, kTileY), 0, st>>>(S, ncon);
}

// Precision conversion for FP32 contexts (host arrays are always double).
// Host arrays reach the device through a contiguous double staging buffer (one plain copy
// each way); these kernels move between it (rows of w elements) and the device's padded rows
// (pitch elements), converting for FP32 contexts.  With offset 0 FP64 values are copied as
// they are.
template <class T> __global__ void k_rows_in(T *dst, const double *src, int w, int64_t rows, int pitch, double offset) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= w) return;
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y) {
        const double v = src[r * w + c];
        dst[r * pitch + c] = (T)(offset == 0.0 ? v : v - offset);
    }
}
template <class T> __global__ void k_rows_out(double *dst, const T *src, int w, int64_t rows, int pitch, double offset) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= w) return;
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y) {
        const double v = (double)src[r * pitch + c];
        dst[r * w + c] = offset == 0.0 ? v : v + offset;
    }
}
template <class T>
__global__ void k_rows_face_density(double *dst, const T *p, int w, int64_t rows, int pitch, double ro0, double rc2) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= w) return;
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y) dst[r * w + c] = ro0 + (double)p[r * pitch + c] * rc2;
}
// The same conversions with the host array read or written in place (page-locked host memory
// over the host link): the host side walked flat, two doubles per 16-byte access, four accesses
// in flight per thread; the device side scattered into its padded rows.  The host array must
// start on a 16-byte boundary.
template <class T> __global__ void k_flat_in(T *dst, const double2 *src, int w, int64_t n, int pitch, double offset) {
    const int64_t n2 = n >> 1, step = (int64_t)gridDim.x * blockDim.x;
    auto put = [&](int64_t e, double v) {
        const int64_t r = e / w;
        dst[r * pitch + (e - r * w)] = (T)(offset == 0.0 ? v : v - offset);
    };
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n2; q += 4 * step) {
        double2 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (q + u * step < n2) v[u] = src[q + u * step];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (q + u * step < n2) {
                put(2 * (q + u * step), v[u].x);
                put(2 * (q + u * step) + 1, v[u].y);
            }
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) put(n - 1, ((const double *)src)[n - 1]);
}
template <class T> __global__ void k_flat_out(double2 *dst, const T *src, int w, int64_t n, int pitch, double offset) {
    const int64_t n2 = n >> 1, step = (int64_t)gridDim.x * blockDim.x;
    auto get = [&](int64_t e) {
        const int64_t r = e / w;
        const double v = (double)src[r * pitch + (e - r * w)];
        return offset == 0.0 ? v : v + offset;
    };
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n2; q += step)
        dst[q] = make_double2(get(2 * q), get(2 * q + 1));
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) ((double *)dst)[n - 1] = get(n - 1);
}

inline dim3 rows_grid(int w, int64_t rows) {
    return dim3((w + 127) / 128, (unsigned)(rows < 16384 ? (rows < 1 ? 1 : rows) : 16384));
}

template <class T>
void rows_from_double(T *dst, const double *src, int w, int64_t rows, int pitch, double offset, cudaStream_t st) {
    k_rows_in<T><<<rows_grid(w, rows), 128, 0, st>>>(dst, src, w, rows, pitch, offset);
}
template <class T>
void rows_to_double(double *dst, const T *src, int w, int64_t rows, int pitch, double offset, cudaStream_t st) {
    k_rows_out<T><<<rows_grid(w, rows), 128, 0, st>>>(dst, src, w, rows, pitch, offset);
}
template <class T>
void flat_from_host(T *dst, const double *src, int w, int64_t rows, int pitch, double offset, cudaStream_t st) {
    k_flat_in<T><<<152 * 8, 256, 0, st>>>(dst, (const double2 *)src, w, (int64_t)w * rows, pitch, offset);
}
template <class T>
void flat_to_host(double *dst, const T *src, int w, int64_t rows, int pitch, double offset, cudaStream_t st) {
    k_flat_out<T><<<152 * 8, 256, 0, st>>>((double2 *)dst, src, w, (int64_t)w * rows, pitch, offset);
}
template <class T>
void rows_face_density(double *dst, const T *p, int w, int64_t rows, int pitch, double ro0, double rc2, cudaStream_t st) {
    k_rows_face_density<T><<<rows_grid(w, rows), 128, 0, st>>>(dst, p, w, rows, pitch, ro0, rc2);
}

} // namespace ark
