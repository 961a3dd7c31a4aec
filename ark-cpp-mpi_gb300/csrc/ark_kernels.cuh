// CUDA kernels of the CABARET step, templated on the storage/arithmetic type T.
//
// ark_fp64.cu instantiates T = double in a translation unit compiled with --fmad=false:
// every expression below keeps the reference's operand order (source/main.cpp), so the
// FP64 path rounds exactly like the reference built with -ffp-contract=off.
// ark_fp32.cu instantiates T = float with FMA contraction allowed.
//
// Kernels and the reference code they restate:
//   k_reduce_start / k_finalize_dt   TimeStepSize (main.cpp:374-415) + bulk-flow sum
//   k_wrap                           the single-rank halo exchange (main.cpp:603-801,
//                                    1049-1631) as a periodic ghost copy
//   k_phase1<MODE>                   Phase1 (main.cpp:417-575), optionally fused with
//                                    StressTensor's force (main.cpp:856-1023) and
//                                    UseForces (main.cpp:1026-1045)
//   k_stress_faces                   StressTensor's face stresses (main.cpp:856-982)
//   k_sweep_x, k_sweep_col<AX>       Phase2 sweeps (main.cpp:1726-2011, 2023-2255, 2261-2494)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "ark_state.h"

namespace ark {

// ---------------------------------------------------------------------------------------
// scalar helpers
// ---------------------------------------------------------------------------------------

// min3d / max3d of main.cpp:2963-2973: ternaries, a NaN argument is skipped.
template <class T> __device__ __forceinline__ T min3d(T x1, T x2, T x3) {
    x1 = x1 > x2 ? x2 : x1;
    x1 = x1 > x3 ? x3 : x1;
    return x1;
}
template <class T> __device__ __forceinline__ T max3d(T x1, T x2, T x3) {
    x1 = x1 < x2 ? x2 : x1;
    x1 = x1 < x3 ? x3 : x1;
    return x1;
}

// Division by a run constant b whose reciprocal rb is known.  FP64: the IEEE quotient
// (the parity bar).  FP32: multiplication by the reciprocal.
__device__ __forceinline__ double divk(double a, double b, double rb) {
    (void)rb;
    return a / b;
}
__device__ __forceinline__ float divk(float a, float b, float rb) {
    (void)b;
    return a * rb;
}

// Division by a cell-dependent value.
__device__ __forceinline__ double divv(double a, double b) { return a / b; }
__device__ __forceinline__ float divv(float a, float b) { return __fdiv_rn(a, b); }

// Run constants rounded to T.
template <class T> struct K {
    T dx[3], rdx[3], ds[3], dvc, vis, two_vis, sound, ro0, c2, rc2, roc, rroc;
    __device__ __forceinline__ explicit K(const Consts &k) {
        for (int d = 0; d < 3; ++d) {
            dx[d] = (T)k.dx[d];
            rdx[d] = (T)k.rdx[d];
            ds[d] = (T)k.ds[d];
        }
        dvc = (T)k.dvc;
        vis = (T)k.vis;
        two_vis = (T)k.two_vis;
        sound = (T)k.sound;
        ro0 = (T)k.ro0;
        c2 = (T)k.c2;
        rc2 = (T)k.rc2;
        roc = (T)k.roc;
        rroc = (T)k.rroc;
    }
};

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

// Fixed-point image of a value: round(v * 2^32), NaN -> 0, clamped to +-2^30.
__device__ __forceinline__ long long fixed32(double v) {
    if (v != v) v = 0.0;
    v = fmin(fmax(v, -1073741824.0), 1073741824.0);
    return __double2ll_rn(v * 4294967296.0);
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

// Max |u_d| over interior cells of level `con` (dt is monotone in it: min over cells of
// CFL*dx/(c + |u|) is CFL*dx/(c + max|u|) exactly, since IEEE + and / are monotone), and
// the fixed-point sum of u1 over fluid cells of level `ncon`.  Integer max and sum are
// order independent, so any grid gives the same bits.
template <class T>
__global__ void __launch_bounds__(256) k_reduce_start(DevState<T> S, int con, int with_sum) {
    const Geom g = S.g;
    const Level<T> Lc = S.lv[con], Ln = S.lv[con ^ 1];
    const int64_t n = (int64_t)g.C1 * g.C2 * g.C3;
    unsigned long long m0 = 0, m1 = 0, m2 = 0;
    long long s = 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.C1) + 1;
        const int64_t r = t / g.C1;
        const int j = (int)(r % g.C2) + 1;
        const int k = (int)(r / g.C2) + 1;
        const int64_t c = g.cell(i, j, k);
        unsigned long long b0 = abs_bits(Lc.u1[c]), b1 = abs_bits(Lc.u2[c]), b2 = abs_bits(Lc.u3[c]);
        m0 = b0 > m0 ? b0 : m0;
        m1 = b1 > m1 ? b1 : m1;
        m2 = b2 > m2 ? b2 : m2;
        if (with_sum && (S.flags[c] & FL_EQ0)) s += fixed32((double)Ln.u1[c]);
    }
    m0 = warp_max_u64(m0);
    m1 = warp_max_u64(m1);
    m2 = warp_max_u64(m2);
    s = warp_sum_i64(s);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&S.sc->umax[0], m0);
        atomicMax(&S.sc->umax[1], m1);
        atomicMax(&S.sc->umax[2], m2);
        if (with_sum && s != 0) atomicAdd((unsigned long long *)&S.sc->usum, (unsigned long long)s);
    }
}

// One thread: dt as TimeStepSize forms it, then the bulk force, then reset the accumulators.
template <class T> __global__ void k_finalize_dt(DevState<T> S, int advance_time) {
    DevScalars *sc = S.sc;
    const Consts &k = S.k;
    const unsigned long long inf_bits = 0x7FF0000000000000ull;
    if (sc->umax[0] >= inf_bits || sc->umax[1] >= inf_bits || sc->umax[2] >= inf_bits) sc->status |= STATUS_NONFINITE;
    const double M0 = __longlong_as_double((long long)sc->umax[0]);
    const double M1 = __longlong_as_double((long long)sc->umax[1]);
    const double M2 = __longlong_as_double((long long)sc->umax[2]);
    const double dtu1 = k.cfl_dx[0] / (k.sound + M0);
    const double dtu2 = k.cfl_dx[1] / (k.sound + M1);
    const double dtu3 = k.cfl_dx[2] / (k.sound + M2);
    const double dtu = min3d(dtu1, dtu2, dtu3);
    const double dt = min3d(1e8, dtu, k.dtv);
    sc->dt = dt;
    if (k.forcing) {
        const double ub =
            sc->nfluid > 0 ? ((double)sc->usum * (1.0 / 4294967296.0)) / (double)sc->nfluid : 0.0;
        sc->ub = ub;
        sc->G = (k.u_target - ub) / dt;
    }
    if (advance_time) {
        sc->nstep += 1;
        sc->time += 0.5 * dt;
        sc->time += 0.5 * dt;
    }
    sc->umax[0] = sc->umax[1] = sc->umax[2] = 0;
    sc->usum = 0;
}

// ---------------------------------------------------------------------------------------
// ghost fill (periodic x and z)
// ---------------------------------------------------------------------------------------

struct WrapJob {
    void *a[16];
    uint8_t face[16];
    uint8_t axis_mask[16]; // bit 0: wrap in x, bit 1: wrap in z
    int n;
};

// The halo exchange of one rank with itself: ghost 0 <- cell C, ghost C+1 <- cell 1
// (faces: halo 0 <- face C, halo C+2 <- face 2), over the interior of the other axes.
template <class T> __global__ void k_wrap(Geom g, WrapJob J) {
    const int64_t nx = (int64_t)g.C2 * g.C3, nz = (int64_t)g.C1 * g.C2;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nx) {
        const int j = (int)(t % g.C2) + 1, k = (int)(t / g.C2) + 1;
        for (int q = 0; q < J.n; ++q) {
            if (!(J.axis_mask[q] & 1)) continue;
            T *a = (T *)J.a[q];
            if (J.face[q]) {
                a[g.face(0, j, k)] = a[g.face(g.C1, j, k)];
                a[g.face(g.C1 + 2, j, k)] = a[g.face(2, j, k)];
            } else {
                a[g.cell(0, j, k)] = a[g.cell(g.C1, j, k)];
                a[g.cell(g.C1 + 1, j, k)] = a[g.cell(1, j, k)];
            }
        }
    } else if (t < nx + nz) {
        const int64_t u = t - nx;
        const int i = (int)(u % g.C1) + 1, j = (int)(u / g.C1) + 1;
        for (int q = 0; q < J.n; ++q) {
            if (!(J.axis_mask[q] & 2)) continue;
            T *a = (T *)J.a[q];
            if (J.face[q]) {
                a[g.face(i, j, 0)] = a[g.face(i, j, g.C3)];
                a[g.face(i, j, g.C3 + 2)] = a[g.face(i, j, 2)];
            } else {
                a[g.cell(i, j, 0)] = a[g.cell(i, j, g.C3)];
                a[g.cell(i, j, g.C3 + 1)] = a[g.cell(i, j, 1)];
            }
        }
    }
}

// BoundaryConditions::alongX1/2/3 (source/BoundaryConditions.cpp:22-83) on one cell level,
// without the temperature.  axis 1: zero-gradient; axes 2, 3: periodic copy or no-slip.
template <class T> __global__ void k_boundary_fill(Geom g, Level<T> L, int axis, int periodic) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    T *a[4] = {L.u1, L.u2, L.u3, L.ro};
    if (axis == 1) {
        if (t >= (int64_t)g.C2 * g.C3) return;
        const int j = (int)(t % g.C2) + 1, k = (int)(t / g.C2) + 1;
        for (int q = 0; q < 4; ++q) {
            a[q][g.cell(g.C1 + 1, j, k)] = a[q][g.cell(g.C1, j, k)];
            a[q][g.cell(0, j, k)] = a[q][g.cell(1, j, k)];
        }
    } else if (axis == 2) {
        if (t >= (int64_t)g.C1 * g.C3) return;
        const int i = (int)(t % g.C1) + 1, k = (int)(t / g.C1) + 1;
        const int64_t top = g.cell(i, g.C2 + 1, k), bot = g.cell(i, 0, k);
        for (int q = 0; q < 3; ++q) {
            a[q][top] = periodic ? a[q][g.cell(i, 1, k)] : (T)0;
            a[q][bot] = periodic ? a[q][g.cell(i, g.C2, k)] : (T)0;
        }
        a[3][top] = periodic ? a[3][g.cell(i, 1, k)] : a[3][g.cell(i, g.C2, k)];
        a[3][bot] = periodic ? a[3][g.cell(i, g.C2, k)] : a[3][g.cell(i, 1, k)];
    } else {
        if (t >= (int64_t)g.C1 * g.C2) return;
        const int i = (int)(t % g.C1) + 1, j = (int)(t / g.C1) + 1;
        const int64_t top = g.cell(i, j, g.C3 + 1), bot = g.cell(i, j, 0);
        for (int q = 0; q < 3; ++q) {
            a[q][top] = periodic ? a[q][g.cell(i, j, 1)] : (T)0;
            a[q][bot] = periodic ? a[q][g.cell(i, j, g.C3)] : (T)0;
        }
        a[3][top] = periodic ? a[3][g.cell(i, j, 1)] : a[3][g.cell(i, j, g.C3)];
        a[3][bot] = periodic ? a[3][g.cell(i, j, g.C3)] : a[3][g.cell(i, j, 1)];
    }
}

// ---------------------------------------------------------------------------------------
// viscous stress on one face (main.cpp:856-982), component by component
// ---------------------------------------------------------------------------------------

template <class T>
__device__ __forceinline__ T sigma(uint8_t fw, uint8_t fc, T u_cw, T u_c, const K<T> &kk, int d) {
    if ((fw & FL_LT) && (fc & FL_LT)) return divk(kk.vis * (u_c - u_cw), kk.dx[d], kk.rdx[d]);
    if ((fw & FL_LT) && (fc & FL_GT)) return divk(kk.two_vis * (-u_cw), kk.dx[d], kk.rdx[d]);
    if ((fw & FL_GT) && (fc & FL_LT)) return divk(kk.two_vis * u_c, kk.dx[d], kk.rdx[d]);
    return (T)0;
}

// ---------------------------------------------------------------------------------------
// Phase1 (+ stress force, bulk force, UseForces)
// ---------------------------------------------------------------------------------------

// src: the level read as "Con" (the previous "nCon"); dst: the level written as "nCon".
template <class T, int MODE>
__global__ void __launch_bounds__(128) k_phase1(DevState<T> S, int src, int dst) {
    const Geom g = S.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.C1 || j > g.C2) return;
    const K<T> kk(S.k);
    const T dt = (T)S.sc->dt;
    const Level<T> Ls = S.lv[src], Ld = S.lv[dst];
    const int64_t c = g.cell(i, j, k);
    const uint8_t fl = S.flags[c];
    const T ro_c = Ls.ro[c];
    const T uc[3] = {Ls.u1[c], Ls.u2[c], Ls.u3[c]};
    T ro_cn, ucn[3];
    if (fl & FL_LT) {
        const int64_t fw = g.face(i, j, k);
        const int64_t fh[3] = {fw + 1, fw + g.fs1, fw + g.fs2};
        T rl[3], rh[3], pl[3], ph[3], ul[3][3], uh[3][3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const FaceSet<T> F = S.fc[d];
            rl[d] = F.ro[fw];
            rh[d] = F.ro[fh[d]];
            pl[d] = F.p[fw];
            ph[d] = F.p[fh[d]];
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                ul[d][m] = F.u[m][fw];
                uh[d][m] = F.u[m][fh[d]];
            }
        }
        // new density (main.cpp:530-533)
        ro_cn = divk(ro_c * kk.dvc - (T)0.5 * dt * ((rh[0] * uh[0][0] - rl[0] * ul[0][0]) * kk.ds[0] +
                                                    (rh[1] * uh[1][1] - rl[1] * ul[1][1]) * kk.ds[1] +
                                                    (rh[2] * uh[2][2] - rl[2] * ul[2][2]) * kk.ds[2]),
                     kk.dvc, (T)(1.0 / S.k.dvc));
        // momentum (main.cpp:536-551): flux of u_m through faces normal to d is
        // (ro*u_m)*u_d, plus p when m == d
        const T den = ro_cn * kk.dvc;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            T fx[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (m == d)
                    fx[d] = (rh[d] * uh[d][m] * uh[d][d] + ph[d]) - (rl[d] * ul[d][m] * ul[d][d] + pl[d]);
                else
                    fx[d] = rh[d] * uh[d][m] * uh[d][d] - rl[d] * ul[d][m] * ul[d][d];
            }
            ucn[m] = divv(ro_c * uc[m] * kk.dvc - (T)0.5 * dt * (fx[0] * kk.ds[0] + fx[1] * kk.ds[1] + fx[2] * kk.ds[2]),
                          den);
        }
    } else {
        ucn[0] = ucn[1] = ucn[2] = (T)0;
        ro_cn = kk.ro0;
    }

    if (MODE & (P1_STRESS | P1_FORCES)) {
        T f[3];
        if (MODE & P1_STRESS) {
            // StressTensor force of this cell (main.cpp:995-1023) from the six face stresses
            if (fl & FL_EQ0) {
                const int64_t nb[6] = {c - 1, c + 1, c - g.cs1, c + g.cs1, c - g.cs2, c + g.cs2};
                uint8_t fln[6];
                T un[6][3];
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    fln[q] = S.flags[nb[q]];
                    un[q][0] = Ls.u1[nb[q]];
                    un[q][1] = Ls.u2[nb[q]];
                    un[q][2] = Ls.u3[nb[q]];
                }
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
                if (MODE & P1_BULK) f[0] = f[0] + (ro_c * kk.dvc) * (T)S.sc->G;
            } else {
                f[0] = f[1] = f[2] = (T)0;
            }
            S.f[0][c] = f[0];
            S.f[1][c] = f[1];
            S.f[2][c] = f[2];
        } else {
            f[0] = S.f[0][c];
            f[1] = S.f[1][c];
            f[2] = S.f[2][c];
        }
        if ((MODE & P1_FORCES) && (fl & FL_EQ0)) {
            // UseForces (main.cpp:1035-1041)
            const T den = kk.dvc * ro_cn;
#pragma unroll
            for (int m = 0; m < 3; ++m) ucn[m] = divv(ro_cn * kk.dvc * ucn[m] + (T)0.5 * dt * f[m], den);
        }
    }
    Ld.ro[c] = ro_cn;
    Ld.u1[c] = ucn[0];
    Ld.u2[c] = ucn[1];
    Ld.u3[c] = ucn[2];
}

// StressTensor's face stresses into the sigm arrays (kept only on request), faces normal
// to d with index 1..C_d+1 along d (main.cpp:856-982).
template <class T> __global__ void k_stress_faces(DevState<T> S, int con, int d) {
    const Geom g = S.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    const int hi0 = g.C1 + (d == 0), hi1 = g.C2 + (d == 1), hi2 = g.C3 + (d == 2);
    if (i > hi0 || j > hi1 || k > hi2) return;
    const K<T> kk(S.k);
    const Level<T> L = S.lv[con];
    const int64_t c = g.cell(i, j, k);
    const int64_t cw = c - (d == 0 ? 1 : d == 1 ? g.cs1 : g.cs2);
    const uint8_t fc = S.flags[c], fw = S.flags[cw];
    const int64_t fi = g.face(i, j, k);
    S.sig[d][0][fi] = sigma(fw, fc, L.u1[cw], L.u1[c], kk, d);
    S.sig[d][1][fi] = sigma(fw, fc, L.u2[cw], L.u2[c], kk, d);
    S.sig[d][2][fi] = sigma(fw, fc, L.u3[cw], L.u3[c], kk, d);
}

// UseForces alone (main.cpp:1026-1045) on level ncon.
template <class T> __global__ void k_use_forces(DevState<T> S, int ncon) {
    const Geom g = S.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.C1 || j > g.C2) return;
    const int64_t c = g.cell(i, j, k);
    if (!(S.flags[c] & FL_EQ0)) return;
    const K<T> kk(S.k);
    const T dt = (T)S.sc->dt;
    const Level<T> L = S.lv[ncon];
    const T ro_cn = L.ro[c];
    const T den = kk.dvc * ro_cn;
    L.u1[c] = divv(ro_cn * kk.dvc * L.u1[c] + (T)0.5 * dt * S.f[0][c], den);
    L.u2[c] = divv(ro_cn * kk.dvc * L.u2[c] + (T)0.5 * dt * S.f[1][c], den);
    L.u3[c] = divv(ro_cn * kk.dvc * L.u3[c] + (T)0.5 * dt * S.f[2][c], den);
}

// ---------------------------------------------------------------------------------------
// Phase2: characteristic extrapolation, limiter, face update
// ---------------------------------------------------------------------------------------

// What one cell hands to its two faces: forward values (to face s+1) and backward values
// (to face s) of the invariant and the two tangential velocities.
template <class T> struct Ext { T rf, qb, af, ab, bf, bb; };

template <class T> struct SweepK {
    T sound, ro0, c2, rc2, roc, rroc, dt, rdt, dx, rdx;
};

// One cell of a sweep (main.cpp:1756-1873 for x1; the x2 and x3 sweeps are the same with
// the axes permuted).  n: the velocity component normal to the sweep, a/b: tangential.
// Q_USES_R selects the x1/x3 form of the Q-limiter source, 2*(r_cn - r_c)/dt
// (main.cpp:1804, 2321); the x2 sweep uses 2*(q_cn - q_c)/dt (main.cpp:2083).
template <class T, bool Q_USES_R>
__device__ __forceinline__ Ext<T> extrapolate(T u1_f, T u1_b, T u1_cn, T u1_c, T u2_f, T u2_b, T u2_cn,
                                              T u2_c, T u3_f, T u3_b, T u3_cn, T u3_c, T ro_cn, T ro_c,
                                              T p_f, T p_b, const SweepK<T> &q) {
    const T p_cn = q.c2 * (ro_cn - q.ro0);
    const T p_c = q.c2 * (ro_c - q.ro0);
    const T pf = divk(p_f, q.roc, q.rroc), pb = divk(p_b, q.roc, q.rroc);
    const T pcn = divk(p_cn, q.roc, q.rroc), pc = divk(p_c, q.roc, q.rroc);

    const T r_f = u1_f + pf, r_b = u1_b + pb, r_cn = u1_cn + pcn, r_c = u1_c + pc;
    T r_fn = (T)2 * r_cn - r_b;
    const T q_f = u1_f - pf, q_b = u1_b - pb, q_cn = u1_cn - pcn, q_c = u1_c - pc;
    T q_bn = (T)2 * q_cn - q_f;

    T u2_fn = (T)2 * u2_cn - u2_b;
    T u2_bn = (T)2 * u2_cn - u2_f;
    T u3_fn = (T)2 * u3_cn - u3_b;
    T u3_bn = (T)2 * u3_cn - u3_f;

    const T gr = divk((T)2 * (r_cn - r_c), q.dt, q.rdt) + divk((u1_cn + q.sound) * (r_f - r_b), q.dx, q.rdx);
    const T gq = divk((T)2 * (Q_USES_R ? (r_cn - r_c) : (q_cn - q_c)), q.dt, q.rdt) +
                 divk((u1_cn - q.sound) * (q_f - q_b), q.dx, q.rdx);
    const T gu2 = divk((T)2 * (u2_cn - u2_c), q.dt, q.rdt) + divk(u1_cn * (u2_f - u2_b), q.dx, q.rdx);
    const T gu3 = divk((T)2 * (u3_cn - u3_c), q.dt, q.rdt) + divk(u1_cn * (u3_f - u3_b), q.dx, q.rdx);

    const T rmax = max3d(r_f, r_c, r_b) + q.dt * gr;
    const T rmin = min3d(r_f, r_c, r_b) + q.dt * gr;
    const T qmax = max3d(q_f, q_c, q_b) + q.dt * gq;
    const T qmin = min3d(q_f, q_c, q_b) + q.dt * gq;
    const T u2_max = max3d(u2_f, u2_c, u2_b) + q.dt * gu2;
    const T u2_min = min3d(u2_f, u2_c, u2_b) + q.dt * gu2;
    const T u3_max = max3d(u3_f, u3_c, u3_b) + q.dt * gu3;
    const T u3_min = min3d(u3_f, u3_c, u3_b) + q.dt * gu3;

    if (r_fn > rmax) r_fn = rmax;
    if (r_fn < rmin) r_fn = rmin;
    if (q_bn > qmax) q_bn = qmax;
    if (q_bn < qmin) q_bn = qmin;
    if (u2_fn > u2_max) u2_fn = u2_max;
    if (u2_fn < u2_min) u2_fn = u2_min;
    if (u2_bn > u2_max) u2_bn = u2_max;
    if (u2_bn < u2_min) u2_bn = u2_min;
    if (u3_fn > u3_max) u3_fn = u3_max;
    if (u3_fn < u3_min) u3_fn = u3_min;
    if (u3_bn > u3_max) u3_bn = u3_max;
    if (u3_bn < u3_min) u3_bn = u3_min;
    Ext<T> e;
    e.rf = r_fn;
    e.qb = q_bn;
    e.af = u2_fn;
    e.ab = u2_bn;
    e.bf = u3_fn;
    e.bb = u3_bn;
    return e;
}

// Face update (main.cpp:1920-2008).  prev = the cell behind the face (index f-1), cur = the
// cell ahead (index f).  cb/cf index those cells, fc the face; n/a/b the component indices
// of the sweep.  uA_old/uB_old: the face's previous tangential velocities.  WALL_A_FROM_N:
// the x2 sweep takes the tangential u1 from u2nCon in its wall branches (main.cpp:2219,
// 2238).
template <class T, bool WALL_A_FROM_N>
__device__ __forceinline__ void face_update(const DevState<T> &S, const Level<T> &Ln, const FaceSet<T> &F,
                                            int n, int a, int b, int64_t cb, int64_t cf, int64_t fc,
                                            const Ext<T> &prev, const Ext<T> &cur, T uA_old, T uB_old,
                                            const SweepK<T> &q) {
    const T *nN = n == 0 ? Ln.u1 : n == 1 ? Ln.u2 : Ln.u3;
    const T *nA = a == 0 ? Ln.u1 : Ln.u2;
    const T *nB = b == 1 ? Ln.u2 : Ln.u3;
    const uint8_t flb = S.flags[cb], flf = S.flags[cf];
    T un, pn, ro_n, ua, ub;
    if ((flb & FL_LT) && (flf & FL_LT)) {
        const T rn = prev.rf, qn = cur.qb;
        un = (rn + qn) / (T)2;
        pn = (rn - qn) * q.sound * q.ro0 / (T)2;
        ro_n = q.ro0 + divk(pn, q.c2, q.rc2);
        const T ucf = nN[cf], ucb = nN[cb];
        if (ucf >= (T)0 && ucb >= (T)0) {
            ua = prev.af;
            ub = prev.bf;
        } else if (ucf <= (T)0 && ucb <= (T)0) {
            ua = cur.ab;
            ub = cur.bb;
        } else if (ucb >= (T)0 && ucf <= (T)0) {
            if (ucb > -ucf) {
                ua = prev.af;
                ub = prev.bf;
            } else {
                ua = cur.ab;
                ub = cur.bb;
            }
        } else {
            ua = nA[cf] + nA[cb] - uA_old;
            ub = nB[cf] + nB[cb] - uB_old;
        }
    } else {
        un = (T)0;
        if ((flb & FL_GT) && (flf & FL_LT)) {
            if (nN[cf] <= (T)0) {
                const T qn = cur.qb;
                pn = -qn * q.sound * q.ro0;
                ro_n = q.ro0 + divk(pn, q.c2, q.rc2);
                ua = cur.ab;
                ub = cur.bb;
            } else {
                ro_n = Ln.ro[cf];
                pn = (ro_n - q.ro0) * q.c2;
                ua = WALL_A_FROM_N ? nN[cf] : nA[cf];
                ub = nB[cf];
            }
        } else if ((flb & FL_LT) && (flf & FL_GT)) {
            if (nN[cb] >= (T)0) {
                const T rn = prev.rf;
                pn = rn * q.sound * q.ro0;
                ro_n = q.ro0 + divk(pn, q.c2, q.rc2);
                ua = prev.af;
                ub = prev.bf;
            } else {
                ro_n = Ln.ro[cb];
                pn = (ro_n - q.ro0) * q.c2;
                ua = WALL_A_FROM_N ? nN[cb] : nA[cb];
                ub = nB[cb];
            }
        } else {
            pn = (T)0;
            ro_n = q.ro0;
            ua = (T)0;
            ub = (T)0;
        }
    }
    F.p[fc] = pn;
    F.u[n][fc] = un;
    F.ro[fc] = ro_n;
    F.u[a][fc] = ua;
    F.u[b][fc] = ub;
}

template <class T> __device__ __forceinline__ SweepK<T> sweep_consts(const DevState<T> &S, int d) {
    SweepK<T> q;
    const double dt = S.sc->dt;
    q.sound = (T)S.k.sound;
    q.ro0 = (T)S.k.ro0;
    q.c2 = (T)S.k.c2;
    q.rc2 = (T)S.k.rc2;
    q.roc = (T)S.k.roc;
    q.rroc = (T)S.k.rroc;
    q.dt = (T)dt;
    q.rdt = (T)(1.0 / dt);
    q.dx = (T)S.k.dx[d];
    q.rdx = (T)S.k.rdx[d];
    return q;
}

// x1 sweep: one warp per (j,k) line, lanes on consecutive cells (coalesced), marching along
// i in chunks of 32.  A face needs the forward values of the cell behind it: a shuffle
// from the neighbouring lane, or the carry from the previous chunk's last lane.  Each
// warp owns all faces of its line, so the faces are updated in place.
template <class T> __global__ void __launch_bounds__(128) k_sweep_x(DevState<T> S, int con) {
    const Geom g = S.g;
    const int lane = threadIdx.x & 31;
    const int line = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    if (line >= g.C2 * g.C3) return;
    const int j = line % g.C2 + 1, k = line / g.C2 + 1;
    const Level<T> Lc = S.lv[con], Ln = S.lv[con ^ 1];
    const FaceSet<T> F = S.fc[0];
    const SweepK<T> q = sweep_consts(S, 0);
    const int64_t c0 = g.cell(0, j, k), f0 = g.face(0, j, k);
    const int nd = g.C1 + 1;
    Ext<T> carry = {};
    for (int s0 = 0; s0 <= nd; s0 += 32) {
        const int s = s0 + lane;
        const bool act = s <= nd;
        Ext<T> e = {};
        T uA_old = 0, uB_old = 0;
        if (act) {
            const int64_t c = c0 + s, fb = f0 + s, ff = fb + 1;
            uA_old = F.u[1][fb];
            uB_old = F.u[2][fb];
            e = extrapolate<T, true>(F.u[0][ff], F.u[0][fb], Ln.u1[c], Lc.u1[c], F.u[1][ff], uA_old, Ln.u2[c],
                                     Lc.u2[c], F.u[2][ff], uB_old, Ln.u3[c], Lc.u3[c], Ln.ro[c], Lc.ro[c],
                                     F.p[ff], F.p[fb], q);
        }
        Ext<T> prev;
        prev.rf = __shfl_up_sync(0xffffffffu, e.rf, 1);
        prev.af = __shfl_up_sync(0xffffffffu, e.af, 1);
        prev.bf = __shfl_up_sync(0xffffffffu, e.bf, 1);
        if (lane == 0) {
            prev.rf = carry.rf;
            prev.af = carry.af;
            prev.bf = carry.bf;
        }
        carry.rf = __shfl_sync(0xffffffffu, e.rf, 31);
        carry.af = __shfl_sync(0xffffffffu, e.af, 31);
        carry.bf = __shfl_sync(0xffffffffu, e.bf, 31);
        __syncwarp();
        if (act && s >= 1)
            face_update<T, false>(S, Ln, F, 0, 1, 2, c0 + s - 1, c0 + s, f0 + s, prev, e, uA_old, uB_old, q);
        __syncwarp();
    }
}

// x2 (AX = 1) and x3 (AX = 2) sweeps: one thread per line, threads on consecutive i
// (coalesced), marching along the sweep axis; the face behind the current cell is carried
// in registers, so every face is read once and updated in place.
template <class T, int AX> __global__ void __launch_bounds__(128) k_sweep_col(DevState<T> S, int con) {
    const Geom g = S.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int o = blockIdx.y + 1;
    if (i > g.C1) return;
    const Level<T> Lc = S.lv[con], Ln = S.lv[con ^ 1];
    const FaceSet<T> F = S.fc[AX];
    const SweepK<T> q = sweep_consts(S, AX);
    constexpr int A = 0, B = (AX == 1) ? 2 : 1;
    const int64_t cst = AX == 1 ? g.cs1 : g.cs2, fst = AX == 1 ? g.fs1 : g.fs2;
    const int64_t c0 = AX == 1 ? g.cell(i, 0, o) : g.cell(i, o, 0);
    const int64_t f0 = AX == 1 ? g.face(i, 0, o) : g.face(i, o, 0);
    const int nd = (AX == 1 ? g.C2 : g.C3) + 1;
    const T *cN = AX == 1 ? Lc.u2 : Lc.u3, *nN = AX == 1 ? Ln.u2 : Ln.u3;
    const T *cA = Lc.u1, *nA = Ln.u1;
    const T *cB = B == 2 ? Lc.u3 : Lc.u2, *nB = B == 2 ? Ln.u3 : Ln.u2;
    T uN_b = F.u[AX][f0], uA_b = F.u[A][f0], uB_b = F.u[B][f0], p_b = F.p[f0];
    Ext<T> prev = {};
    for (int s = 0; s <= nd; ++s) {
        const int64_t c = c0 + s * cst, ff = f0 + (s + 1) * fst;
        const T uN_f = F.u[AX][ff], uA_f = F.u[A][ff], uB_f = F.u[B][ff], p_f = F.p[ff];
        const Ext<T> e = extrapolate<T, AX == 2>(uN_f, uN_b, nN[c], cN[c], uA_f, uA_b, nA[c], cA[c], uB_f, uB_b,
                                                 nB[c], cB[c], Ln.ro[c], Lc.ro[c], p_f, p_b, q);
        if (s >= 1) face_update<T, AX == 1>(S, Ln, F, AX, A, B, c - cst, c, f0 + s * fst, prev, e, uA_b, uB_b, q);
        prev = e;
        uN_b = uN_f;
        uA_b = uA_f;
        uB_b = uB_f;
        p_b = p_f;
    }
}

// ---------------------------------------------------------------------------------------
// conservation sums of one level (fixed point: identical for any grid)
// ---------------------------------------------------------------------------------------

template <class T> __global__ void __launch_bounds__(256) k_sums(DevState<T> S, int ncon) {
    const Geom g = S.g;
    const Level<T> L = S.lv[ncon];
    const int64_t n = (int64_t)g.C1 * g.C2 * g.C3;
    long long a[5] = {0, 0, 0, 0, 0}, cnt = 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.C1) + 1;
        const int64_t r = t / g.C1;
        const int j = (int)(r % g.C2) + 1;
        const int k = (int)(r / g.C2) + 1;
        const int64_t c = g.cell(i, j, k);
        if (!(S.flags[c] & FL_EQ0)) continue;
        const double ro = L.ro[c], u1 = L.u1[c], u2 = L.u2[c], u3 = L.u3[c];
        a[0] += fixed32(ro);
        a[1] += fixed32(ro * u1);
        a[2] += fixed32(ro * u2);
        a[3] += fixed32(ro * u3);
        a[4] += fixed32((u1 * u1 + u2 * u2 + u3 * u3) / 2);
        cnt += 1;
    }
    for (int q = 0; q < 5; ++q) a[q] = warp_sum_i64(a[q]);
    cnt = warp_sum_i64(cnt);
    if ((threadIdx.x & 31) == 0) {
        for (int q = 0; q < 5; ++q) atomicAdd((unsigned long long *)&S.sc->sums[q], (unsigned long long)a[q]);
        atomicAdd((unsigned long long *)&S.sc->sum_cells, (unsigned long long)cnt);
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

template <class T> inline void cell_grid(const Geom &g, dim3 &grid, dim3 &block) {
    block = dim3(g.C1 >= 64 ? 64 : 32, 2, 1);
    grid = dim3((g.C1 + block.x - 1) / block.x, (g.C2 + block.y - 1) / block.y, g.C3);
}

template <class T>
void Launch<T>::reduce_start(const DevState<T> &S, int con, int with_sum, cudaStream_t st) {
    const int64_t n = (int64_t)S.g.C1 * S.g.C2 * S.g.C3;
    k_reduce_start<T><<<grid_for(n, 256, 152 * 8), 256, 0, st>>>(S, con, with_sum);
}

template <class T> void Launch<T>::finalize_dt(const DevState<T> &S, int advance_time, cudaStream_t st) {
    k_finalize_dt<T><<<1, 1, 0, st>>>(S, advance_time);
}

template <class T> void Launch<T>::wrap_cells(const DevState<T> &S, T *const *arrs, int n, cudaStream_t st) {
    WrapJob J = {};
    J.n = n;
    for (int q = 0; q < n; ++q) {
        J.a[q] = arrs[q];
        J.face[q] = 0;
        J.axis_mask[q] = 3;
    }
    const int64_t tot = (int64_t)S.g.C2 * S.g.C3 + (int64_t)S.g.C1 * S.g.C2;
    k_wrap<T><<<grid_for(tot, 256, 1 << 30), 256, 0, st>>>(S.g, J);
}

// The halo exchange before Phase2 (main.cpp:1049-1631): cells u?nCon, ronCon and roCon in x
// and z; faces normal to x1 wrapped in x, faces normal to x3 wrapped in z.
template <class T> void Launch<T>::wrap_phase2(const DevState<T> &S, int con, cudaStream_t st) {
    WrapJob J = {};
    const Level<T> Ln = S.lv[con ^ 1], Lc = S.lv[con];
    T *cells[5] = {Ln.u1, Ln.u2, Ln.u3, Ln.ro, Lc.ro};
    int n = 0;
    for (int q = 0; q < 5; ++q) {
        J.a[n] = cells[q];
        J.face[n] = 0;
        J.axis_mask[n++] = 3;
    }
    T *fx[5] = {S.fc[0].p, S.fc[0].ro, S.fc[0].u[0], S.fc[0].u[1], S.fc[0].u[2]};
    T *fz[5] = {S.fc[2].p, S.fc[2].ro, S.fc[2].u[0], S.fc[2].u[1], S.fc[2].u[2]};
    for (int q = 0; q < 5; ++q) {
        J.a[n] = fx[q];
        J.face[n] = 1;
        J.axis_mask[n++] = 1;
    }
    for (int q = 0; q < 5; ++q) {
        J.a[n] = fz[q];
        J.face[n] = 1;
        J.axis_mask[n++] = 2;
    }
    J.n = n;
    const int64_t tot = (int64_t)S.g.C2 * S.g.C3 + (int64_t)S.g.C1 * S.g.C2;
    k_wrap<T><<<grid_for(tot, 256, 1 << 30), 256, 0, st>>>(S.g, J);
}

template <class T> void Launch<T>::phase1(const DevState<T> &S, int src, int dst, int mode, cudaStream_t st) {
    dim3 grid, block;
    cell_grid<T>(S.g, grid, block);
    switch (mode) {
    case P1_PLAIN: k_phase1<T, P1_PLAIN><<<grid, block, 0, st>>>(S, src, dst); break;
    case P1_STRESS | P1_FORCES: k_phase1<T, P1_STRESS | P1_FORCES><<<grid, block, 0, st>>>(S, src, dst); break;
    case P1_STRESS | P1_FORCES | P1_BULK:
        k_phase1<T, P1_STRESS | P1_FORCES | P1_BULK><<<grid, block, 0, st>>>(S, src, dst);
        break;
    case P1_FORCES: k_phase1<T, P1_FORCES><<<grid, block, 0, st>>>(S, src, dst); break;
    default: break;
    }
}

// StressTensor alone: the force (the same device code as the fused Phase1 computes it,
// with nothing else written) and, on request, the face stresses.
template <class T> __global__ void k_stress_force(DevState<T> S, int con, int bulk) {
    const Geom g = S.g;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int k = blockIdx.z + 1;
    if (i > g.C1 || j > g.C2) return;
    const K<T> kk(S.k);
    const Level<T> L = S.lv[con];
    const int64_t c = g.cell(i, j, k);
    const uint8_t fl = S.flags[c];
    T f[3] = {(T)0, (T)0, (T)0};
    if (fl & FL_EQ0) {
        const T ro_c = L.ro[c];
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
        for (int m = 0; m < 3; ++m) {
            T sw[3], se[3];
            for (int d = 0; d < 3; ++d) {
                sw[d] = sigma(fln[2 * d], fl, un[2 * d][m], uc[m], kk, d);
                se[d] = sigma(fl, fln[2 * d + 1], uc[m], un[2 * d + 1][m], kk, d);
            }
            f[m] = ((se[0] - sw[0]) * kk.ds[0] + (se[1] - sw[1]) * kk.ds[1] + (se[2] - sw[2]) * kk.ds[2]) * ro_c;
        }
        if (bulk) f[0] = f[0] + (ro_c * kk.dvc) * (T)S.sc->G;
    }
    S.f[0][c] = f[0];
    S.f[1][c] = f[1];
    S.f[2][c] = f[2];
}

template <class T> void Launch<T>::stress(const DevState<T> &S, int con, int bulk, cudaStream_t st) {
    dim3 grid, block;
    cell_grid<T>(S.g, grid, block);
    k_stress_force<T><<<grid, block, 0, st>>>(S, con, bulk);
    if (S.sig[0][0]) {
        for (int d = 0; d < 3; ++d) {
            dim3 gd((S.g.C1 + (d == 0) + block.x - 1) / block.x, (S.g.C2 + (d == 1) + block.y - 1) / block.y,
                    S.g.C3 + (d == 2));
            k_stress_faces<T><<<gd, block, 0, st>>>(S, con, d);
        }
    }
}

template <class T> void Launch<T>::use_forces(const DevState<T> &S, int ncon, cudaStream_t st) {
    dim3 grid, block;
    cell_grid<T>(S.g, grid, block);
    k_use_forces<T><<<grid, block, 0, st>>>(S, ncon);
}

template <class T> void Launch<T>::sweep(const DevState<T> &S, int con, int axis, cudaStream_t st) {
    if (axis == 0) {
        const int lines_x = S.g.C2 * S.g.C3;
        k_sweep_x<T><<<(lines_x + 3) / 4, 128, 0, st>>>(S, con);
    } else if (axis == 1) {
        k_sweep_col<T, 1><<<dim3((S.g.C1 + 127) / 128, S.g.C3), 128, 0, st>>>(S, con);
    } else {
        k_sweep_col<T, 2><<<dim3((S.g.C1 + 127) / 128, S.g.C2), 128, 0, st>>>(S, con);
    }
}

template <class T>
void Launch<T>::boundary_fill(const DevState<T> &S, int ncon, int axis, int periodic, cudaStream_t st) {
    const int64_t n = axis == 1 ? (int64_t)S.g.C2 * S.g.C3 : axis == 2 ? (int64_t)S.g.C1 * S.g.C3
                                                                       : (int64_t)S.g.C1 * S.g.C2;
    k_boundary_fill<T><<<grid_for(n, 256, 1 << 30), 256, 0, st>>>(S.g, S.lv[ncon], axis, periodic);
}

template <class T> void Launch<T>::sums(const DevState<T> &S, int ncon, cudaStream_t st) {
    const int64_t n = (int64_t)S.g.C1 * S.g.C2 * S.g.C3;
    k_sums<T><<<grid_for(n, 256, 152 * 8), 256, 0, st>>>(S, ncon);
}

} // namespace ark

namespace ark {

// Precision conversion for FP32 contexts (host arrays are always double).
template <class T> __global__ void k_from_double(T *dst, const double *src, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        dst[t] = (T)src[t];
}
template <class T> __global__ void k_to_double(double *dst, const T *src, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        dst[t] = (double)src[t];
}

template <class T> void convert_from_double(T *dst, const double *src, int64_t n, cudaStream_t st) {
    k_from_double<T><<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(dst, src, n);
}
template <class T> void convert_to_double(double *dst, const T *src, int64_t n, cudaStream_t st) {
    k_to_double<T><<<grid_for(n, 256, 152 * 16), 256, 0, st>>>(dst, src, n);
}

} // namespace ark
