// The learned eddy-viscosity closure (a project extension; the reference has none).
//
//   * training data: the "nCon" velocities of a (fine) context, 3 x 3 x 3 box-filtered on the
//     device, give per sampled cell 10 features of the filtered velocity gradient and the
//     least-squares eddy viscosity of the filtered-out stress as the target;
//   * network: 10 -> 32 (GELU) -> 32 (GELU) -> 1 (softplus) = nu_t / nu, BF16 weights, FP32
//     accumulation; trained by the kernels here (the layers' products over a tile of samples as
//     BF16 tensor-core multiplies with two-term BF16 operands, tile-wise fixed-order gradient
//     sums, Adam on FP32 master weights);
//   * inference: nu_t of every cell of a (coarse) FP32 context before its stress, which then
//     uses nu + nu_t averaged to each face.
// Definitions (filter, features, target, network) are restated in numpy in oracle/closure.py.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ark_gpu.h"
#include "ark_check.cuh"
#include "ark_state.h"

namespace ark {
namespace cl {

constexpr int NIN = 10, NH = 32;
constexpr int NPARAM = NH * NIN + NH + NH * NH + NH + NH + 1; // 1441
constexpr int O_W1 = 0, O_B1 = O_W1 + NH * NIN, O_W2 = O_B1 + NH, O_B2 = O_W2 + NH * NH, O_W3 = O_B2 + NH,
              O_B3 = O_W3 + NH;
static_assert(O_B3 + 1 == NPARAM, "parameter layout");

// ---- network ------------------------------------------------------------------------------

// GELU in its tanh form, z (1 + tanh(k0 (z + k1 z^3))) / 2, and its derivative (training:
// accurate tanhf)
constexpr float GK0 = 0.79788456080286536f, GK1 = 0.044715f;
__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + tanhf(GK0 * (z + GK1 * z * z * z))); }
__device__ __forceinline__ float gelu_grad(float z) {
    const float th = tanhf(GK0 * (z + GK1 * z * z * z));
    return 0.5f * (1.0f + th) + 0.5f * z * (1.0f - th * th) * GK0 * (1.0f + 3.0f * GK1 * z * z);
}
// inference: the same form with the hardware tanh approximation (relative error below 2^-10)
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float gelu_fast(float z) { return 0.5f * z * (1.0f + tanh_approx(GK0 * (z + GK1 * z * z * z))); }
__device__ __forceinline__ float softplus(float z) { return fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z))); }
__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + expf(-z)); }

// Network constants as the kernels read them: weights (BF16 values held as float), input
// normalisation.
struct Net {
    float w[NPARAM];
    float mu[NIN], rsd[NIN];
};

// nu_t / nu of one normalised input, fully unrolled (with the parameters a kernel argument,
// every multiply-add takes its weight from the constant bank)
__device__ __forceinline__ float mlp_forward_unrolled(const float *w, const float xn[NIN]) {
    float h1[NH];
#pragma unroll
    for (int k = 0; k < NH; ++k) {
        float z = w[O_B1 + k];
#pragma unroll
        for (int i = 0; i < NIN; ++i) z += w[O_W1 + k * NIN + i] * xn[i];
        h1[k] = gelu(z);
    }
    float z3 = w[O_B3];
#pragma unroll
    for (int k = 0; k < NH; ++k) {
        float z = w[O_B2 + k];
#pragma unroll
        for (int m = 0; m < NH; ++m) z += w[O_W2 + k * NH + m] * h1[m];
        z3 += w[O_W3 + k] * gelu(z);
    }
    return softplus(z3);
}

// nu_t / nu of one normalised input (w: the parameters, in shared memory)
__device__ __forceinline__ float mlp_forward(const float *w, const float xn[NIN]) {
    float h1[NH];
#pragma unroll 4
    for (int k = 0; k < NH; ++k) {
        float z = w[O_B1 + k];
#pragma unroll
        for (int i = 0; i < NIN; ++i) z += w[O_W1 + k * NIN + i] * xn[i];
        h1[k] = gelu(z);
    }
    float z3 = w[O_B3];
#pragma unroll 2
    for (int k = 0; k < NH; ++k) {
        float z = w[O_B2 + k];
#pragma unroll
        for (int m = 0; m < NH; ++m) z += w[O_W2 + k * NH + m] * h1[m];
        z3 += w[O_W3 + k] * gelu(z);
    }
    return softplus(z3);
}

// ---- tensor-core inference ----------------------------------------------------------------
// A warp evaluates 32 inputs at once with warp-level BF16 matrix multiply-accumulate
// (m16n8k16, FP32 accumulation): layer 1 is [16 x 16] x [16 x 32] per half-warp tile (inputs
// padded from 10 to 16), layer 2 [16 x 32] x [32 x 32]; the FP32 accumulator fragment of a
// layer, after bias and GELU, is in exactly the register layout of the next layer's A fragment
// (rows = inputs, columns = units), packed to BF16 pairs.  Layer 3 (32 -> 1) is a dot product
// reduced over the four threads of a quad.  Activations enter the multiplies as BF16.

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<unsigned *>(&v);
}
__device__ __forceinline__ void mma_bf16(float c[4], const unsigned a[4], unsigned b0, unsigned b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// The B fragments of a thread (lane = 4 g + t): layer 1 n-tile j: W1 rows 8j+g, inputs 2t, 2t+1
// and 2t+8, 2t+9 (inputs >= 10 are zero); layer 2 n-tile j, k-step s: W2 row 8j+g, inputs
// 16s+2t(+1), 16s+2t+8(+9).
struct TcWeights {
    unsigned b1[4][2], b2[4][2][2];
};
__device__ __forceinline__ TcWeights tc_weights(const float *w, int lane) {
    const int g = lane >> 2, t = lane & 3;
    TcWeights r;
    auto w1 = [&](int n, int k) { return k < NIN ? w[O_W1 + n * NIN + k] : 0.f; };
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int n = 8 * j + g;
        r.b1[j][0] = pack_bf16(w1(n, 2 * t), w1(n, 2 * t + 1));
        r.b1[j][1] = pack_bf16(w1(n, 2 * t + 8), w1(n, 2 * t + 9));
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            r.b2[j][s][0] = pack_bf16(w[O_W2 + n * NH + 16 * s + 2 * t], w[O_W2 + n * NH + 16 * s + 2 * t + 1]);
            r.b2[j][s][1] = pack_bf16(w[O_W2 + n * NH + 16 * s + 2 * t + 8], w[O_W2 + n * NH + 16 * s + 2 * t + 9]);
        }
    }
    return r;
}

// nu_t / nu of the 16 inputs of one m16 tile, whose normalised features (BF16, 16 per row, the
// last 6 zero) are rows X[0..15] in shared memory; out[0] gets row g, out[1] row g + 8 (every
// thread of the quad holds both).
__device__ __forceinline__ void tc_tile(const float *w, const TcWeights &B, const __nv_bfloat16 *X, int lane, float out[2]) {
    const int g = lane >> 2, t = lane & 3;
    const unsigned *Xw = reinterpret_cast<const unsigned *>(X); // 8 words per row
    unsigned a[4];
    a[0] = Xw[g * 8 + t];
    a[1] = Xw[(g + 8) * 8 + t];
    a[2] = Xw[g * 8 + 4 + t];
    a[3] = Xw[(g + 8) * 8 + 4 + t];
    float h[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        mma_bf16(c, a, B.b1[j][0], B.b1[j][1]);
        const float bl = w[O_B1 + 8 * j + 2 * t], bh = w[O_B1 + 8 * j + 2 * t + 1];
        h[j][0] = gelu_fast(c[0] + bl);
        h[j][1] = gelu_fast(c[1] + bh);
        h[j][2] = gelu_fast(c[2] + bl);
        h[j][3] = gelu_fast(c[3] + bh);
    }
    unsigned a2[2][4];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        a2[s][0] = pack_bf16(h[2 * s][0], h[2 * s][1]);
        a2[s][1] = pack_bf16(h[2 * s][2], h[2 * s][3]);
        a2[s][2] = pack_bf16(h[2 * s + 1][0], h[2 * s + 1][1]);
        a2[s][3] = pack_bf16(h[2 * s + 1][2], h[2 * s + 1][3]);
    }
    float z_lo = 0.f, z_hi = 0.f;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        mma_bf16(c, a2[0], B.b2[j][0][0], B.b2[j][0][1]);
        mma_bf16(c, a2[1], B.b2[j][1][0], B.b2[j][1][1]);
        const int n = 8 * j + 2 * t;
        const float bl = w[O_B2 + n], bh = w[O_B2 + n + 1], wl = w[O_W3 + n], wh = w[O_W3 + n + 1];
        z_lo += gelu_fast(c[0] + bl) * wl + gelu_fast(c[1] + bh) * wh;
        z_hi += gelu_fast(c[2] + bl) * wl + gelu_fast(c[3] + bh) * wh;
    }
    z_lo += __shfl_xor_sync(0xffffffffu, z_lo, 1);
    z_lo += __shfl_xor_sync(0xffffffffu, z_lo, 2);
    z_hi += __shfl_xor_sync(0xffffffffu, z_hi, 1);
    z_hi += __shfl_xor_sync(0xffffffffu, z_hi, 2);
    out[0] = softplus(z_lo + w[O_B3]);
    out[1] = softplus(z_hi + w[O_B3]);
}

// A warp's 32 inputs: this lane's normalised features x into row `lane` of the warp's X (32
// rows of 16 BF16), then both m16 tiles; returns nu_t / nu of this lane's input.
__device__ __forceinline__ float tc_warp(const float *w, const TcWeights &B, __nv_bfloat16 *X, const float x[NIN], int lane) {
    unsigned *row = reinterpret_cast<unsigned *>(X + lane * 16);
#pragma unroll
    for (int q = 0; q < 5; ++q) row[q] = pack_bf16(x[2 * q], x[2 * q + 1]);
    row[5] = row[6] = row[7] = 0u;
    __syncwarp();
    float o0[2], o1[2];
    tc_tile(w, B, X, lane, o0);
    tc_tile(w, B, X + 16 * 16, lane, o1);
    __syncwarp();
    // row r of tile m: held by every thread of quad (r mod 8); hand each lane its own row
    const int src = (lane & 7) * 4;
    const float a0 = __shfl_sync(0xffffffffu, o0[0], src), a1 = __shfl_sync(0xffffffffu, o0[1], src);
    const float b0 = __shfl_sync(0xffffffffu, o1[0], src), b1 = __shfl_sync(0xffffffffu, o1[1], src);
    return lane < 8 ? a0 : lane < 16 ? a1 : lane < 24 ? b0 : b1;
}

// ---- features -----------------------------------------------------------------------------

// signed roots x^(1/3), x^(1/4), x^(1/6) of |x| with the sign of x
__device__ __forceinline__ float sroot3(float x) { return cbrtf(x); }
__device__ __forceinline__ float sroot4(float x) { return copysignf(sqrtf(sqrtf(fabsf(x))), x); }
__device__ __forceinline__ float sroot6(float x) { return copysignf(cbrtf(sqrtf(fabsf(x))), x); }
__device__ __forceinline__ double sroot3(double x) { return cbrt(x); }
__device__ __forceinline__ double sroot4(double x) { return copysign(sqrt(sqrt(fabs(x))), x); }
__device__ __forceinline__ double sroot6(double x) { return copysign(cbrt(sqrt(fabs(x))), x); }

// The 10 raw features from the velocity gradient A[m][d] = d u_m / d x_d of a cell at height y
// (R = float for inference, double for training data).
template <class R>
__device__ __forceinline__ void features_of(const R A[3][3], R y, R ly, R yplus_scale, R f[NIN]) {
    R S[3][3], W[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            S[a][b] = 0.5f * (A[a][b] + A[b][a]);
            W[a][b] = 0.5f * (A[a][b] - A[b][a]);
        }
    R S2[3][3], W2[3][3], W2S[3][3], W2S2[3][3], WS2[3][3];
    auto mul = [](const R X[3][3], const R Y[3][3], R Z[3][3]) {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) Z[a][b] = X[a][0] * Y[0][b] + X[a][1] * Y[1][b] + X[a][2] * Y[2][b];
    };
    auto tr_of = [](const R X[3][3], const R Y[3][3]) {
        R t = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) t += X[a][b] * Y[b][a];
        return t;
    };
    mul(S, S, S2);
    mul(W, W, W2);
    mul(W2, S, W2S);
    mul(W2S, S, W2S2);
    mul(W, S2, WS2);
    const R trS = S[0][0] + S[1][1] + S[2][2];
    const R trS2 = S2[0][0] + S2[1][1] + S2[2][2];
    const R trW2 = W2[0][0] + W2[1][1] + W2[2][2];
    f[0] = trS;
    f[1] = sqrt(trS2 > 0 ? trS2 : (R)0);
    f[2] = sqrt(-trW2 > 0 ? -trW2 : (R)0);
    f[3] = sroot3(tr_of(S2, S));
    f[4] = sroot3(W2S[0][0] + W2S[1][1] + W2S[2][2]);
    f[5] = sroot4(W2S2[0][0] + W2S2[1][1] + W2S2[2][2]);
    f[6] = sroot6(tr_of(W2S, WS2));
    const R sg = y > 0 ? (R)-1 : (y < 0 ? (R)1 : (R)0);
    f[7] = sg * S[0][1];
    f[8] = sg * W[0][1];
    f[9] = ((R)0.5 * ly - fabs(y)) * yplus_scale;
}

// ---- dataset kernels (compact interior arrays [k][j][i], float) --------------------------

template <class T> __global__ void k_gather(const __grid_constant__ DevState<T> S, int lvl, double *u0, double *u1, double *u2) {
    const Geom g = S.g;
    const int n = g.C1 * g.C2 * g.C3;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int i = t % g.C1, r = t / g.C1, j = r % g.C2, k = r / g.C2;
        const int64_t c = g.cell(i + 1, j + 1, k + 1);
        u0[t] = (double)S.lv[lvl].u1[c];
        u1[t] = (double)S.lv[lvl].u2[c];
        u2[t] = (double)S.lv[lvl].u3[c];
    }
}

__global__ void k_products(const double *u0, const double *u1, const double *u2, double *p, int n) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const double a = u0[t], b = u1[t], c = u2[t];
        p[0 * (size_t)n + t] = a * a;
        p[1 * (size_t)n + t] = a * b;
        p[2 * (size_t)n + t] = a * c;
        p[3 * (size_t)n + t] = b * b;
        p[4 * (size_t)n + t] = b * c;
        p[5 * (size_t)n + t] = c * c;
    }
}

// One three-point pass of the box filter along axis d (FP64); y treats j = -1 and j = C2 as
// solid (sign * a_c).
__global__ void k_filter_pass(const double *in, double *out, int C1, int C2, int C3, int d, double sign) {
    const int n = C1 * C2 * C3;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int i = t % C1, r = t / C1, j = r % C2, k = r / C2;
        const double c = in[t];
        double lo, hi;
        if (d == 0) {
            lo = in[t - i + (i == 0 ? C1 - 1 : i - 1)];
            hi = in[t - i + (i == C1 - 1 ? 0 : i + 1)];
        } else if (d == 1) {
            lo = j == 0 ? sign * c : in[t - C1];
            hi = j == C2 - 1 ? sign * c : in[t + C1];
        } else {
            const int pl = C1 * C2;
            lo = in[t + ((k == 0 ? C3 - 1 : k - 1) - k) * pl];
            hi = in[t + ((k == C3 - 1 ? 0 : k + 1) - k) * pl];
        }
        out[t] = (lo + c + hi) / 3.0;
    }
}

// gradient of compact arrays at (i, j, k): x, z periodic, y walls (solid neighbour = -u_c)
__device__ __forceinline__ void grad_compact(const double *const u[3], int i, int j, int k, int C1, int C2, int C3,
                                             const double rdx2[3], double A[3][3]) {
    const int pl = C1 * C2, t = (k * C2 + j) * C1 + i;
    const int im = t - i + (i == 0 ? C1 - 1 : i - 1), ip = t - i + (i == C1 - 1 ? 0 : i + 1);
    const int km = t + ((k == 0 ? C3 - 1 : k - 1) - k) * pl, kp = t + ((k == C3 - 1 ? 0 : k + 1) - k) * pl;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const double c = u[m][t];
        const double jl = j == 0 ? -c : u[m][t - C1], jh = j == C2 - 1 ? -c : u[m][t + C1];
        A[m][0] = (u[m][ip] - u[m][im]) * rdx2[0];
        A[m][1] = (jh - jl) * rdx2[1];
        A[m][2] = (u[m][kp] - u[m][km]) * rdx2[2];
    }
}

struct SampleArgs {
    const double *ub[3]; // filtered velocities
    const double *pb;    // filtered products (6 fields: 11 12 13 22 23 33)
    float *feat, *targ;  // dataset rows written from `at`
    long long at;
    int C1, C2, C3, sx, sz, ox, oz, nx, nz;
    double rdx2[3], ly, dy, yplus_scale, rnu;
};

// Features of the filtered field and the least-squares target at the sampled cells (i = ox +
// sx*a, k = oz + sz*b, every j); sample (a, j, b) goes to row at + (b*C2 + j)*nx + a.
__global__ void k_samples(SampleArgs s) {
    const int n = s.nx * s.C2 * s.nz;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int a = t % s.nx, r = t / s.nx, j = r % s.C2, b = r / s.C2;
        const int i = s.ox + s.sx * a, k = s.oz + s.sz * b;
        double A[3][3];
        grad_compact(s.ub, i, j, k, s.C1, s.C2, s.C3, s.rdx2, A);
        const double y = -0.5 * s.ly + ((double)j + 0.5) * s.dy;
        double f[NIN];
        features_of<double>(A, y, s.ly, s.yplus_scale, f);
        const size_t cn = (size_t)s.C1 * s.C2 * s.C3, c = ((size_t)k * s.C2 + j) * s.C1 + i;
        const double u[3] = {s.ub[0][c], s.ub[1][c], s.ub[2][c]};
        double tau[3][3];
        const int pidx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = 0; q < 3; ++q) tau[p][q] = s.pb[pidx[p][q] * cn + c] - u[p] * u[q];
        const double trS = A[0][0] + A[1][1] + A[2][2];
        const double trT = tau[0][0] + tau[1][1] + tau[2][2];
        double num = 0.0, den = 0.0;
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const double sd = 0.5 * (A[p][q] + A[q][p]) - (p == q ? trS / 3.0 : 0.0);
                const double td = tau[p][q] - (p == q ? trT / 3.0 : 0.0);
                num -= td * sd;
                den += 2.0 * sd * sd;
            }
        const double nut = den > 1e-30 ? fmax(num / den, 0.0) : 0.0;
        const long long row = s.at + t;
#pragma unroll
        for (int q = 0; q < NIN; ++q) s.feat[row * NIN + q] = (float)f[q];
        s.targ[row] = (float)(nut * s.rnu);
    }
}

// Plane statistics of the filtered velocities (compact FP64 arrays): block j, the same nine
// means as the context's plane statistics, fixed-order sums.
__global__ void __launch_bounds__(256) k_plane_stats_compact(const double *u0, const double *u1, const double *u2, int C1,
                                                             int C2, int C3, double *out) {
    __shared__ double red[9][256];
    const int j = blockIdx.x;
    double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int n = C1 * C3;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int i = t % C1, k = t / C1;
        const size_t c = ((size_t)k * C2 + j) * C1 + i;
        const double v1 = u0[c], v2 = u1[c], v3 = u2[c];
        a[0] += v1;
        a[1] += v2;
        a[2] += v3;
        a[3] += v1 * v1;
        a[4] += v2 * v2;
        a[5] += v3 * v3;
        a[6] += v1 * v2;
        a[7] += v1 * v3;
        a[8] += v2 * v3;
    }
    for (int q = 0; q < 9; ++q) red[q][threadIdx.x] = a[q];
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int q = 0; q < 9; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x < 9) out[9 * j + threadIdx.x] = red[threadIdx.x][0] / (double)n;
}

// ---- training kernels ---------------------------------------------------------------------

constexpr int TS = 128; // samples per tile (one per thread in the elementwise phases)

// ---- training on the tensor cores ---------------------------------------------------------
// The layers' products over a tile of TS samples are warp-level BF16 matrix multiply-accumulates
// (m16n8k16, FP32 accumulation): the forward layers Z1 = X W1^T, Z2 = H1 W2^T, the backward
// product D2 W2, and the weight gradients D1^T X and D2^T H1 summed over the tile.  The weights
// are BF16 values already (the working weights), so they enter the multiplies exactly; every
// activation or derivative a enters as a two-term BF16 expansion a = hi + lo (hi = bf16(a),
// lo = bf16(a - hi)), and a product of two such operands as hi*hi + hi*lo + lo*hi, which keeps
// about 16 significand bits (relative error near 2^-16 per product) where one BF16 product
// keeps 8.  The elementwise parts (normalisation, GELU and its derivative, the softplus output,
// the loss) stay in FP32 per sample.  All sums run in a fixed order, so the gradient is
// deterministic.

constexpr int LDX = 20;      // floats per staged input row (10 inputs padded to 16, + 4 against bank conflicts)
constexpr int LDH = NH + 4;  // floats per staged hidden row

// a two-term BF16 expansion of a pair of values, packed as the pair registers of a fragment
struct Pair2 {
    unsigned hi, lo;
};
__device__ __forceinline__ Pair2 split_pair(float a, float b) {
    const __nv_bfloat16 ah = __float2bfloat16_rn(a), bh = __float2bfloat16_rn(b);
    Pair2 r;
    __nv_bfloat162 h;
    h.x = ah;
    h.y = bh;
    r.hi = *reinterpret_cast<unsigned *>(&h);
    r.lo = pack_bf16(a - __bfloat162float(ah), b - __bfloat162float(bh));
    return r;
}

// C[16 x 8] += A[16 x 16k] B[16k x 8] for an operand A given by element reads a(row, col) (split
// into two BF16 terms) and B by b(row, col): exact BF16 (wexact, one term) or split (three
// products).  Thread lane = 4 g + t holds C[g][2t], C[g][2t+1], C[g+8][2t], C[g+8][2t+1].
template <int KSTEPS, bool B_EXACT, class FA, class FB>
__device__ __forceinline__ void mma_tile(float c[4], int lane, FA a, FB b) {
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int ks = 0; ks < KSTEPS; ++ks) {
        const int k0 = 16 * ks;
        const Pair2 a0 = split_pair(a(g, k0 + 2 * t), a(g, k0 + 2 * t + 1));
        const Pair2 a1 = split_pair(a(g + 8, k0 + 2 * t), a(g + 8, k0 + 2 * t + 1));
        const Pair2 a2 = split_pair(a(g, k0 + 2 * t + 8), a(g, k0 + 2 * t + 9));
        const Pair2 a3 = split_pair(a(g + 8, k0 + 2 * t + 8), a(g + 8, k0 + 2 * t + 9));
        const unsigned ahi[4] = {a0.hi, a1.hi, a2.hi, a3.hi}, alo[4] = {a0.lo, a1.lo, a2.lo, a3.lo};
        if (B_EXACT) {
            const unsigned b0 = pack_bf16(b(k0 + 2 * t, g), b(k0 + 2 * t + 1, g));
            const unsigned b1 = pack_bf16(b(k0 + 2 * t + 8, g), b(k0 + 2 * t + 9, g));
            mma_bf16(c, ahi, b0, b1);
            mma_bf16(c, alo, b0, b1);
        } else {
            const Pair2 b0 = split_pair(b(k0 + 2 * t, g), b(k0 + 2 * t + 1, g));
            const Pair2 b1 = split_pair(b(k0 + 2 * t + 8, g), b(k0 + 2 * t + 9, g));
            mma_bf16(c, ahi, b0.hi, b1.hi);
            mma_bf16(c, ahi, b0.lo, b1.lo);
            mma_bf16(c, alo, b0.hi, b1.hi);
        }
    }
}

// Gradient of the mean squared error over samples [first, first + count) of the batch map
// (sample index = (first + q) * stride + offset), into block partials part[block][NPARAM + 1]
// (the last entry: the block's sum of squared errors).  scale = 2 / (samples of the batch).
__global__ void __launch_bounds__(TS, 2) k_mlp_grad(const float *__restrict__ feat, const float *__restrict__ targ,
                                                    long long first, long long count, long long stride, long long offset,
                                                    const Net *__restrict__ net, float scale, float *part) {
    extern __shared__ float smem[];
    float *w = smem;                  // NPARAM (BF16-exact working weights)
    float *acc = w + NPARAM;          // NPARAM + 1 (this block's sums)
    float *X = acc + NPARAM + 1;      // TS x LDX: normalised inputs, zero past NIN
    float *Z1 = X + TS * LDX;         // TS x LDH: z1, then dL/dz1
    float *H1 = Z1 + TS * LDH;        // TS x LDH: gelu(z1)
    float *Z2 = H1 + TS * LDH;        // TS x LDH: z2, then dL/dz2
    float *H2 = Z2 + TS * LDH;        // TS x LDH: gelu(z2)
    float *D3 = H2 + TS * LDH;        // TS: dL/dz3
    float *R2 = D3 + TS;              // TS: squared errors
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5, g = lane >> 2, tq = lane & 3;
    for (int q = t; q < NPARAM; q += TS) {
        w[q] = net->w[q];
        acc[q] = 0.f;
    }
    if (t == 0) acc[NPARAM] = 0.f;
    __shared__ float mu[NIN], rsd[NIN];
    if (t < NIN) {
        mu[t] = net->mu[t];
        rsd[t] = net->rsd[t];
    }
    __syncthreads();
    const long long ntiles = (count + TS - 1) / TS;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long q = tile * TS + t;
        const bool live = q < count;
        const long long smp = live ? (first + q) * stride + offset : 0;
        // inputs (a sample past the end enters as zeros; its error and derivatives are zero)
#pragma unroll
        for (int i = 0; i < 16; ++i) X[t * LDX + i] = (live && i < NIN) ? (feat[smp * NIN + i] - mu[i]) * rsd[i] : 0.f;
        __syncthreads();
        // Z1 = X W1^T + b1: warp w takes sample rows 32w .. 32w+31 (two m-tiles), all four n-tiles
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int s0 = 32 * wid + 16 * mt, n0 = 8 * nt;
                float c[4] = {0.f, 0.f, 0.f, 0.f};
                mma_tile<1, true>(c, lane, [&](int r, int k) { return X[(s0 + r) * LDX + k]; },
                                  [&](int k, int n) { return k < NIN ? w[O_W1 + (n0 + n) * NIN + k] : 0.f; });
                const int n = n0 + 2 * tq;
                Z1[(s0 + g) * LDH + n] = c[0] + w[O_B1 + n];
                Z1[(s0 + g) * LDH + n + 1] = c[1] + w[O_B1 + n + 1];
                Z1[(s0 + g + 8) * LDH + n] = c[2] + w[O_B1 + n];
                Z1[(s0 + g + 8) * LDH + n + 1] = c[3] + w[O_B1 + n + 1];
            }
        __syncthreads();
        for (int k = 0; k < NH; ++k) H1[t * LDH + k] = gelu(Z1[t * LDH + k]);
        __syncthreads();
        // Z2 = H1 W2^T + b2
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int s0 = 32 * wid + 16 * mt, n0 = 8 * nt;
                float c[4] = {0.f, 0.f, 0.f, 0.f};
                mma_tile<2, true>(c, lane, [&](int r, int k) { return H1[(s0 + r) * LDH + k]; },
                                  [&](int k, int n) { return w[O_W2 + (n0 + n) * NH + k]; });
                const int n = n0 + 2 * tq;
                Z2[(s0 + g) * LDH + n] = c[0] + w[O_B2 + n];
                Z2[(s0 + g) * LDH + n + 1] = c[1] + w[O_B2 + n + 1];
                Z2[(s0 + g + 8) * LDH + n] = c[2] + w[O_B2 + n];
                Z2[(s0 + g + 8) * LDH + n + 1] = c[3] + w[O_B2 + n + 1];
            }
        __syncthreads();
        // per sample: the second activation, the output, the error and dL/dz3, then dL/dz2
        {
            float z3 = w[O_B3];
            for (int k = 0; k < NH; ++k) {
                const float h2 = gelu(Z2[t * LDH + k]);
                H2[t * LDH + k] = h2;
                z3 += w[O_W3 + k] * h2;
            }
            float d3 = 0.f, r2 = 0.f;
            if (live) {
                const float y = softplus(z3), r = y - targ[smp];
                r2 = r * r;
                d3 = scale * r * sigmoid(z3);
            }
            D3[t] = d3;
            R2[t] = r2;
            for (int k = 0; k < NH; ++k) Z2[t * LDH + k] = d3 * w[O_W3 + k] * gelu_grad(Z2[t * LDH + k]);
        }
        __syncthreads();
        // dL/dz1 = (D2 W2) * gelu'(z1), in place of z1
        {
            float d1[2][4][4];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const int s0 = 32 * wid + 16 * mt, n0 = 8 * nt;
                    float *c = d1[mt][nt];
                    c[0] = c[1] = c[2] = c[3] = 0.f;
                    mma_tile<2, true>(c, lane, [&](int r, int k) { return Z2[(s0 + r) * LDH + k]; },
                                      [&](int k, int n) { return w[O_W2 + k * NH + n0 + n]; });
                }
            // every warp reads only its own sample rows of Z1: no barrier between
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const int s0 = 32 * wid + 16 * mt, n = 8 * nt + 2 * tq;
                    const float *c = d1[mt][nt];
                    float *z = &Z1[(s0 + g) * LDH + n];
                    z[0] = c[0] * gelu_grad(z[0]);
                    z[1] = c[1] * gelu_grad(z[1]);
                    z = &Z1[(s0 + g + 8) * LDH + n];
                    z[0] = c[2] * gelu_grad(z[0]);
                    z[1] = c[3] * gelu_grad(z[1]);
                }
        }
        __syncthreads();
        // weight gradients over the tile: gW2 = D2^T H1 (warp w: unit rows 16 (w & 1) .. +15,
        // n-tiles 2 (w >> 1), +1), gW1 = D1^T X (warp w: unit rows 16 (w & 1), input n-tile w >> 1)
        {
            const int k0 = 16 * (wid & 1);
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int n0 = 8 * (2 * (wid >> 1) + j);
                float c[4] = {0.f, 0.f, 0.f, 0.f};
                mma_tile<TS / 16, false>(c, lane, [&](int r, int s) { return Z2[s * LDH + k0 + r]; },
                                         [&](int s, int n) { return H1[s * LDH + n0 + n]; });
                const int n = n0 + 2 * tq;
                acc[O_W2 + (k0 + g) * NH + n] += c[0];
                acc[O_W2 + (k0 + g) * NH + n + 1] += c[1];
                acc[O_W2 + (k0 + g + 8) * NH + n] += c[2];
                acc[O_W2 + (k0 + g + 8) * NH + n + 1] += c[3];
            }
            const int i0 = 8 * (wid >> 1);
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            mma_tile<TS / 16, false>(c, lane, [&](int r, int s) { return Z1[s * LDH + k0 + r]; },
                                     [&](int s, int n) { return X[s * LDX + i0 + n]; });
            const int i = i0 + 2 * tq;
            if (i < NIN) {
                acc[O_W1 + (k0 + g) * NIN + i] += c[0];
                acc[O_W1 + (k0 + g + 8) * NIN + i] += c[2];
            }
            if (i + 1 < NIN) {
                acc[O_W1 + (k0 + g) * NIN + i + 1] += c[1];
                acc[O_W1 + (k0 + g + 8) * NIN + i + 1] += c[3];
            }
        }
        // the bias gradients, the last layer's and the squared errors: sums over the tile in order
        for (int p = t; p <= NPARAM; p += TS) {
            float gsum = 0.f;
            if (p >= O_B1 && p < O_W2) {
                const int k = p - O_B1;
                for (int s2 = 0; s2 < TS; ++s2) gsum += Z1[s2 * LDH + k];
            } else if (p >= O_B2 && p < O_W3) {
                const int k = p - O_B2;
                for (int s2 = 0; s2 < TS; ++s2) gsum += Z2[s2 * LDH + k];
            } else if (p >= O_W3 && p < O_B3) {
                const int k = p - O_W3;
                for (int s2 = 0; s2 < TS; ++s2) gsum += D3[s2] * H2[s2 * LDH + k];
            } else if (p == O_B3) {
                for (int s2 = 0; s2 < TS; ++s2) gsum += D3[s2];
            } else if (p == NPARAM) {
                for (int s2 = 0; s2 < TS; ++s2) gsum += R2[s2];
            } else {
                continue; // W1 and W2: taken by the multiplies above
            }
            acc[p] += gsum;
        }
        __syncthreads();
    }
    for (int p = t; p <= NPARAM; p += TS) part[(size_t)blockIdx.x * (NPARAM + 1) + p] = acc[p];
}

// Sum of the block partials in block order (deterministic): out[p] for p <= NPARAM.
__global__ void k_mlp_reduce(const float *part, int nblocks, float *out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > NPARAM) return;
    float s = 0.f;
    for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * (NPARAM + 1) + p];
    out[p] = s;
}

struct Adam {
    float lr, beta1, beta2, eps;
};

// One Adam step on the FP32 master weights; the network's working weights are their BF16
// roundings.  step: 1-based count for the bias corrections.
__global__ void k_adam(float *master, float *m, float *v, const float *grad, Net *net, Adam a, int step) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    const float g = grad[p];
    const float mm = a.beta1 * m[p] + (1.f - a.beta1) * g;
    const float vv = a.beta2 * v[p] + (1.f - a.beta2) * g * g;
    m[p] = mm;
    v[p] = vv;
    const float mh = mm / (1.f - powf(a.beta1, (float)step));
    const float vh = vv / (1.f - powf(a.beta2, (float)step));
    const float x = master[p] - a.lr * mh / (sqrtf(vh) + a.eps);
    master[p] = x;
    net->w[p] = __bfloat162float(__float2bfloat16_rn(x));
}

__global__ void k_add_loss(const float *grad, float *acc, float scale) {
    if (threadIdx.x == 0) *acc += grad[NPARAM] * scale;
}

__global__ void k_set_working(const float *master, Net *net) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < NPARAM) net->w[p] = __bfloat162float(__float2bfloat16_rn(master[p]));
}

// nu_t / nu of samples [0, n) (prediction for tests and evaluation)
__global__ void k_mlp_predict(const float *feat, long long n, const Net *net, float *out) {
    __shared__ float w[NPARAM];
    __shared__ float mu[NIN], rsd[NIN];
    for (int q = threadIdx.x; q < NPARAM; q += blockDim.x) w[q] = net->w[q];
    if (threadIdx.x < NIN) {
        mu[threadIdx.x] = net->mu[threadIdx.x];
        rsd[threadIdx.x] = net->rsd[threadIdx.x];
    }
    __syncthreads();
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
        float xn[NIN];
#pragma unroll
        for (int i = 0; i < NIN; ++i) xn[i] = (feat[s * NIN + i] - mu[i]) * rsd[i];
        out[s] = mlp_forward(w, xn);
    }
}

// per-feature sums (sum, sum of squares) of samples [0, n), for the input normalisation
__global__ void k_feature_moments(const float *feat, long long n, double *mom) {
    __shared__ double red[2 * NIN][8];
    double s[NIN], s2[NIN];
#pragma unroll
    for (int i = 0; i < NIN; ++i) s[i] = s2[i] = 0.0;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
#pragma unroll
        for (int i = 0; i < NIN; ++i) {
            const double x = feat[q * NIN + i];
            s[i] += x;
            s2[i] += x * x;
        }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NIN; ++i) {
        for (int o = 16; o > 0; o >>= 1) {
            s[i] += __shfl_xor_sync(0xffffffffu, s[i], o);
            s2[i] += __shfl_xor_sync(0xffffffffu, s2[i], o);
        }
        if (lane == 0) {
            red[i][wid] = s[i];
            red[NIN + i][wid] = s2[i];
        }
    }
    __syncthreads();
    if (threadIdx.x < 2 * NIN) {
        double z = 0.0;
        for (int v = 0; v < (int)(blockDim.x >> 5); ++v) z += red[threadIdx.x][v];
        atomicAdd(&mom[threadIdx.x], z);
    }
}

// ---- inference in a context ---------------------------------------------------------------

// nu_t of every interior cell of level lvl, and of the ghost cells of periodic x and z (their
// images); solid cells 0.  Reads interior cells and flags only.
// The network staged in shared memory (coalesced loads; the fragments then read it with
// per-lane addresses, which shared memory serves without serialising).
struct NetSmem {
    float w[NPARAM];
    float mu[NIN], rsd[NIN];
};
__device__ __forceinline__ void stage_net(NetSmem &sm, const Net *__restrict__ net) {
    for (int q = threadIdx.x; q < NPARAM; q += blockDim.x) sm.w[q] = net->w[q];
    if (threadIdx.x < NIN) {
        sm.mu[threadIdx.x] = net->mu[threadIdx.x];
        sm.rsd[threadIdx.x] = net->rsd[threadIdx.x];
    }
    __syncthreads();
}

// Run constants of the inference in FP32, computed once on the host (no FP64 per cell).
struct NutConst {
    float rdx2[3];   // 1 / (2 dx_d)
    float ly, dy;    // channel height, cell height
    float vis;       // nu
    float yplus;     // u_tau / nu
};

template <class T> __global__ void __launch_bounds__(128)
    k_nut(const __grid_constant__ DevState<T> S, int lvl, const Net *__restrict__ netd, const NutConst K) {
    __shared__ __align__(16) __nv_bfloat16 X[4][32 * 16];
    __shared__ NetSmem net;
    stage_net(net, netd);
    const float *w = net.w;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const TcWeights B = tc_weights(w, lane);
    const Geom g = S.g;
    const Level<T> L = S.lv[lvl];
    const int nx = g.C1 + 2, nz = g.C3 + 2;
    const int n = nx * g.C2 * nz;
    const int nwarps = gridDim.x * 4;
    // warp-uniform loop: every lane of a warp takes part in each multiply
    for (int base = (blockIdx.x * 4 + wid) * 32; base < n; base += nwarps * 32) {
        const int t = base + lane;
        const bool live = t < n;
        const int tt = live ? t : n - 1;
        const int ig = tt % nx, r = tt / nx, j = r % g.C2 + 1, kg = r / g.C2;
        // the interior cell whose value this position takes (periodic image, else nearest)
        const int i = ig == 0 ? (S.k.periodic_x ? g.C1 : 1) : (ig == g.C1 + 1 ? (S.k.periodic_x ? 1 : g.C1) : ig);
        const int k = kg == 0 ? (S.k.periodic_z ? g.C3 : 1) : (kg == g.C3 + 1 ? (S.k.periodic_z ? 1 : g.C3) : kg);
        const int64_t ncell = g.ncell();
        const int64_t c = ARK_CK(g.cell(i, j, k), ncell);
        const bool fluid = (S.flags[c] & FL_EQ0) != 0;
        float f[NIN];
        {
            float A[3][3];
            // neighbours in x and z by index (periodic image or the zero-gradient copy), so the
            // level's ghost cells are not needed: this runs beside the step's ghost fill
            const int im = i > 1 ? i - 1 : (S.k.periodic_x ? g.C1 : 1), ip = i < g.C1 ? i + 1 : (S.k.periodic_x ? 1 : g.C1);
            const int km = k > 1 ? k - 1 : (S.k.periodic_z ? g.C3 : 1), kp = k < g.C3 ? k + 1 : (S.k.periodic_z ? 1 : g.C3);
            int64_t nb[6] = {g.cell(im, j, k), g.cell(ip, j, k), c - g.cs1, c + g.cs1, g.cell(i, j, km), g.cell(i, j, kp)};
#pragma unroll
            for (int q = 0; q < 6; ++q) nb[q] = ARK_CK(nb[q], ncell);
            const T *u[3] = {L.u1, L.u2, L.u3};
            bool solid[6];
#pragma unroll
            for (int q = 0; q < 6; ++q) solid[q] = (S.flags[nb[q]] & FL_GT) != 0;
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                const float uc = (float)u[m][c];
                float v[6];
#pragma unroll
                for (int q = 0; q < 6; ++q) v[q] = solid[q] ? -uc : (float)u[m][nb[q]];
                A[m][0] = (v[1] - v[0]) * K.rdx2[0];
                A[m][1] = (v[3] - v[2]) * K.rdx2[1];
                A[m][2] = (v[5] - v[4]) * K.rdx2[2];
            }
            const float y = -0.5f * K.ly + ((float)j - 0.5f) * K.dy;
            features_of<float>(A, y, K.ly, K.yplus, f);
#pragma unroll
            for (int q = 0; q < NIN; ++q) f[q] = (f[q] - net.mu[q]) * net.rsd[q];
        }
        const float y_nu = tc_warp(w, B, X[wid], f, lane);
        if (live) S.nut[ARK_CK(g.cell(ig, j, kg), ncell)] = fluid ? (T)(y_nu * K.vis) : (T)0;
    }
}

// nu_t / nu of dataset rows through the tensor-core inference of the step (tests)
__global__ void __launch_bounds__(128) k_mlp_predict_tc(const float *feat, long long n, const Net *__restrict__ netd,
                                                        float *out) {
    __shared__ __align__(16) __nv_bfloat16 X[4][32 * 16];
    __shared__ NetSmem net;
    stage_net(net, netd);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const TcWeights B = tc_weights(net.w, lane);
    const long long nwarps = (long long)gridDim.x * 4;
    for (long long base = ((long long)blockIdx.x * 4 + wid) * 32; base < n; base += nwarps * 32) {
        const long long s = base + lane < n ? base + lane : n - 1;
        float x[NIN];
#pragma unroll
        for (int i = 0; i < NIN; ++i) x[i] = (feat[s * NIN + i] - net.mu[i]) * net.rsd[i];
        const float y = tc_warp(net.w, B, X[wid], x, lane);
        if (base + lane < n) out[base + lane] = y;
    }
}

int grid_for(long long n, int threads = 256) {
    const long long b = (n + threads - 1) / threads;
    return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

} // namespace cl

template <class T> void closure_nut(const DevState<T> &S, int lvl, const void *net, float yplus_scale, cudaStream_t st) {
    const long long n = (long long)(S.g.C1 + 2) * S.g.C2 * (S.g.C3 + 2);
    cl::NutConst K;
    for (int d = 0; d < 3; ++d) K.rdx2[d] = (float)(0.5 / S.k.dx[d]);
    K.ly = (float)(S.k.dx[1] * S.g.C2);
    K.dy = (float)S.k.dx[1];
    K.vis = (float)S.k.vis;
    K.yplus = yplus_scale;
    cl::k_nut<T><<<cl::grid_for(n, 128), 128, 0, st>>>(S, lvl, (const cl::Net *)net, K);
}
template void closure_nut<float>(const DevState<float> &, int, const void *, float, cudaStream_t);
template void closure_nut<double>(const DevState<double> &, int, const void *, float, cudaStream_t);

template <class T> void closure_gather(const DevState<T> &S, int lvl, double *u0, double *u1, double *u2, cudaStream_t st) {
    cl::k_gather<T><<<cl::grid_for((long long)S.g.C1 * S.g.C2 * S.g.C3), 256, 0, st>>>(S, lvl, u0, u1, u2);
}
template void closure_gather<float>(const DevState<float> &, int, double *, double *, double *, cudaStream_t);
template void closure_gather<double>(const DevState<double> &, int, double *, double *, double *, cudaStream_t);

} // namespace ark

// ---- C ABI --------------------------------------------------------------------------------

using namespace ark;

namespace {
thread_local std::string g_cl_error;
int cfail(int code, const std::string &m) {
    g_cl_error = m;
    return code;
}
#define CL_CUDA(x)                                                                                    \
    do {                                                                                              \
        cudaError_t e_ = (x);                                                                         \
        if (e_ != cudaSuccess) return cfail(ARK_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)
} // namespace

struct ark_closure_data {
    int device = 0;
    cudaStream_t st = nullptr;
    long long cap = 0, n = 0;
    float *feat = nullptr, *targ = nullptr;
    // FP64 filter scratch for the grid last sampled: 3 velocities, 6 products, 9 filtered, 1 temp
    double *scratch = nullptr;
    long long scratch_cells = 0;
    int last[3] = {0, 0, 0}; // grid of the last filtered field (in the scratch)
};

struct ark_mlp {
    int device = 0;
    cudaStream_t st = nullptr;
    cl::Net *net = nullptr; // device: working weights and normalisation
    float *master = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *part = nullptr;
    int nblocks = 0;
    int step = 0;
};

extern "C" {

const char *ark_closure_last_error(void) { return g_cl_error.c_str(); }

ark_closure_data *ark_closure_data_create(long long capacity, int device, int *status) {
    int dummy;
    if (!status) status = &dummy;
    if (capacity < 1) {
        *status = cfail(ARK_ERR_PARAM, "capacity < 1");
        return nullptr;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        *status = cfail(ARK_ERR_CUDA, "cudaSetDevice failed");
        return nullptr;
    }
    ark_closure_data *d = new ark_closure_data();
    d->device = device;
    d->cap = capacity;
    if (cudaStreamCreateWithFlags(&d->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&d->feat, sizeof(float) * cl::NIN * capacity) != cudaSuccess ||
        cudaMalloc(&d->targ, sizeof(float) * capacity) != cudaSuccess) {
        *status = cfail(ARK_ERR_NOMEM, "dataset allocation failed");
        ark_closure_data_destroy(d);
        return nullptr;
    }
    *status = ARK_OK;
    return d;
}

int ark_closure_data_destroy(ark_closure_data *d) {
    if (!d) return ARK_OK;
    if (d->st) cudaStreamSynchronize(d->st);
    cudaFree(d->feat);
    cudaFree(d->targ);
    cudaFree(d->scratch);
    if (d->st) cudaStreamDestroy(d->st);
    delete d;
    return ARK_OK;
}

long long ark_closure_data_size(const ark_closure_data *d) { return d ? d->n : -1; }

int ark_closure_data_clear(ark_closure_data *d) {
    if (!d) return cfail(ARK_ERR_PARAM, "dataset is NULL");
    d->n = 0;
    return ARK_OK;
}

int ark_closure_data_get(ark_closure_data *d, long long first, long long count, float *features, float *targets) {
    if (!d || first < 0 || count < 0 || first + count > d->n) return cfail(ARK_ERR_PARAM, "bad range");
    CL_CUDA(cudaStreamSynchronize(d->st));
    if (features) CL_CUDA(cudaMemcpy(features, d->feat + first * cl::NIN, sizeof(float) * cl::NIN * count, cudaMemcpyDeviceToHost));
    if (targets) CL_CUDA(cudaMemcpy(targets, d->targ + first, sizeof(float) * count, cudaMemcpyDeviceToHost));
    return ARK_OK;
}

int ark_closure_data_filtered_stats(ark_closure_data *d, double *out) {
    if (!d || !out) return cfail(ARK_ERR_PARAM, "NULL argument");
    const int C1 = d->last[0], C2 = d->last[1], C3 = d->last[2];
    if (C1 < 1) return cfail(ARK_ERR_STATE, "no field has been sampled");
    const long long cells = (long long)C1 * C2 * C3;
    const double *ub = d->scratch + 9 * cells;
    double *o = nullptr;
    CL_CUDA(cudaMalloc(&o, sizeof(double) * 9 * C2));
    cl::k_plane_stats_compact<<<C2, 256, 0, d->st>>>(ub, ub + cells, ub + 2 * cells, C1, C2, C3, o);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
    if (e == cudaSuccess) e = cudaMemcpy(out, o, sizeof(double) * 9 * C2, cudaMemcpyDeviceToHost);
    cudaFree(o);
    if (e != cudaSuccess) return cfail(ARK_ERR_CUDA, std::string("filtered statistics: ") + cudaGetErrorString(e));
    return ARK_OK;
}

int ark_closure_data_append(ark_closure_data *d, long long count, const float *features, const float *targets) {
    if (!d || count < 0 || !features || !targets) return cfail(ARK_ERR_PARAM, "bad arguments");
    if (d->n + count > d->cap) return cfail(ARK_ERR_PARAM, "dataset full");
    CL_CUDA(cudaStreamSynchronize(d->st));
    CL_CUDA(cudaMemcpy(d->feat + d->n * cl::NIN, features, sizeof(float) * cl::NIN * count, cudaMemcpyHostToDevice));
    CL_CUDA(cudaMemcpy(d->targ + d->n, targets, sizeof(float) * count, cudaMemcpyHostToDevice));
    d->n += count;
    return ARK_OK;
}

} // extern "C"

// Used by ark_api.cu (needs the context's internals): the gather buffers for a grid's velocities
// (3 compact interior arrays), then the samples of what was gathered into them on ctx_st.
namespace ark {
int closure_scratch(ark_closure_data *d, long long cells, double **u) {
    if (d->scratch_cells != cells) {
        cudaFree(d->scratch);
        d->scratch = nullptr;
        d->scratch_cells = 0;
        if (cudaMalloc(&d->scratch, sizeof(double) * 19 * (size_t)cells) != cudaSuccess)
            return cfail(ARK_ERR_NOMEM, "filter scratch allocation failed");
        d->scratch_cells = cells;
    }
    *u = d->scratch;
    return ARK_OK;
}

long long closure_count(int C1, int C2, int C3, int sx, int sz, int ox, int oz) {
    if (sx < 1 || sz < 1 || ox < 0 || oz < 0 || ox >= sx || oz >= sz || ox >= C1 || oz >= C3) return -1;
    return (long long)((C1 - ox + sx - 1) / sx) * C2 * ((C3 - oz + sz - 1) / sz);
}

long long closure_room(const ark_closure_data *d) { return d->cap - d->n; }

int closure_sample(ark_closure_data *d, int C1, int C2, int C3, double lx, double ly, double lz, double vis, int sx,
                   int sz, int ox, int oz, double u_tau, cudaStream_t ctx_st) {
    const int nx = (C1 - ox + sx - 1) / sx, nz = (C3 - oz + sz - 1) / sz;
    const long long count = (long long)nx * C2 * nz;
    const long long cells = (long long)C1 * C2 * C3;
    double *u = d->scratch;           // 3 gathered velocities
    double *p = u + 3 * cells;        // 6 products
    double *ub = p + 6 * cells;       // 3 filtered velocities
    double *pb = ub + 3 * cells;      // 6 filtered products
    double *tmp = pb + 6 * cells;     // 1
    CL_CUDA(cudaGetLastError());
    CL_CUDA(cudaStreamSynchronize(ctx_st));
    const int gb = cl::grid_for(cells);
    cl::k_products<<<gb, 256, 0, d->st>>>(u, u + cells, u + 2 * cells, p, (int)cells);
    for (int f = 0; f < 9; ++f) {
        const double *src = f < 3 ? u + f * cells : p + (f - 3) * cells;
        double *dst = f < 3 ? ub + f * cells : pb + (f - 3) * cells;
        const double sign = f < 3 ? -1.0 : 1.0;
        cl::k_filter_pass<<<gb, 256, 0, d->st>>>(src, dst, C1, C2, C3, 0, sign);
        cl::k_filter_pass<<<gb, 256, 0, d->st>>>(dst, tmp, C1, C2, C3, 1, sign);
        cl::k_filter_pass<<<gb, 256, 0, d->st>>>(tmp, dst, C1, C2, C3, 2, sign);
    }
    cl::SampleArgs s;
    for (int m = 0; m < 3; ++m) s.ub[m] = ub + m * cells;
    s.pb = pb;
    s.feat = d->feat;
    s.targ = d->targ;
    s.at = d->n;
    s.C1 = C1;
    s.C2 = C2;
    s.C3 = C3;
    s.sx = sx;
    s.sz = sz;
    s.ox = ox;
    s.oz = oz;
    s.nx = nx;
    s.nz = nz;
    const double dx[3] = {lx / C1, ly / C2, lz / C3};
    for (int q = 0; q < 3; ++q) s.rdx2[q] = 0.5 / dx[q];
    s.ly = ly;
    s.dy = dx[1];
    s.yplus_scale = u_tau / vis;
    s.rnu = 1.0 / vis;
    cl::k_samples<<<cl::grid_for(count), 256, 0, d->st>>>(s);
    CL_CUDA(cudaGetLastError());
    CL_CUDA(cudaStreamSynchronize(d->st));
    d->n += count;
    d->last[0] = C1;
    d->last[1] = C2;
    d->last[2] = C3;
    return ARK_OK;
}
} // namespace ark

extern "C" {

ark_mlp *ark_mlp_create(unsigned long long seed, int device, int *status) {
    int dummy;
    if (!status) status = &dummy;
    if (cudaSetDevice(device) != cudaSuccess) {
        *status = cfail(ARK_ERR_CUDA, "cudaSetDevice failed");
        return nullptr;
    }
    ark_mlp *M = new ark_mlp();
    M->device = device;
    M->nblocks = 152 * 4;
    bool ok = cudaStreamCreateWithFlags(&M->st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&M->net, sizeof(cl::Net)) == cudaSuccess &&
              cudaMalloc(&M->master, sizeof(float) * cl::NPARAM) == cudaSuccess &&
              cudaMalloc(&M->m, sizeof(float) * cl::NPARAM) == cudaSuccess &&
              cudaMalloc(&M->v, sizeof(float) * cl::NPARAM) == cudaSuccess &&
              cudaMalloc(&M->grad, sizeof(float) * (cl::NPARAM + 1)) == cudaSuccess &&
              cudaMalloc(&M->part, sizeof(float) * (cl::NPARAM + 1) * M->nblocks) == cudaSuccess;
    if (!ok) {
        *status = cfail(ARK_ERR_NOMEM, "network allocation failed");
        ark_mlp_destroy(M);
        return nullptr;
    }
    // initial weights: uniform(-1, 1) * sqrt(3 / fan_in) (splitmix64), zero biases; identity
    // normalisation
    std::vector<float> w(cl::NPARAM, 0.f);
    unsigned long long x = seed;
    auto next = [&]() {
        unsigned long long z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int q = 0; q < cl::NH * cl::NIN; ++q) w[cl::O_W1 + q] = (float)((2 * next() - 1) * std::sqrt(3.0 / cl::NIN));
    for (int q = 0; q < cl::NH * cl::NH; ++q) w[cl::O_W2 + q] = (float)((2 * next() - 1) * std::sqrt(3.0 / cl::NH));
    for (int q = 0; q < cl::NH; ++q) w[cl::O_W3 + q] = (float)((2 * next() - 1) * std::sqrt(3.0 / cl::NH));
    std::vector<double> mu(cl::NIN, 0.0), sd(cl::NIN, 1.0);
    std::vector<double> wd(w.begin(), w.end());
    *status = ark_mlp_set(M, wd.data(), mu.data(), sd.data());
    if (*status) {
        ark_mlp_destroy(M);
        return nullptr;
    }
    return M;
}

int ark_mlp_destroy(ark_mlp *M) {
    if (!M) return ARK_OK;
    if (M->st) cudaStreamSynchronize(M->st);
    cudaFree(M->net);
    cudaFree(M->master);
    cudaFree(M->m);
    cudaFree(M->v);
    cudaFree(M->grad);
    cudaFree(M->part);
    if (M->st) cudaStreamDestroy(M->st);
    delete M;
    return ARK_OK;
}

int ark_mlp_set(ark_mlp *M, const double *params, const double *mu, const double *sd) {
    if (!M || !params || !mu || !sd) return cfail(ARK_ERR_PARAM, "NULL argument");
    std::vector<float> w(cl::NPARAM);
    for (int q = 0; q < cl::NPARAM; ++q) w[q] = (float)params[q];
    cl::Net h;
    std::memset(&h, 0, sizeof h);
    for (int q = 0; q < cl::NIN; ++q) {
        if (!(sd[q] > 0)) return cfail(ARK_ERR_PARAM, "sd must be > 0");
        h.mu[q] = (float)mu[q];
        h.rsd[q] = (float)(1.0 / sd[q]);
    }
    CL_CUDA(cudaStreamSynchronize(M->st));
    CL_CUDA(cudaMemcpy(M->master, w.data(), sizeof(float) * cl::NPARAM, cudaMemcpyHostToDevice));
    CL_CUDA(cudaMemset(M->m, 0, sizeof(float) * cl::NPARAM));
    CL_CUDA(cudaMemset(M->v, 0, sizeof(float) * cl::NPARAM));
    CL_CUDA(cudaMemcpy(M->net, &h, sizeof h, cudaMemcpyHostToDevice));
    cl::k_set_working<<<(cl::NPARAM + 255) / 256, 256, 0, M->st>>>(M->master, M->net);
    CL_CUDA(cudaGetLastError());
    CL_CUDA(cudaStreamSynchronize(M->st));
    M->step = 0;
    return ARK_OK;
}

int ark_mlp_get(ark_mlp *M, double *params, double *mu, double *sd) {
    if (!M) return cfail(ARK_ERR_PARAM, "network is NULL");
    CL_CUDA(cudaStreamSynchronize(M->st));
    if (params) {
        std::vector<float> w(cl::NPARAM);
        CL_CUDA(cudaMemcpy(w.data(), M->master, sizeof(float) * cl::NPARAM, cudaMemcpyDeviceToHost));
        for (int q = 0; q < cl::NPARAM; ++q) params[q] = w[q];
    }
    if (mu || sd) {
        cl::Net h;
        CL_CUDA(cudaMemcpy(&h, M->net, sizeof h, cudaMemcpyDeviceToHost));
        for (int q = 0; q < cl::NIN; ++q) {
            if (mu) mu[q] = h.mu[q];
            if (sd) sd[q] = 1.0 / (double)h.rsd[q];
        }
    }
    return ARK_OK;
}

int ark_mlp_fit_normalization(ark_mlp *M, ark_closure_data *d) {
    if (!M || !d || d->n < 2) return cfail(ARK_ERR_PARAM, "need a network and at least two samples");
    double *mom = nullptr;
    CL_CUDA(cudaMalloc(&mom, sizeof(double) * 2 * cl::NIN));
    CL_CUDA(cudaMemsetAsync(mom, 0, sizeof(double) * 2 * cl::NIN, d->st));
    cl::k_feature_moments<<<cl::grid_for(d->n), 256, 0, d->st>>>(d->feat, d->n, mom);
    double h[2 * cl::NIN];
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(d->st);
    if (e == cudaSuccess) e = cudaMemcpy(h, mom, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(mom);
    if (e != cudaSuccess) return cfail(ARK_ERR_CUDA, std::string("moments: ") + cudaGetErrorString(e));
    cl::Net net;
    CL_CUDA(cudaStreamSynchronize(M->st));
    CL_CUDA(cudaMemcpy(&net, M->net, sizeof net, cudaMemcpyDeviceToHost));
    for (int q = 0; q < cl::NIN; ++q) {
        const double mean = h[q] / d->n;
        const double var = std::max(h[cl::NIN + q] / d->n - mean * mean, 0.0);
        const double sd = std::sqrt(var);
        net.mu[q] = (float)mean;
        net.rsd[q] = (float)(sd > 1e-20 ? 1.0 / sd : 1.0);
    }
    CL_CUDA(cudaMemcpy(M->net, &net, sizeof net, cudaMemcpyHostToDevice));
    return ARK_OK;
}

} // extern "C"

namespace {

size_t grad_smem() {
    return sizeof(float) * (2 * cl::NPARAM + 1 + cl::TS * cl::LDX + 4 * cl::TS * cl::LDH + 2 * cl::TS);
}

// gradient (and summed squared error) of samples (first + q) * stride + offset, q < count,
// with scale 2 / count, into M->grad on M->st
void launch_grad(ark_mlp *M, const ark_closure_data *d, long long first, long long count, long long stride,
                 long long offset) {
    const long long tiles = (count + cl::TS - 1) / cl::TS;
    const int nb = (int)std::min<long long>(tiles, M->nblocks);
    cl::k_mlp_grad<<<nb, cl::TS, grad_smem(), M->st>>>(d->feat, d->targ, first, count, stride, offset, M->net,
                                                       (float)(2.0 / (double)count), M->part);
    cl::k_mlp_reduce<<<(cl::NPARAM + 1 + 255) / 256, 256, 0, M->st>>>(M->part, nb, M->grad);
}

int prepare_grad() {
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        err = cudaFuncSetAttribute(cl::k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)grad_smem());
    });
    return err == cudaSuccess ? ARK_OK : cfail(ARK_ERR_CUDA, "k_mlp_grad shared memory attribute");
}

} // namespace

extern "C" {

int ark_mlp_gradient(ark_mlp *M, ark_closure_data *d, long long first, long long count, double *grad, double *loss) {
    if (!M || !d || first < 0 || count < 1 || first + count > d->n) return cfail(ARK_ERR_PARAM, "bad range");
    if (int rc = prepare_grad()) return rc;
    CL_CUDA(cudaStreamSynchronize(d->st));
    launch_grad(M, d, first, count, 1, 0);
    CL_CUDA(cudaGetLastError());
    std::vector<float> h(cl::NPARAM + 1);
    CL_CUDA(cudaStreamSynchronize(M->st));
    CL_CUDA(cudaMemcpy(h.data(), M->grad, sizeof(float) * (cl::NPARAM + 1), cudaMemcpyDeviceToHost));
    if (grad)
        for (int q = 0; q < cl::NPARAM; ++q) grad[q] = h[q];
    if (loss) *loss = (double)h[cl::NPARAM] / (double)count;
    return ARK_OK;
}

// Mini-batch Adam: epochs over the dataset in batches of `batch` samples; batch b of nb takes
// samples b, b + nb, b + 2 nb, ... (every batch spans the whole dataset).  loss (may be NULL):
// mean squared error of the last epoch's batches (each taken before its step).
int ark_mlp_train(ark_mlp *M, ark_closure_data *d, int epochs, long long batch, double lr, double *loss) {
    if (!M || !d || epochs < 0 || batch < 1 || !(lr > 0)) return cfail(ARK_ERR_PARAM, "bad arguments");
    const long long nb = d->n / batch;
    if (nb < 1) return cfail(ARK_ERR_PARAM, "fewer samples than one batch");
    if (int rc = prepare_grad()) return rc;
    CL_CUDA(cudaStreamSynchronize(d->st));
    float *lossacc = nullptr;
    CL_CUDA(cudaMalloc(&lossacc, sizeof(float)));
    const cl::Adam a = {(float)lr, 0.9f, 0.999f, 1e-8f};
    int rc = ARK_OK;
    for (int ep = 0; ep < epochs && rc == ARK_OK; ++ep) {
        cudaMemsetAsync(lossacc, 0, sizeof(float), M->st);
        for (long long b = 0; b < nb; ++b) {
            launch_grad(M, d, 0, batch, nb, b);
            M->step += 1;
            cl::k_adam<<<(cl::NPARAM + 255) / 256, 256, 0, M->st>>>(M->master, M->m, M->v, M->grad, M->net, a, M->step);
            cl::k_add_loss<<<1, 32, 0, M->st>>>(M->grad, lossacc, (float)(1.0 / ((double)batch * (double)nb)));
            if (cudaGetLastError() != cudaSuccess) {
                rc = cfail(ARK_ERR_CUDA, "training launch failed");
                break;
            }
        }
    }
    float h = 0.f;
    if (rc == ARK_OK) {
        cudaError_t e = cudaStreamSynchronize(M->st);
        if (e == cudaSuccess) e = cudaMemcpy(&h, lossacc, sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cfail(ARK_ERR_CUDA, std::string("training: ") + cudaGetErrorString(e));
    }
    cudaFree(lossacc);
    if (rc) return rc;
    if (loss) *loss = epochs > 0 ? (double)h : 0.0;
    return ARK_OK;
}

int ark_mlp_predict_tc(ark_mlp *M, ark_closure_data *d, long long first, long long count, float *out) {
    if (!M || !d || !out || first < 0 || count < 0 || first + count > d->n) return cfail(ARK_ERR_PARAM, "bad range");
    if (count == 0) return ARK_OK;
    float *o = nullptr;
    CL_CUDA(cudaStreamSynchronize(d->st));
    CL_CUDA(cudaMalloc(&o, sizeof(float) * count));
    cl::k_mlp_predict_tc<<<cl::grid_for(count, 128), 128, 0, M->st>>>(d->feat + first * cl::NIN, count, M->net, o);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(M->st);
    if (e == cudaSuccess) e = cudaMemcpy(out, o, sizeof(float) * count, cudaMemcpyDeviceToHost);
    cudaFree(o);
    if (e != cudaSuccess) return cfail(ARK_ERR_CUDA, std::string("predict: ") + cudaGetErrorString(e));
    return ARK_OK;
}

int ark_mlp_predict(ark_mlp *M, ark_closure_data *d, long long first, long long count, float *out) {
    if (!M || !d || !out || first < 0 || count < 0 || first + count > d->n) return cfail(ARK_ERR_PARAM, "bad range");
    if (count == 0) return ARK_OK;
    float *o = nullptr;
    CL_CUDA(cudaStreamSynchronize(d->st));
    CL_CUDA(cudaMalloc(&o, sizeof(float) * count));
    cl::k_mlp_predict<<<cl::grid_for(count), 256, 0, M->st>>>(d->feat + first * cl::NIN, count, M->net, o);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(M->st);
    if (e == cudaSuccess) e = cudaMemcpy(out, o, sizeof(float) * count, cudaMemcpyDeviceToHost);
    cudaFree(o);
    if (e != cudaSuccess) return cfail(ARK_ERR_CUDA, std::string("predict: ") + cudaGetErrorString(e));
    return ARK_OK;
}

} // extern "C"

// the network constants, for ark_api.cu's closure step
namespace ark {
const void *mlp_device_net(const ark_mlp *M) { return M ? (const void *)M->net : nullptr; }
size_t mlp_bytes() { return sizeof(cl::Net); }
int mlp_snapshot_device(const ark_mlp *M, void *dev_out) {
    if (!M || !dev_out) return ARK_ERR_PARAM;
    if (cudaStreamSynchronize(M->st) != cudaSuccess) return ARK_ERR_CUDA;
    if (cudaMemcpy(dev_out, M->net, sizeof(cl::Net), cudaMemcpyDeviceToDevice) != cudaSuccess) return ARK_ERR_CUDA;
    return ARK_OK;
}
} // namespace ark
