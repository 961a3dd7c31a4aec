// Output and statistics on the device: the cell data of the reference's VTK writers
// (WriteDataParaView main.cpp:2577-2745, WriteAverageValues main.cpp:2747-2849) packed in file
// order and byte order, the time averages of AverageValues (main.cpp:2878-2891), and the
// kinetic energy of WriteEnergy (main.cpp:2851-2876).  Both precisions; results in double.
#include "ark_state.h"

namespace ark {
namespace {

// IEEE double in big-endian byte order (the reference writes with needSwap = true,
// main.cpp:120, swap8 main.cpp:2975-2989): reverse the 8 bytes.
__device__ __forceinline__ double be64(double v, int swap) {
    if (!swap) return v;
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned lo = (unsigned)b, hi = (unsigned)(b >> 32);
    const unsigned long long r = ((unsigned long long)__byte_perm(lo, 0, 0x0123) << 32) | __byte_perm(hi, 0, 0x0123);
    return __longlong_as_double((long long)r);
}

template <class T> __device__ __forceinline__ double cell_density(const DevState<T> &S, T v) {
    return Storage<T>::deviation ? S.k.ro0 + (double)v : (double)v;
}

// One thread per interior cell of planes [k0, k1), numbered in file order (i fastest).
template <class T> __global__ void k_pack(const __grid_constant__ DevState<T> S, int ncon, int fcur, CellPack a) {
    const Geom g = S.g;
    const int plane = g.C1 * g.C2;
    const int n = (a.k1 - a.k0) * plane;
    const Level<T> L = S.lv[ncon];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int kk = t / plane, rem = t - kk * plane;
        const int j = rem / g.C1 + 1, i = rem - (j - 1) * g.C1 + 1, k = a.k0 + kk;
        const int64_t c = g.cell(i, j, k);
        if (a.u) { // U: u1nCon, u2nCon, u3nCon (main.cpp:2653-2667)
            a.u[3 * (int64_t)t + 0] = be64((double)L.u1[c], a.swap);
            a.u[3 * (int64_t)t + 1] = be64((double)L.u2[c], a.swap);
            a.u[3 * (int64_t)t + 2] = be64((double)L.u3[c], a.swap);
        }
        if (a.pc) a.pc[t] = be64(cell_density(S, L.ro[c]), a.swap); // PC: ronCon (main.cpp:2686-2690)
        if (a.r) {
            // R: the curl from face differences (main.cpp:2716-2733), in double
            const FaceSet<T> &F1 = S.fc[fcur][0], &F2 = S.fc[fcur][1], &F3 = S.fc[fcur][2];
            const int64_t f = g.face(i, j, k);
            const double d2u3 = ((double)F2.u[2][f + g.fs1] - (double)F2.u[2][f]) / S.k.dx[1];
            const double d3u2 = ((double)F3.u[1][f + g.fs2] - (double)F3.u[1][f]) / S.k.dx[2];
            const double d3u1 = ((double)F3.u[0][f + g.fs2] - (double)F3.u[0][f]) / S.k.dx[2];
            const double d1u3 = ((double)F1.u[2][f + 1] - (double)F1.u[2][f]) / S.k.dx[0];
            const double d1u2 = ((double)F1.u[1][f + 1] - (double)F1.u[1][f]) / S.k.dx[0];
            const double d2u1 = ((double)F2.u[0][f + g.fs1] - (double)F2.u[0][f]) / S.k.dx[1];
            a.r[3 * (int64_t)t + 0] = be64(d2u3 - d3u2, a.swap);
            a.r[3 * (int64_t)t + 1] = be64(d3u1 - d1u3, a.swap);
            a.r[3 * (int64_t)t + 2] = be64(d1u2 - d2u1, a.swap);
        }
        if (a.avg_out) { // averageU / (TIME - start) (main.cpp:2826-2838)
            const int64_t q = avg_index(g, i, j, k);
            for (int m = 0; m < 3; ++m) a.avg_out[3 * (int64_t)t + m] = be64(a.avg[m][q] / a.avg_div, a.swap);
        }
    }
}

// averageU_m += u_m nCon * dt over interior cells, dt of the step just taken.
template <class T> __global__ void k_average_add(const __grid_constant__ DevState<T> S, int ncon, AvgArrays A) {
    const Geom g = S.g;
    const int plane = g.C1 * g.C2;
    const int n = plane * g.C3;
    const Level<T> L = S.lv[ncon];
    const double dt = S.sc->dt;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int k = t / plane + 1, rem = t - (k - 1) * plane;
        const int j = rem / g.C1 + 1, i = rem - (j - 1) * g.C1 + 1;
        const int64_t c = g.cell(i, j, k), q = avg_index(g, i, j, k);
        A.a[0][q] += (double)L.u1[c] * dt;
        A.a[1][q] += (double)L.u2[c] * dt;
        A.a[2][q] += (double)L.u3[c] * dt;
    }
}

// Kinetic energy, pass 1: one block per kTileX x kTileY column tile, each thread summing its
// column over k in order, then a fixed shared-memory tree.  Deterministic.
constexpr int kEnergyThreads = kTileX * kTileY;
template <class T> __global__ void __launch_bounds__(kEnergyThreads) k_energy_tiles(const __grid_constant__ DevState<T> S, int ncon, double *part) {
    __shared__ double red[kEnergyThreads];
    const Geom g = S.g;
    const Level<T> L = S.lv[ncon];
    const int i = blockIdx.x * kTileX + threadIdx.x + 1;
    const int j = blockIdx.y * kTileY + threadIdx.y + 1;
    double e = 0.0;
    if (i <= g.C1 && j <= g.C2)
        for (int k = 1; k <= g.C3; ++k) {
            const int64_t c = g.cell(i, j, k);
            const double u1 = L.u1[c], u2 = L.u2[c], u3 = L.u3[c];
            e += (u1 * u1 + u2 * u2 + u3 * u3) / 2;
        }
    const int t = threadIdx.y * kTileX + threadIdx.x;
    red[t] = e;
    __syncthreads();
    for (int h = kEnergyThreads / 2; h > 0; h >>= 1) {
        if (t < h) red[t] += red[t + h];
        __syncthreads();
    }
    if (t == 0) part[blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// Pass 2: one block of 1024 threads, strided sums in order, then the same tree.
__global__ void __launch_bounds__(1024) k_energy_total(const double *part, int n, double *out) {
    __shared__ double red[1024];
    double e = 0.0;
    for (int q = threadIdx.x; q < n; q += 1024) e += part[q];
    red[threadIdx.x] = e;
    __syncthreads();
    for (int h = 512; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// Plane statistics (one block per y plane, fixed-order sums): over the interior cells of plane
// j of level ncon, the means of u1, u2, u3, u1^2, u2^2, u3^2, u1 u2, u1 u3, u2 u3 into
// out[9*(j-1) + q].
template <class T> __global__ void __launch_bounds__(256) k_plane_stats(const __grid_constant__ DevState<T> S, int ncon, double *out) {
    __shared__ double red[9][256];
    const Geom g = S.g;
    const int j = blockIdx.x + 1;
    const Level<T> L = S.lv[ncon];
    double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int n = g.C1 * g.C3;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int i = t % g.C1 + 1, k = t / g.C1 + 1;
        const int64_t c = g.cell(i, j, k);
        const double u1 = L.u1[c], u2 = L.u2[c], u3 = L.u3[c];
        a[0] += u1;
        a[1] += u2;
        a[2] += u3;
        a[3] += u1 * u1;
        a[4] += u2 * u2;
        a[5] += u3 * u3;
        a[6] += u1 * u2;
        a[7] += u1 * u3;
        a[8] += u2 * u3;
    }
    for (int q = 0; q < 9; ++q) red[q][threadIdx.x] = a[q];
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int q = 0; q < 9; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x < 9) out[9 * (j - 1) + threadIdx.x] = red[threadIdx.x][0] / (double)n;
}

int grid_for(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

} // namespace

template <class T> void output_pack(const DevState<T> &S, int ncon, int fcur, const CellPack &a, cudaStream_t st) {
    const int64_t n = (int64_t)(a.k1 - a.k0) * S.g.C1 * S.g.C2;
    if (n > 0) k_pack<T><<<grid_for(n), 256, 0, st>>>(S, ncon, fcur, a);
}

template <class T> void output_average_add(const DevState<T> &S, int ncon, const AvgArrays &A, cudaStream_t st) {
    const int64_t n = (int64_t)S.g.C1 * S.g.C2 * S.g.C3;
    k_average_add<T><<<grid_for(n), 256, 0, st>>>(S, ncon, A);
}

int energy_scratch_count(const Geom &g) { return tiles_x(g) * tiles_y(g); }

template <class T> void output_energy(const DevState<T> &S, int ncon, double *scratch, double *out, cudaStream_t st) {
    const dim3 grid(tiles_x(S.g), tiles_y(S.g));
    k_energy_tiles<T><<<grid, dim3(kTileX, kTileY), 0, st>>>(S, ncon, scratch);
    k_energy_total<<<1, 1024, 0, st>>>(scratch, (int)(grid.x * grid.y), out);
}

template <class T> void output_plane_stats(const DevState<T> &S, int ncon, double *out, cudaStream_t st) {
    k_plane_stats<T><<<S.g.C2, 256, 0, st>>>(S, ncon, out);
}
template void output_plane_stats<double>(const DevState<double> &, int, double *, cudaStream_t);
template void output_plane_stats<float>(const DevState<float> &, int, double *, cudaStream_t);

template void output_pack<double>(const DevState<double> &, int, int, const CellPack &, cudaStream_t);
template void output_pack<float>(const DevState<float> &, int, int, const CellPack &, cudaStream_t);
template void output_average_add<double>(const DevState<double> &, int, const AvgArrays &, cudaStream_t);
template void output_average_add<float>(const DevState<float> &, int, const AvgArrays &, cudaStream_t);
template void output_energy<double>(const DevState<double> &, int, double *, double *, cudaStream_t);
template void output_energy<float>(const DevState<float> &, int, double *, double *, cudaStream_t);

} // namespace ark
