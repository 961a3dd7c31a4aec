// Device-side data model of the CABARET step (shared by host launch code and kernels).
//
// Layout in HBM: every field is its own array in the reference's Arr3d index space
// (source/Arr3d.cpp:19-21, i fastest), so the host<->device transfer of a reference array
// is one contiguous copy:
//   cells  (C1+2)(C2+2)(C3+2)   interior 1..C, one ghost layer (main.cpp:198-224)
//   faces  (C1+3)(C2+3)(C3+3)   faces normal to d: 1..C_d+1 along d, halo 0 and C_d+2
// Two cell levels hold "Con" and "nCon"; the step swaps their roles instead of copying
// (Phase1's nCon -> Con copy, main.cpp:419-432, becomes a relabelling).
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <cuda_runtime.h>

namespace ark {

// A divisor known before its quotients are taken (a run constant, or dt for one step), for
// FP64 division on the integer pipes (qdiv): r = ceil(2^116 / M) for the divisor's 53-bit
// significand M in [2^52, 2^53) (2^64 - 1 when M = 2^52), k = 1022 - the divisor's biased
// exponent, sgn = its sign bit in the high word.  A zero, subnormal or non-finite divisor gets
// k = -100000, which sends every quotient to the FP64 path.
struct QRecip {
    unsigned r0, r1; // r: low and high words
    int k;
    unsigned sgn;
};

__host__ __device__ inline QRecip make_qrecip(double b) {
    unsigned long long bits;
#ifdef __CUDA_ARCH__
    bits = (unsigned long long)__double_as_longlong(b);
#else
    std::memcpy(&bits, &b, sizeof bits);
#endif
    QRecip q;
    const int eb = (int)((bits >> 52) & 0x7FFull);
    q.sgn = (unsigned)(bits >> 32) & 0x80000000u;
    q.r0 = q.r1 = 0u;
    q.k = -100000;
    if (eb == 0 || eb == 0x7FF) return q;
    const unsigned long long M = (bits & 0x000FFFFFFFFFFFFFull) | (1ull << 52);
    unsigned long long r = ~0ull;
    if (M != (1ull << 52)) {
        // d = RN(2^116 / M) is an integer within 2^10 of the quotient (its ulp is 2^11), so the
        // remainder 2^116 - M d lies within M 2^10 < 2^63 of zero: its low 64 bits are exact.
        const double d = 0x1p116 / (double)M;
        const unsigned long long q0 = (unsigned long long)d;
        const long long rem = (long long)(0ull - M * q0);
        long long c = rem / (long long)M;
        if (rem - c * (long long)M < 0) c -= 1; // floor division
        // 2^116 / M is not an integer (M is not a power of two): ceil = floor + 1
        r = q0 + (unsigned long long)c + 1ull;
    }
    q.r0 = (unsigned)r;
    q.r1 = (unsigned)(r >> 32);
    q.k = 1022 - eb;
    return q;
}

struct Geom {
    int C1, C2, C3;
    int64_t cs1, cs2; // cell strides of j and k
    int64_t fs1, fs2; // face strides of j and k
    __host__ __device__ __forceinline__ int64_t cell(int i, int j, int k) const {
        return (int64_t)k * cs2 + (int64_t)j * cs1 + i;
    }
    __host__ __device__ __forceinline__ int64_t face(int i, int j, int k) const {
        return (int64_t)k * fs2 + (int64_t)j * fs1 + i;
    }
    // 32-bit forms for the hot kernels (ark_create keeps every array below 2^31 elements)
    __host__ __device__ __forceinline__ int ci(int i, int j, int k) const {
        return (k * (int)cs1 * (C2 + 2)) + j * (int)cs1 + i;
    }
    __host__ __device__ __forceinline__ int fi(int i, int j, int k) const {
        return (k * (int)fs1 * (C2 + 3)) + j * (int)fs1 + i;
    }
    __host__ __device__ int64_t ncell() const { return cs2 * (C3 + 2); }
    __host__ __device__ int64_t nface() const { return fs2 * (C3 + 3); }
};

// The reference's Arr3d layout (source/Arr3d.cpp:19-21, i fastest): rows of C1+2 cells or
// C1+3 faces.  Host arrays always have it.
inline Geom host_geom(int C1, int C2, int C3) {
    Geom g;
    g.C1 = C1;
    g.C2 = C2;
    g.C3 = C3;
    g.cs1 = C1 + 2;
    g.cs2 = (int64_t)(C1 + 2) * (C2 + 2);
    g.fs1 = C1 + 3;
    g.fs2 = (int64_t)(C1 + 3) * (C2 + 3);
    return g;
}

// Lines per warp in the x1 sweep: a warp walks the cells 0..C1+1 of that many consecutive lines as
// one stream of positions, 32 at a time, so a chunk that ends one line carries on with the next
// instead of leaving lanes idle (a 32-cell line alone fills 34 of 64 lanes).  Short lines: 4.
// Long lines waste less, and the count also sets how evenly the blocks fill the GPU's waves:
// FP64 takes 3 (at 256x128x128: 1 line 0.495 ms, 2 lines 0.484, 3 lines 0.457, where the
// blocks make 3.0 waves; 4 lines 20% slower), FP32 1 (2 lines: 0.422 -> 0.431 ms at
// 512x256x256).  ark_autotune tries 1 to 4 per context.
__host__ __device__ inline int x_lines_per_warp(const Geom &g, bool fp64 = false) {
    return g.C1 < 200 ? 4 : fp64 ? 3 : 1;
}

// Device arrays keep the same (i, j, k) indexing with every row padded to one pitch for cells
// and faces: a multiple of 32 elements (rows start on 128-byte boundaries, as bulk copies need),
// and long enough that the row segment a 64-cell tile stages (68 elements from x = 64*tile, or
// 80 flag bytes) never leaves its row.
constexpr int kRowAlign = 32;
inline int device_pitch(int C1) {
    const int need_seg = 64 * ((C1 + 63) / 64) + 16;
    const int need = C1 + 3 > need_seg ? C1 + 3 : need_seg;
    return (need + kRowAlign - 1) / kRowAlign * kRowAlign;
}
// staged = false: rows only aligned (a multiple of 32 elements, at least C1 + 3), for arrays the
// shared-memory-staged kernels never read (ensemble members)
inline Geom device_geom(int C1, int C2, int C3, bool staged = true) {
    Geom g = host_geom(C1, C2, C3);
    const int P = staged ? device_pitch(C1) : (C1 + 3 + kRowAlign - 1) / kRowAlign * kRowAlign;
    g.cs1 = P;
    g.cs2 = (int64_t)P * (C2 + 2);
    g.fs1 = P;
    g.fs2 = (int64_t)P * (C2 + 3);
    return g;
}

// One array between the host's Arr3d layout and the device's padded rows (rows of C1+2 cells
// or C1+3 faces; elem bytes per element).  Asynchronous on st.
inline cudaError_t copy_rows(void *dst, const void *src, const Geom &dg, int face, size_t elem, cudaMemcpyKind kind,
                             cudaStream_t st) {
    const size_t w = (size_t)(face ? dg.C1 + 3 : dg.C1 + 2) * elem;
    const size_t rows = face ? (size_t)(dg.C2 + 3) * (dg.C3 + 3) : (size_t)(dg.C2 + 2) * (dg.C3 + 2);
    const size_t dpitch = (size_t)(face ? dg.fs1 : dg.cs1) * elem;
    if (kind == cudaMemcpyHostToDevice) return cudaMemcpy2DAsync(dst, dpitch, src, w, w, rows, kind, st);
    return cudaMemcpy2DAsync(dst, w, src, dpitch, w, rows, kind, st);
}

// Tiling of the per-cell kernels: a block covers kTileX x kTileY cells of a k-column chunk
// of kTileK planes and marches through it in k.  The reductions that TimeStepSize and the
// bulk forcing need are taken per block into partial slots (one per block).
constexpr int kTileX = 64, kTileY = 2, kTileK = 16;
__host__ __device__ inline int tiles_x(const Geom &g) { return (g.C1 + kTileX - 1) / kTileX; }
__host__ __device__ inline int tiles_y(const Geom &g) { return (g.C2 + kTileY - 1) / kTileY; }
__host__ __device__ inline int tiles_k(const Geom &g) { return (g.C3 + kTileK - 1) / kTileK; }
__host__ __device__ inline int tile_count(const Geom &g) { return tiles_x(g) * tiles_y(g) * tiles_k(g); }

// Blocks fold their partials into kBuckets slots with atomics (block b -> slot b % kBuckets);
// k_finalize_dt reads the slots and clears them.  Max and integer sums are order
// independent, so the result does not depend on the launch configuration.
constexpr int kBuckets = 256;

// Sticky device status bits.
// STATUS_STAGING: a shared-memory staging wait (TMA copies on an mbarrier) gave up
enum : int { STATUS_NONFINITE = 1, STATUS_STAGING = 2 };

// Cell-flag bits: the reference tests the double `condition` three ways.
enum : uint8_t {
    FL_LT = 1, // condition < 0.5   (fluid in Phase1, stress and Phase2 branches)
    FL_GT = 2, // condition > 0.5   (solid in stress and Phase2 branches)
    FL_EQ0 = 4 // condition == 0    (StressTensor force and UseForces, main.cpp:999,1035)
};

template <class T> struct Level { T *ro, *u1, *u2, *u3; };

// Faces normal to one axis: pressure, density, velocity components u[0..2].
template <class T> struct FaceSet { T *p, *ro, *u[3]; };

// Constants of a run rounded to one precision, computed on the host (kernels never convert
// or divide to get them: FP64 instructions run at 1/64 of the FP32 rate on this part).
template <class T> struct KT {
    T dx[3], rdx[3];  // grid steps and their reciprocals
    T vrdx[3];        // VIS / dx_d (FP32 stress coefficients)
    T ds[3], dvc, rdvc;
    T vis, two_vis, sound, ro0, c2, rc2, roc, rroc;
    QRecip q_dx[3], q_dvc, q_roc, q_c2; // FP64: the divisors dx, dvc, ro0*c and c^2 for qdiv
};

// Constants of a run, computed once on the host in double, plus their per-precision copies.
struct Consts {
    double dx[3], rdx[3];  // grid steps and their correctly rounded reciprocals
    double ds[3], dvc;     // face areas dx2*dx3, dx1*dx3, dx1*dx2 and cell volume dx1*dx2*dx3
    double vis, two_vis;   // VIS and 2*VIS
    double sound, ro0;
    double c2, rc2;        // sound*sound and its reciprocal
    double roc, rroc;      // ro0_g*sound and its reciprocal
    double cfl_dx[3];      // CFL*dx_d (TimeStepSize's numerators)
    double dtv;            // viscous dt limit of TimeStepSize (cell independent)
    double u_target;
    int forcing;
    int periodic_x, periodic_z; // 0: the reference's bounded edges (see k_wrap, k_sweep_x)
    int ext_z;                  // 1: the z ghosts are filled from outside (a slab of a z split)
    KT<double> kd;
    KT<float> kf;
};

template <class T> __host__ __device__ inline const KT<T> &kconst(const Consts &k);
template <> __host__ __device__ inline const KT<double> &kconst<double>(const Consts &k) { return k.kd; }
template <> __host__ __device__ inline const KT<float> &kconst<float>(const Consts &k) { return k.kf; }

// Scalars and reduction accumulators living on the device, so a whole step (and a
// CUDA graph of it) never waits for the host.
struct DevScalars {
    double dt, time, ub, G;
    long long nstep;
    long long nfluid;  // fluid cells (condition == 0), set at upload
    int status;        // sticky error bits (STATUS_NONFINITE, STATUS_STAGING)
    int pad;
    long long sums[5]; // conservation sums (fixed point), see ark_sums
    long long sum_cells;
    double rdt;        // 1/dt
    float dtf, rdtf, Gf, padf; // dt, 1/dt and G rounded to FP32 for the FP32 kernels
    QRecip qdt;        // dt for qdiv
};

template <class T> __device__ __forceinline__ T sc_dt(const DevScalars *s);
template <> __device__ __forceinline__ double sc_dt<double>(const DevScalars *s) { return s->dt; }
template <> __device__ __forceinline__ float sc_dt<float>(const DevScalars *s) { return s->dtf; }
template <class T> __device__ __forceinline__ T sc_rdt(const DevScalars *s);
template <> __device__ __forceinline__ double sc_rdt<double>(const DevScalars *s) { return s->rdt; }
template <> __device__ __forceinline__ float sc_rdt<float>(const DevScalars *s) { return s->rdtf; }
__device__ __forceinline__ QRecip sc_qdt(const DevScalars *s) { return s->qdt; }
template <class T> __device__ __forceinline__ T sc_G(const DevScalars *s);
template <> __device__ __forceinline__ double sc_G<double>(const DevScalars *s) { return s->G; }
template <> __device__ __forceinline__ float sc_G<float>(const DevScalars *s) { return s->Gf; }

template <class T> struct DevState {
    Geom g;
    Consts k;
    Level<T> lv[2];  // the two cell levels; which one is "Con" is passed to each kernel
    Level<T> spare;  // FP32: where the one-kernel Phase2 + second Phase1 writes the new level
    T *f[3];
    FaceSet<T> fc[2][3]; // two face generations: Phase2 reads fc[cur] and writes fc[cur^1]
    T *sig[3][3];        // sig[d][m]: component m on faces normal to d (nullptr unless kept)
    uint8_t *flags;
    DevScalars *sc;
    // partial-slot buckets: max |u_d| of the "Con" level as IEEE double bit patterns (3 per
    // slot) and the fixed-point sum of u1 over fluid cells of the "nCon" level (1 per slot)
    unsigned long long *part_max;
    long long *part_sum;
    T *nut; // eddy viscosity of the learned closure, cell layout (nullptr unless enabled)
};

// FP32 contexts store the density deviation rho - ro0 in the cell levels and derive face
// density from face pressure (ro0 + p / c^2); FP64 contexts store rho itself, as the
// reference does, so its arithmetic is mirrored operation by operation.
template <class T> struct Storage { static constexpr bool deviation = false; };
template <> struct Storage<float> { static constexpr bool deviation = true; };

// ---- z-slab decomposition (ark_slabs.cu) ----
// A grid of C3 planes split into n slabs: slab s owns the global interior planes
// [k_first, k_last] (1-based), C3 / n planes each and one more for the first C3 % n slabs.
struct SlabRange {
    int k_first, k_last, below, above; // neighbour slabs; -1: bounded edge (zero-gradient)
};
__host__ __device__ inline SlabRange slab_range(int C3, int n, int s, int periodic) {
    const int q = C3 / n, r = C3 % n;
    SlabRange R;
    R.k_first = 1 + s * q + (s < r ? s : r);
    R.k_last = R.k_first + q + (s < r ? 1 : 0) - 1;
    R.below = s > 0 ? s - 1 : (periodic ? n - 1 : -1);
    R.above = s < n - 1 ? s + 1 : (periodic ? 0 : -1);
    return R;
}
// The local plane a z ghost of a slab of c3 planes takes, and the plane of the source slab (a
// neighbour of c3_src planes, or the slab itself at a bounded edge) it comes from, as the
// periodic wrap and the zero-gradient copy of a whole domain take them (k_wrap): cells: ghost 0
// <- the plane below's last interior plane, ghost c3+1 <- the plane above's first; faces normal
// or parallel to z alike (face k lies below cell k): halo 0 <- the source's face c3_src (the
// face below its last cell), halo c3+2 <- its face 2 (the face above its first cell).  At a
// bounded edge the source is the slab itself: ghost 0 <- 1, ghost c3+1 <- c3, halo 0 <- face 1,
// halo c3+2 <- face c3+1.  side 0: below, 1: above.
struct HaloPlanes {
    int dst, src;
};
__host__ __device__ inline HaloPlanes halo_planes(int face, int side, int c3, int c3_src, bool bounded) {
    HaloPlanes h;
    if (!face) {
        h.dst = side ? c3 + 1 : 0;
        h.src = bounded ? (side ? c3 : 1) : (side ? 1 : c3_src);
    } else {
        h.dst = side ? c3 + 2 : 0;
        h.src = bounded ? (side ? c3 + 1 : 1) : (side ? 2 : c3_src);
    }
    return h;
}
// One plane copy of a halo exchange: the interior (i, j) of plane src_plane of src into plane
// dst_plane of dst, arrays of one row and plane geometry (cells or faces: face) and
// dst_planes / src_planes planes.
struct HaloJob {
    void *dst;
    const void *src;
    int dst_plane, src_plane, face, dst_planes, src_planes, pad;
};

// The x1 sweep folded into the first Phase1 (FP32, TMA-staged): a tile of tw cells of a line
// sweeps the x faces between its own cells and leaves the face at each of its seams (below its
// first column; C1 + 1 after the last tile) to the seam kernel, writing what its side of such a
// face needs.  Per slot, b: the cell behind the face (its forward extrapolation rf, af, bf, its
// half-step u1, u2, u3, ro and its flags), a: the cell ahead (qb, ab, bb, half-step u1, u2, u3,
// ro, flags, and the face's old u2, u3; slots 0 and nb also its old u1 and p, so that the seam
// kernel compares faces 1 and C1 + 1 from the seam arrays).  The ghost positions' flags (and, on a bounded x axis,
// their edge invariants and the values of the cells they stand for) are written by the tiles
// holding cells 1 and C1.  Slot (b, j, k) is element ((k - 1) * C2 + j - 1) * (nb + 1) + b of
// each array, b = 0 .. nb = ceil(C1 / tw): the seams of a line side by side, as the seam kernel's
// threads take them; seam_slots(g, 32) elements per array cover every tw.  Flags are stored as
// the bits of a float.
struct XSeams {
    float *b[8], *a[12];
    int tw, n; // tile width; elements per array (bounds-checked builds)
    int kch;   // planes per block of the launch (the chunks whose first planes' z faces are left)
};
__host__ __device__ inline long long seam_slots(const Geom &g, int tw) {
    return (long long)((g.C1 + tw - 1) / tw + 1) * g.C2 * g.C3;
}
__host__ __device__ inline int seam_slot(const Geom &g, int tw, int b, int j, int k) {
    return ((k - 1) * g.C2 + j - 1) * ((g.C1 + tw - 1) / tw + 1) + b;
}

// Launch entry points (defined per precision in ark_fp64.cu / ark_fp32.cu).
// P1_RMAX / P1_RSUM: also take the dt partials (max |u| of the level written) or the bulk-flow
// partials (sum of u1 of the level written) for the next step.
// P1_NUT: the stress uses vis + nu_t averaged to each face (learned closure; one-cell kernel).
enum Phase1Mode { P1_PLAIN = 0, P1_STRESS = 1, P1_FORCES = 2, P1_BULK = 4, P1_RMAX = 8, P1_RSUM = 16, P1_NUT = 32 };

template <class T> struct Launch {
    static void reduce_start(const DevState<T> &S, int con, cudaStream_t st);
    static void finalize_dt(const DevState<T> &S, int advance_time, cudaStream_t st);
    // with_ro: 1 also roCon on z, 2 on x and z (for the one-kernel Phase2 forms)
    static void wrap_con(const DevState<T> &S, int con, int with_ro, cudaStream_t st);
    // xlines: also the x ghosts (the one-kernel Phase2 forms read them; the x1 sweep does not)
    static void wrap_phase2(const DevState<T> &S, int con, int fcur, cudaStream_t st, int xlines = 0);
    // kch: planes per block of the staged and face-centric forms (0: their default)
    static void phase1(const DevState<T> &S, int src, int dst, int fcur, int mode, int march, cudaStream_t st,
                       int kch = 0);
    // FP32, TMA-staged shapes (march 4 / 5): Phase1 + stress with the x1 sweep folded in (the x
    // faces between the cells of each tile; X.tw is set to the tile width).  Returns false,
    // launching nothing, where that form is not available (the caller runs phase1 and the x1
    // sweep instead).
    // fold: 1 the x1 sweep, 3 the x1 and x3 sweeps (X.kch set to the planes per block)
    static bool phase1_sweep_x(const DevState<T> &S, int src, int dst, int fcur, int mode, int march, cudaStream_t st,
                               int kch, XSeams &X, int fold = 1);
    // the x faces phase1_sweep_x leaves: the tile seams and the faces beside the ghost positions
    static void sweep_x_seams(const DevState<T> &S, int con, int fcur, const XSeams &X, cudaStream_t st);
    // the z faces it leaves with the x3 sweep folded in: below each chunk's first plane, and C3 + 1
    static void sweep_z_seams(const DevState<T> &S, int con, int fcur, int kch, cudaStream_t st);
    static void stress(const DevState<T> &S, int con, int bulk, cudaStream_t st);
    static void use_forces(const DevState<T> &S, int ncon, cudaStream_t st);
    // x2/x3 sweeps: lines cut into balanced segments of at most `target` faces
    // x1 sweep: xlines lines per warp (0: x_lines_per_warp's choice)
    static void sweep(const DevState<T> &S, int con, int fcur, int axis, cudaStream_t st, int target = 32, int xlines = 0);
    // the three sweeps in one kernel (same results)
    static void phase2_fused(const DevState<T> &S, int con, int fcur, cudaStream_t st);
    // FP32: the three sweeps and the second Phase1 (UseForces, bulk-flow partials) in one kernel,
    // the new level written to `out` (not a level the launch reads); same results as the
    // separate kernels.  No-op for FP64.
    // tma: stage the planes with tensor-map copies (same results)
    static void phase2_phase1(const DevState<T> &S, int con, int fcur, const Level<T> &out, cudaStream_t st, bool tma = false);
    static void boundary_fill(const DevState<T> &S, int ncon, int axis, int periodic, cudaStream_t st);
    static void sums(const DevState<T> &S, int ncon, cudaStream_t st);
    static void mean_profile(const DevState<T> &S, int ncon, long long *acc, cudaStream_t st);
    // the plane copies of a slab group's halo exchange (device job table of njobs entries);
    // g: the geometry of the slabs' rows and planes (all slabs share C1, C2 and the pitch)
    static void halo_exchange(const Geom &g, const HaloJob *jobs, int njobs, cudaStream_t st);
    // one-time launch attributes (the staged Phase1's shared memory); host only
    static void prepare();
    // FP32: a TMA-staged Phase1 + stress whose planes expect 16 bytes more than they bring, so
    // its bounded waits give up and set STATUS_STAGING (the error path, without a fault); 1 if
    // launched, 0 if the TMA form is unavailable (FP64: 0)
    static int staging_unmet(const DevState<T> &S, int src, int dst, int fcur, cudaStream_t st);
};

// Checks the staged Phase1's copy plan of a C1 x C2 x C3 grid with kch planes per block (0:
// the launch's choice) on the host: every 16-byte copy in bounds, aligned, inside its stage,
// and every shared-memory read of every thread mapped to the global element the one-cell
// kernel reads.  Returns the number of problems
// (a description of the first in msg).
int staging_plan_check(int C1, int C2, int C3, int kch, char *msg, int cap);
// The same check for the one-kernel Phase2 + second Phase1 (s2 namespace): every copy, and every
// shared-memory read of every thread and halo job mapped to the element the sweeps read.
int step2_plan_check(int C1, int C2, int C3, int kch, char *msg, int cap);

// ---- output and statistics (ark_output.cu) ----
// The reference's averageU arrays are (n1+1) x (n2+2) x (n3+1) = (C1+2) x (C2+3) x (C3+2)
// (main.cpp:225-227): one j row more than the cell arrays.
__host__ __device__ inline int64_t avg_index(const Geom &g, int i, int j, int k) {
    return ((int64_t)k * (g.C2 + 3) + j) * (g.C1 + 2) + i;
}
__host__ __device__ inline int64_t avg_count(const Geom &g) { return (int64_t)(g.C1 + 2) * (g.C2 + 3) * (g.C3 + 2); }

struct AvgArrays {
    double *a[3];
};

// Cells of planes [k0, k1) (1-based) in file order, i fastest; a null pointer skips a field.
// u, r: 3 doubles per cell; pc: 1; avg_out: 3 (avg[m] / avg_div).  swap: big-endian bytes.
struct CellPack {
    double *u, *pc, *r, *avg_out;
    const double *avg[3];
    double avg_div;
    int k0, k1, swap;
};

template <class T> void output_pack(const DevState<T> &S, int ncon, int fcur, const CellPack &a, cudaStream_t st);
template <class T> void output_average_add(const DevState<T> &S, int ncon, const AvgArrays &A, cudaStream_t st);
// sum over interior cells of (u1^2 + u2^2 + u3^2)/2 of level ncon into *out (device), in a
// fixed order; scratch holds energy_scratch_count(g) doubles
int energy_scratch_count(const Geom &g);
// per y plane of level ncon: means of u1, u2, u3, u1^2, u2^2, u3^2, u1u2, u1u3, u2u3 (9 * C2, device)
template <class T> void output_plane_stats(const DevState<T> &S, int ncon, double *out, cudaStream_t st);
template <class T> void output_energy(const DevState<T> &S, int ncon, double *scratch, double *out, cudaStream_t st);

// ---- learned closure (ark_closure.cu) ----
} // namespace ark
struct ark_mlp;
namespace ark {
// nu_t of level lvl into S.nut (interior cells and periodic ghost images); net: the network's
// device constants (mlp_device_net); yplus_scale = u_tau / vis.
template <class T> void closure_nut(const DevState<T> &S, int lvl, const void *net, float yplus_scale, cudaStream_t st);
// the network's constants (weights, normalisation) copied into a device buffer of mlp_bytes()
// bytes, which closure_nut reads
size_t mlp_bytes();
int mlp_snapshot_device(const ark_mlp *M, void *dev_out);
// the interior velocities of level lvl into three compact FP64 arrays
template <class T> void closure_gather(const DevState<T> &S, int lvl, double *u0, double *u1, double *u2, cudaStream_t st);
// samples of a C1 x C2 x C3 grid on the lattice (sx, sz, ox, oz), or -1 for a bad lattice
long long closure_count(int C1, int C2, int C3, int sx, int sz, int ox, int oz);

// div_rn and qdiv against the hardware division on n random operand pairs (mismatches added to *bad)
int selftest_division(long long n, unsigned long long seed, unsigned long long *bad, cudaStream_t st);

// Between a contiguous double staging buffer (rows of w values) and the device's padded rows
// (pitch): dst = (T)(src - offset), dst = (double)src + offset, and for FP32 contexts the face
// density dst = ro0 + (double)p * rc2.
template <class T>
void rows_from_double(T *dst, const double *src, int w, int64_t rows, int pitch, double offset, cudaStream_t st);
template <class T>
void rows_to_double(double *dst, const T *src, int w, int64_t rows, int pitch, double offset, cudaStream_t st);
// the same with dst / src page-locked host memory (16-byte aligned) read or written in place
template <class T>
void flat_from_host(T *dst, const double *src, int w, int64_t rows, int pitch, double offset, cudaStream_t st);
template <class T>
void flat_to_host(double *dst, const T *src, int w, int64_t rows, int pitch, double offset, cudaStream_t st);
template <class T>
void rows_face_density(double *dst, const T *p, int w, int64_t rows, int pitch, double ro0, double rc2, cudaStream_t st);
// the row shape of a cell (face = 0) or face (1) array: w values per row, rows, pitch
struct RowShape {
    int w;
    int64_t rows;
    int pitch;
};
inline RowShape row_shape(const Geom &dg, int face) {
    RowShape r;
    r.w = face ? dg.C1 + 3 : dg.C1 + 2;
    r.rows = face ? (int64_t)(dg.C2 + 3) * (dg.C3 + 3) : (int64_t)(dg.C2 + 2) * (dg.C3 + 2);
    r.pitch = (int)(face ? dg.fs1 : dg.cs1);
    return r;
}

} // namespace ark

namespace ark {
// Records msg as the calling thread's ark_last_error() text and returns status (ark_api.cu).
int api_fail(int status, const std::string &msg);
} // namespace ark

struct ark_closure_data;
struct ark_mlp;
namespace ark {
long long closure_room(const ark_closure_data *d);
int closure_scratch(ark_closure_data *d, long long cells, double **u);
int closure_sample(ark_closure_data *d, int C1, int C2, int C3, double lx, double ly, double lz, double vis, int sx,
                   int sz, int ox, int oz, double u_tau, cudaStream_t ctx_st);
const void *mlp_device_net(const ark_mlp *M);
} // namespace ark
