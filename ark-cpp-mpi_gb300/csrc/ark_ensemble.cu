// Ensembles: many independent channels of different sizes and parameters advanced together,
// one launch per phase of the step for all members, the whole step captured in one CUDA graph.
//
// Each batched kernel is persistent: a grid sized to what the GPU holds at once walks a work
// list that concatenates every member's blocks ("tiles").  A block finds its member by
// binary search over the list's start offsets and then runs exactly the device code the
// single-grid kernels run (the *_body functions of ark_kernels.cuh), so each member's
// result is bit-identical to running it alone in its own ark_ctx.  Members are FP32
// contexts (density stored as rho - ro0; FP64 reductions), as the FP32 path is the
// throughput path.
//
// Kernel shapes (Phase1 marching or one cell per thread, for each of the two Phase1s; the
// face-segment length of the x2/x3 sweeps) change which thread computes what but not the
// results; ark_ensemble_autotune times every combination on the live state and keeps the
// fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ark_gpu.h"
#include "ark_kernels.cuh"

using namespace ark;

namespace ark {
Consts make_run_consts(const ark_params &p); // ark_api.cu
}

namespace {

thread_local std::string g_ens_error;

int efail(int st, const std::string &m) {
    g_ens_error = m;
    return st;
}

#define ENS_CUDA(call)                                                                               \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return efail(e_ == cudaErrorMemoryAllocation ? ARK_ERR_NOMEM : ARK_ERR_CUDA,             \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

// A work list: info[q] = {first block of member q, blocks in x, blocks in y, unused};
// extra[q] a per-member integer (the sweep segment length).
struct WorkList {
    const int4 *info;
    const int *extra;
    int n;
    int total;
};

__device__ __forceinline__ int find_member(const WorkList &W, int b) {
    int lo = 0, hi = W.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (W.info[mid].x <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ BIx decode(const WorkList &W, int q, int b) {
    // bounds-checked builds: the member found owns block b
    if (!ARK_CK_IN(q, 0, W.n - 1) || !ARK_CK_IN(b, W.info[q].x, (q + 1 < W.n ? W.info[q + 1].x : W.total) - 1)) q = 0;
    const int4 f = W.info[q];
    const int local = b - f.x;
    BIx bx;
    bx.gx = f.y;
    bx.gy = f.z;
    bx.x = local % f.y;
    const int r = local / f.y;
    bx.y = r % f.z;
    bx.z = r / f.z;
    return bx;
}

using DS = DevState<float>;

__global__ void __launch_bounds__(1024) kb_finalize(const DS *__restrict__ inst, int advance) {
    finalize_dt_body<float>(inst[blockIdx.x], advance);
}

__global__ void __launch_bounds__(kTileX *kTileY) kb_reduce(const DS *__restrict__ inst, WorkList W, int con) {
    for (int b = blockIdx.x; b < W.total; b += gridDim.x) {
        const int q = find_member(W, b);
        reduce_start_body<float>(inst[q], con, decode(W, q, b));
        __syncthreads();
    }
}

// jobs[q]: member q's ghost-fill job; threads of a block cover 128 plane points
__global__ void __launch_bounds__(128) kb_wrap(const DS *__restrict__ inst, const WrapJob *__restrict__ jobs, WorkList W) {
    for (int b = blockIdx.x; b < W.total; b += gridDim.x) {
        const int q = find_member(W, b);
        const BIx bx = decode(W, q, b);
        wrap_body_lines<float>(inst[q].g, jobs[q], bx.x * 128 + (int)threadIdx.x);
    }
}

template <int MODE, bool MARCH>
__global__ void __launch_bounds__(kTileX *kTileY) kb_phase1(const DS *__restrict__ inst, WorkList W, int src, int dst, int fcur) {
    for (int b = blockIdx.x; b < W.total; b += gridDim.x) {
        const int q = find_member(W, b);
        const BIx bx = decode(W, q, b);
        if (MARCH) phase1_march_body<float, MODE>(inst[q], src, dst, fcur, bx);
        else phase1_cell_body<float, MODE>(inst[q], src, dst, fcur, bx);
        __syncthreads();
    }
}

// Phase1 with its planes staged in shared memory: work item = a member's 64 x 4 tile and chunk of
// planes (the member's chunk length in W.extra), the single-context kernel's body.
template <int MODE>
__global__ void __launch_bounds__(stg::NT, 2) kb_phase1_staged(const DS *__restrict__ inst, WorkList W, int src, int dst,
                                                               int fcur) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ stg::RowTable rt;
    for (int b = blockIdx.x; b < W.total; b += gridDim.x) {
        const int q = find_member(W, b);
        stg::phase1_staged_body<MODE>(inst[q], src, dst, fcur, W.extra[q], decode(W, q, b), sm, rt);
        __syncthreads();
    }
}

// The tensor maps of a member for the TMA form of the staged Phase1 (64 x 4 tiles), in global
// memory: the level boxes with the stress's rows (6) or without (4), per level; the flags
// likewise; the face sets per generation; the forces.
struct MemberMaps {
    CUtensorMap lv[2][2]; // [0 with the stress, 1 without][level]
    CUtensorMap fl[2];    // [0 with the stress, 1 without]
    CUtensorMap fc[2][3]; // [generation][direction]
    CUtensorMap ff;
};

// The staged Phase1 with TMA copies: work item = a member's tile (64 x 4, or 32 x 8 when the
// work list marks the member narrow: extra = planes per chunk | narrow << 16) and chunk of
// planes, the single-context TMA kernel's body with the member's maps for that tile shape
// (maps[2 q + narrow], fenced for the copy engine once per work item); meta[narrow] the boxes.
template <int MODE> struct TmaMetas {
    stg::BoxMeta m[2];
};
template <int MODE> constexpr int tma_ens_smem() {
    return (stg::TLayout<MODE, 64, 4>::SMEM > stg::TLayout<MODE, 32, 8>::SMEM ? stg::TLayout<MODE, 64, 4>::SMEM
                                                                               : stg::TLayout<MODE, 32, 8>::SMEM) +
           128;
}
// Work items are taken from a counter (*next, zeroed before the launch) rather than in a fixed
// stride: the items differ in cost (chunk lengths, partial tiles), so the blocks finish together.
// XS: the sweeps folded in (2: the x3 sweep, the z faces inside each chunk, kb_sweep_z_seams doing
// the rest; 3: the x1 sweep too, with the member's seam arrays seams[q] for kb_sweep_x_seams).
template <int MODE, int XS = 0>
__global__ void __launch_bounds__(stg::NT + 32, 2) kb_phase1_tma(const DS *__restrict__ inst, const MemberMaps *__restrict__ maps,
                                                            const __grid_constant__ TmaMetas<MODE> meta, WorkList W, int src,
                                                            int dst, int fcur, int *next, const XSeams *__restrict__ seams) {
    constexpr bool STRESS = (MODE & P1_STRESS) != 0;
    constexpr int NS = stg::TLayout<MODE, 64, 4>::NS;
    static_assert(NS == stg::TLayout<MODE, 32, 8>::NS, "one ring depth for both tiles");
    extern __shared__ __align__(128) unsigned char sm_raw[];
    __shared__ __align__(8) unsigned long long bar[2 * stg::TLayout<MODE>::NS + 1];
    // the x1 sweep's hand-over slots between the two warps of a 64-wide tile row
    __shared__ __align__(8) unsigned char xh_raw[(XS & 1) ? sizeof(stg::XHand<64, 4, NS>) : 8];
    __shared__ int item;
    unsigned char *const sm = stg::align128(sm_raw);
    for (;;) {
        if (threadIdx.x == 0 && threadIdx.y == 0) item = atomicAdd(next, 1);
        __syncthreads();
        const int b = item;
        if (b >= W.total) break; // (block-uniform)
        const int q = find_member(W, b);
        const int extra = W.extra[q], narrow = extra >> 16, kch = extra & 0xFFFF;
        const MemberMaps *M = maps + 2 * q + narrow;
        auto map = [&](int k) -> const CUtensorMap * {
            if (k == 0) return &M->lv[STRESS ? 0 : 1][src];
            if (k == 1) return &M->fl[STRESS ? 0 : 1];
            if (k <= 4) return &M->fc[fcur][k - 2];
            return &M->ff;
        };
        const XSeams *X = (XS & 1) ? &seams[q] : nullptr;
        if (narrow)
            stg::phase1_tma_body<MODE, 32, 8, XS>(inst[q], map, meta.m[1], true, src, dst, kch, decode(W, q, b), sm, bar, fcur, X,
                                                  reinterpret_cast<stg::XHand<32, 8, NS> *>(xh_raw));
        else
            stg::phase1_tma_body<MODE, 64, 4, XS>(inst[q], map, meta.m[0], true, src, dst, kch, decode(W, q, b), sm, bar, fcur, X,
                                                  reinterpret_cast<stg::XHand<64, 4, NS> *>(xh_raw));
        __syncthreads();
    }
}

// The next work item of a block from the counter *next (zeroed before the launch); every thread
// of the block calls it.
__device__ __forceinline__ int next_item(int *next, int &slot) {
    __syncthreads(); // every thread has read the previous item
    if (threadIdx.x == 0 && threadIdx.y == 0) slot = atomicAdd(next, 1);
    __syncthreads();
    return slot;
}

__global__ void __launch_bounds__(128) kb_sweep_x(const DS *__restrict__ inst, WorkList W, int con, int fcur, int *next) {
    __shared__ int slot;
    for (int b = next_item(next, slot); b < W.total; b = next_item(next, slot)) {
        const int q = find_member(W, b);
        sweep_x_body<float>(inst[q], con, fcur, W.extra[q], decode(W, q, b));
    }
}

template <int AX>
__global__ void __launch_bounds__(128, 5) kb_sweep_col(const DS *__restrict__ inst, WorkList W, int con, int fcur, int *next) {
    __shared__ int slot;
    for (int b = next_item(next, slot); b < W.total; b = next_item(next, slot)) {
        const int q = find_member(W, b);
        sweep_col_body<float, AX>(inst[q], con, fcur, W.extra[q], decode(W, q, b));
    }
}

// The x faces the x1 sweep folded into Phase1 + stress leaves (WL_XSEAMS: per member its seam
// slots in blocks of 128, seams[q] its seam arrays), as k_sweep_x_seams for one grid.
__global__ void __launch_bounds__(128) kb_sweep_x_seams(const DS *__restrict__ inst, const XSeams *__restrict__ seams, WorkList W,
                                                        int con, int fcur, int *next) {
    __shared__ int slot;
    for (int b = next_item(next, slot); b < W.total; b = next_item(next, slot)) {
        const int q = find_member(W, b);
        sweep_x_seams_body<float>(inst[q], con, fcur, seams[q], (b - W.info[q].x) * 128 + (int)threadIdx.x);
    }
}

// The z faces the x3 sweep folded into Phase1 + stress leaves (WL_ZSEAMS: per member the column
// blocks of the x3 sweep times its chunks + 1, extra = its planes per chunk): the face below each
// chunk's first plane and face C3 + 1, each the x3 sweep's own one-face segment (as
// k_sweep_z_seams for one grid).
__global__ void __launch_bounds__(128, 5) kb_sweep_z_seams(const DS *__restrict__ inst, WorkList W, int con, int fcur, int *next) {
    __shared__ int slot;
    for (int b = next_item(next, slot); b < W.total; b = next_item(next, slot)) {
        const int q = find_member(W, b);
        const int kch = W.extra[q], C3 = inst[q].g.C3, nch = (C3 + kch - 1) / kch;
        BIx bx = decode(W, q, b);
        bx.z = bx.z < nch ? bx.z * kch : C3;
        sweep_col_body<float, 2>(inst[q], con, fcur, 1, bx);
    }
}

// Kinds of work list.
// WL_STAGED: 64 x 4 tiles of the staged Phase1 for every member; WL_STAGED_T: 32 x 8 tiles for
// the members whose width is an odd multiple of 32 (a 64-wide tile would be half empty at
// their end), 64 x 4 for the others.
// WL_ZSEAMS: the z faces at the staged Phase1's chunk boundaries (the x3 sweep folded in);
// WL_XSEAMS: the x faces at its tile seams (the x1 sweep folded in).
enum { WL_TILES = 0, WL_CELLS, WL_SWEEPX, WL_COL1, WL_COL2, WL_WRAP, WL_STAGED, WL_STAGED_T, WL_ZSEAMS, WL_XSEAMS, WL_COUNT };

// the staged Phase1 of a member of width C1 in 32 x 8 tiles (WL_STAGED_T)
inline bool narrow_tiles(int C1) { return ((C1 + 31) / 32) % 2 == 1; }

// The candidate kernel shapes the autotuner chooses between.
struct Shape {
    int march_a, march_b; // Phase1 with stress / second Phase1: 0 one cell per thread, 1 marching,
                          // 2 planes staged in shared memory (cp.async copies), 4 the same with
                          // TMA tensor copies, 5 TMA with 32 x 8 tiles for the members whose
                          // width is an odd multiple of 32; Phase1 with stress also 6 and 7:
                          // 4 and 5 with the x3 sweep folded in, 8 and 9: with the x1 and x3
                          // sweeps folded in
    int seg;              // target faces per thread segment in the x2/x3 sweeps
};

} // namespace

struct ark_ensemble {
    int n = 0;
    std::vector<ark_params> P;
    std::vector<Consts> K;
    std::vector<DS> S; // host copies of the members' device states
    std::vector<void *> allocs;
    std::vector<std::vector<double>> cond_host;
    DS *d_inst = nullptr;
    cudaStream_t st = nullptr;
    cudaStream_t fill = nullptr; // the captured step's ghost fill, beside dt
    cudaEvent_t fill_fork = nullptr, fill_join = nullptr;
    cudaEvent_t seam_fork = nullptr, seam_join = nullptr; // the folded sweeps' seams on `fill`
    std::vector<XSeams> seams; // the members' seam arrays for the folded x1 sweep (tw per shape)
    XSeams *d_seams = nullptr;
    double *stage = nullptr; // double staging buffer (largest member)
    // work lists: device arrays, rebuilt when the shape changes
    int4 *d_info[WL_COUNT] = {};
    int *d_extra[WL_COUNT] = {};
    int total[WL_COUNT] = {};
    WrapJob *d_jobs = nullptr; // [2][n]: wrap_con for level 0/1
    int persist = 1;           // persistent blocks per launch (all SMs x resident blocks)
    int persist_staged = 1;    // the same for the staged Phase1 (2 blocks of 256 threads per SM)
    // staged Phase1 with TMA copies for both launches, 32 x 8 tiles on odd-32 widths, the x3 sweep
    // folded into Phase1 + stress (64 members of mixed grids: 1.341 ms per step against 1.439)
    Shape shape = {7, 5, 32};
    MemberMaps *d_maps = nullptr;   // the members' tensor maps, [2 q + narrow] (null: the TMA form falls back)
    int *d_next = nullptr;          // work counters: the two TMA Phase1 launches, the three sweeps, the z and x seams (zeroed per step)
    stg::BoxMeta meta[2][2] = {};   // its boxes: [narrow][0 with the stress, 1 without]
    int con = 0, fcur = 0;
    bool parts_valid = false;
    bool uploaded_all = false;
    std::vector<char> uploaded;
    cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

template <class U> int ens_alloc(ark_ensemble *E, U **out, size_t n) {
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, n * sizeof(U));
    if (e != cudaSuccess) return efail(ARK_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    E->allocs.push_back(p);
    cudaMemset(p, 0, n * sizeof(U));
    *out = (U *)p;
    return ARK_OK;
}

// rows padded as the staged Phase1 needs (its 68-value row segments stay inside a row)
Geom geom_of(const ark_params &p) { return device_geom(p.n1_cells, p.n2_cells, p.n3_cells, true); }

// n arrays of `each` floats in one allocation, a fixed stride apart (one tensor map covers them)
int ens_block(ark_ensemble *E, float **const *out, int n, size_t each) {
    float *base = nullptr;
    if (int rc = ens_alloc(E, &base, each * n)) return rc;
    for (int q = 0; q < n; ++q) *out[q] = base + each * q;
    return ARK_OK;
}

int alloc_member(ark_ensemble *E, DS &S) {
    const size_t nc = (size_t)S.g.ncell(), nf = (size_t)S.g.nface();
    int rc = 0;
    for (int l = 0; l < 2; ++l) {
        float **lv[4] = {&S.lv[l].ro, &S.lv[l].u1, &S.lv[l].u2, &S.lv[l].u3};
        rc |= ens_block(E, lv, 4, nc);
    }
    float **ff[3] = {&S.f[0], &S.f[1], &S.f[2]};
    rc |= ens_block(E, ff, 3, nc);
    for (int gen = 0; gen < 2; ++gen)
        for (int d = 0; d < 3; ++d) {
            FaceSet<float> &F = S.fc[gen][d];
            float **fs[4] = {&F.p, &F.u[0], &F.u[1], &F.u[2]};
            rc |= ens_block(E, fs, 4, nf);
            F.ro = nullptr; // FP32 derives face density from p
        }
    for (int d = 0; d < 3; ++d)
        for (int m = 0; m < 3; ++m) S.sig[d][m] = nullptr;
    rc |= ens_alloc(E, &S.flags, nc);
    rc |= ens_alloc(E, &S.sc, 1);
    rc |= ens_alloc(E, &S.part_max, 3 * (size_t)kBuckets);
    rc |= ens_alloc(E, &S.part_sum, (size_t)kBuckets);
    return rc ? ARK_ERR_NOMEM : ARK_OK;
}

// The members' tensor maps for the TMA form of the staged Phase1 (left null, so that the
// cp.async form runs, when a member's arrays do not allow it or the encoder is missing).
int build_maps(ark_ensemble *E) {
    constexpr int MS = P1_STRESS | P1_FORCES | P1_RMAX, MF = P1_FORCES | P1_RSUM;
    std::vector<MemberMaps> h(2 * (size_t)E->n);
    std::memset(h.data(), 0, sizeof(MemberMaps) * h.size());
    for (int q = 0; q < E->n; ++q) {
        const DS &S = E->S[q];
        for (int narrow = 0; narrow < 2; ++narrow)
            for (int l = 0; l < 2; ++l)
                for (int gen = 0; gen < 2; ++gen) {
                    stg::TmaBox B[stg::kMaxBoxes], F[stg::kMaxBoxes];
                    const stg::Bases bs = stg::bases_of<MS>(S, l, gen), bf = stg::bases_of<MF>(S, l, gen);
                    const int ns = narrow ? stg::tma_boxes<MS, 32, 8>(B, S.g, bs) : stg::tma_boxes<MS, 64, 4>(B, S.g, bs);
                    const int nf = narrow ? stg::tma_boxes<MF, 32, 8>(F, S.g, bf) : stg::tma_boxes<MF, 64, 4>(F, S.g, bf);
                    if (ns != 5 || nf != 6) return ARK_OK;
                    MemberMaps &m = h[2 * q + narrow];
                    bool ok = stg::encode_box(&m.lv[0][l], B[0]) && stg::encode_box(&m.lv[1][l], F[0]) &&
                              stg::encode_box(&m.fl[0], B[1]) && stg::encode_box(&m.fl[1], F[1]) &&
                              stg::encode_box(&m.ff, F[5]);
                    for (int d = 0; d < 3; ++d) ok = ok && stg::encode_box(&m.fc[gen][d], B[2 + d]);
                    if (!ok) return ARK_OK;
                    if (q == 0 && l == 0 && gen == 0) {
                        stg::box_meta(E->meta[narrow][0], B, ns);
                        stg::box_meta(E->meta[narrow][1], F, nf);
                    }
                }
    }
    if (int rc = ens_alloc(E, &E->d_maps, h.size())) return rc;  // [2 q + narrow]
    ENS_CUDA(cudaMemcpy(E->d_maps, h.data(), sizeof(MemberMaps) * h.size(), cudaMemcpyHostToDevice));
    return ARK_OK;
}

int segment_for(int nd, int target) {
    const int ns = (nd + target - 1) / target;
    return (nd + ns - 1) / ns;
}

// The x1 sweep's tile width for a member under a shape: 32 where the shape stages the member's
// planes in 32 x 8 tiles (shapes 5, 7, 9 on odd-32 widths), else 64.
int seam_width(const Shape &s, const Geom &g) {
    const bool t = s.march_a == 5 || s.march_a == 7 || s.march_a == 9;
    return t && narrow_tiles(g.C1) ? 32 : 64;
}

// Builds the work lists for the current shape.
int build_lists(ark_ensemble *E) {
    // Planes per staged Phase1 block, sized over the whole ensemble (about four waves of two
    // blocks per SM, 8 to 64 planes) rather than per member as staged_chunk sizes them for one
    // grid: the members share the GPU, so their chunks are longer than each would take alone,
    // with fewer halo planes and pipeline starts per plane computed.  Measured on the 64-member
    // mixed ensemble: 7,775 Mcell-steps/s at four waves, 7,656 at eight, 7,526 at two, 7,459 at
    // sixteen, 7,226 with each member's own chunks.
    long long colplanes = 0;
    for (int q = 0; q < E->n; ++q) {
        const Geom &g = E->S[q].g;
        colplanes += (long long)tiles_x(g) * ((g.C2 + stg::SY - 1) / stg::SY) * g.C3;
    }
    const int kens = (int)std::max(8ll, std::min(64ll, colplanes / (152 * 2 * 4)));
    for (int kind = 0; kind < WL_COUNT; ++kind) {
        std::vector<int4> info(E->n);
        std::vector<int> extra(E->n, 0);
        int start = 0;
        for (int q = 0; q < E->n; ++q) {
            const Geom &g = E->S[q].g;
            int gx = 1, gy = 1, gz = 1;
            switch (kind) {
            case WL_TILES: gx = tiles_x(g), gy = tiles_y(g), gz = tiles_k(g); break;
            case WL_CELLS: gx = tiles_x(g), gy = tiles_y(g), gz = g.C3; break;
            case WL_SWEEPX: {
                const int gl = x_lines_per_warp(g);
                extra[q] = gl;
                gx = (g.C2 * g.C3 + 4 * gl - 1) / (4 * gl);
                break;
            }
            case WL_COL1: {
                const int seg = segment_for(g.C2 + 1, E->shape.seg);
                extra[q] = seg;
                gx = col_sweep_blocks(g, 1), gz = (g.C2 + 1 + seg - 1) / seg;
                break;
            }
            case WL_COL2: {
                const int seg = segment_for(g.C3 + 1, E->shape.seg);
                extra[q] = seg;
                gx = col_sweep_blocks(g, 2), gz = (g.C3 + 1 + seg - 1) / seg;
                break;
            }
            case WL_WRAP: { // one thread per ghost line, looping over the job's arrays
                const int64_t tot = (int64_t)g.C2 * g.C3 + (int64_t)g.C1 * g.C2;
                gx = (int)((tot + 127) / 128);
                break;
            }
            case WL_STAGED: // tiles and chunks of planes of the staged Phase1
            case WL_STAGED_T: {
                const int nch = (g.C3 + kens - 1) / kens;     // chunks of the column, of
                const int kch = (g.C3 + nch - 1) / nch;       // balanced lengths
                const bool narrow = kind == WL_STAGED_T && narrow_tiles(g.C1);
                extra[q] = kch | (narrow ? 1 << 16 : 0);
                const dim3 gr = narrow ? stg::tile_grid<32, 8>(g, kch) : stg::staged_grid(g, kch);
                gx = (int)gr.x, gy = (int)gr.y, gz = (int)gr.z;
                break;
            }
            case WL_ZSEAMS: { // the staged lists' chunks (both tile kinds chunk alike)
                const int nch = (g.C3 + kens - 1) / kens, kch = (g.C3 + nch - 1) / nch;
                extra[q] = kch;
                gx = col_sweep_blocks(g, 2), gz = (g.C3 + kch - 1) / kch + 1;
                break;
            }
            case WL_XSEAMS: // the seam slots of the member's tile width, 128 per block
                gx = (int)((seam_slots(g, seam_width(E->shape, g)) + 127) / 128);
                break;
            }
            info[q] = make_int4(start, gx, gy, gz);
            start += gx * gy * gz;
        }
        E->total[kind] = start;
        if (!E->d_info[kind]) {
            if (int rc = ens_alloc(E, &E->d_info[kind], (size_t)E->n)) return rc;
            if (int rc = ens_alloc(E, &E->d_extra[kind], (size_t)E->n)) return rc;
        }
        ENS_CUDA(cudaMemcpy(E->d_info[kind], info.data(), sizeof(int4) * E->n, cudaMemcpyHostToDevice));
        ENS_CUDA(cudaMemcpy(E->d_extra[kind], extra.data(), sizeof(int) * E->n, cudaMemcpyHostToDevice));
    }
    if (E->d_seams) { // the tile width of each member's seams under this shape
        for (int q = 0; q < E->n; ++q) E->seams[q].tw = seam_width(E->shape, E->S[q].g);
        ENS_CUDA(cudaMemcpy(E->d_seams, E->seams.data(), sizeof(XSeams) * E->n, cudaMemcpyHostToDevice));
    }
    return ARK_OK;
}

// Ghost-fill jobs of every member for both level roles (the same arrays and modes as
// Launch<float>::wrap_con(with_ro = 0): the ensemble's Phase2 is the three sweep kernels, which
// read their x and z ghost positions from the cells and faces they stand for, so only the
// stress reads ghosts and the Phase2 ghost fill has nothing to do).
int build_jobs(ark_ensemble *E) {
    std::vector<WrapJob> jobs(2 * (size_t)E->n);
    for (int q = 0; q < E->n; ++q) {
        const DS &S = E->S[q];
        const bool px = S.k.periodic_x, pz = S.k.periodic_z;
        const uint8_t cx = px ? GH_WRAP : GH_COPY, cz = pz ? GH_WRAP : GH_COPY;
        for (int lv = 0; lv < 2; ++lv) {
            WrapJob J = {};
            const Level<float> L = S.lv[lv];
            wrap_add(J, L.u1, 0, cx, cz);
            wrap_add(J, L.u2, 0, cx, cz);
            wrap_add(J, L.u3, 0, cx, cz);
            jobs[(size_t)lv * E->n + q] = J;
        }
    }
    if (!E->d_jobs)
        if (int rc = ens_alloc(E, &E->d_jobs, jobs.size())) return rc;
    ENS_CUDA(cudaMemcpy(E->d_jobs, jobs.data(), sizeof(WrapJob) * jobs.size(), cudaMemcpyHostToDevice));
    return ARK_OK;
}

WorkList wl(const ark_ensemble *E, int kind) {
    WorkList W = {E->d_info[kind], E->d_extra[kind], E->n, E->total[kind]};
    return W;
}

int grid_of(const ark_ensemble *E, int kind) { return std::max(1, std::min(E->total[kind], E->persist)); }

// whether a shape folds the x3 sweep (shapes 6 to 9) or the x1 sweep too (8, 9) into Phase1 + stress
inline bool folds_x3(const Shape &s) { return s.march_a >= 6 && s.march_a <= 9; }
inline bool folds_x1(const Shape &s) { return s.march_a == 8 || s.march_a == 9; }

template <int MODE> void launch_p1(ark_ensemble *E, int march, int src, int dst, int fcur) {
    const dim3 blk(kTileX, kTileY);
    const bool fold = (MODE & P1_STRESS) && march >= 6 && march <= 9, fold1 = fold && march >= 8 && E->d_seams;
    if (fold) march -= march >= 8 ? 4 : 2;
    if ((march == 4 || march == 5) && E->d_maps) {
        const int kind = march == 5 ? WL_STAGED_T : WL_STAGED;
        const int grid = std::max(1, std::min(E->total[kind], E->persist_staged));
        const int m = (MODE & P1_STRESS) ? 0 : 1;
        const TmaMetas<MODE> metas = {{E->meta[0][m], E->meta[1][m]}};
        int *next = E->d_next + ((MODE & P1_STRESS) ? 0 : 1);
        bool done = false;
        if constexpr ((MODE & P1_STRESS) != 0)
            if (fold) {
                if (fold1)
                    kb_phase1_tma<MODE, 3><<<grid, dim3(stg::NT + 32), tma_ens_smem<MODE>(), E->st>>>(
                        E->d_inst, E->d_maps, metas, wl(E, kind), src, dst, fcur, next, E->d_seams);
                else
                    kb_phase1_tma<MODE, 2><<<grid, dim3(stg::NT + 32), tma_ens_smem<MODE>(), E->st>>>(
                        E->d_inst, E->d_maps, metas, wl(E, kind), src, dst, fcur, next, nullptr);
                done = true;
            }
        if (!done)
            kb_phase1_tma<MODE><<<grid, dim3(stg::NT + 32), tma_ens_smem<MODE>(), E->st>>>(E->d_inst, E->d_maps, metas,
                                                                                         wl(E, kind), src, dst, fcur, next, nullptr);
    } else if (march == 2 || march == 4 || march == 5) {
        const int grid = std::max(1, std::min(E->total[WL_STAGED], E->persist_staged));
        kb_phase1_staged<MODE><<<grid, dim3(stg::SX, stg::SY), stg::Layout<MODE>::SMEM, E->st>>>(
            E->d_inst, wl(E, WL_STAGED), src, dst, fcur);
    } else if (march == 1) {
        kb_phase1<MODE, true><<<grid_of(E, WL_TILES), blk, 0, E->st>>>(E->d_inst, wl(E, WL_TILES), src, dst, fcur);
    } else {
        kb_phase1<MODE, false><<<grid_of(E, WL_CELLS), blk, 0, E->st>>>(E->d_inst, wl(E, WL_CELLS), src, dst, fcur);
    }
}

// The staged kernels' shared-memory limits (once per process) and their resident blocks per SM.
int prepare_staged_kernels(int sms) {
    auto one = [](auto kern, int smem, int threads = stg::NT) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, threads, smem);
        return per;
    };
    int per = one(kb_phase1_staged<P1_STRESS | P1_FORCES | P1_RMAX>, stg::Layout<P1_STRESS | P1_FORCES | P1_RMAX>::SMEM);
    per = std::min(per, one(kb_phase1_staged<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>,
                            stg::Layout<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>::SMEM));
    per = std::min(per, one(kb_phase1_staged<P1_FORCES | P1_RSUM>, stg::Layout<P1_FORCES | P1_RSUM>::SMEM));
    per = std::min(per, one(kb_phase1_tma<P1_STRESS | P1_FORCES | P1_RMAX>, tma_ens_smem<P1_STRESS | P1_FORCES | P1_RMAX>(), stg::NT + 32));
    per = std::min(per, one(kb_phase1_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>,
                            tma_ens_smem<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>(), stg::NT + 32));
    per = std::min(per, one(kb_phase1_tma<P1_FORCES | P1_RSUM>, tma_ens_smem<P1_FORCES | P1_RSUM>(), stg::NT + 32));
    per = std::min(per, one(kb_phase1_tma<P1_STRESS | P1_FORCES | P1_RMAX, 2>, tma_ens_smem<P1_STRESS | P1_FORCES | P1_RMAX>(),
                            stg::NT + 32));
    per = std::min(per, one(kb_phase1_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 2>,
                            tma_ens_smem<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>(), stg::NT + 32));
    per = std::min(per, one(kb_phase1_tma<P1_STRESS | P1_FORCES | P1_RMAX, 3>, tma_ens_smem<P1_STRESS | P1_FORCES | P1_RMAX>(),
                            stg::NT + 32));
    per = std::min(per, one(kb_phase1_tma<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 3>,
                            tma_ens_smem<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>(), stg::NT + 32));
    return sms * std::max(per, 1);
}

// One step of every member (the order of main.cpp:82-91, as the single-context fused step).
// The launches of an ensemble step, in order (ark_ensemble_kernel_times reports them so).
const char *const kEnsKernels[] = {"finalize_dt", "wrap_con", "phase1_stress_forces", "sweep_x1",
                                   "sweep_x2",    "sweep_x3", "phase1_forces"};
constexpr int kEnsPhases = 7;

void ens_step(ark_ensemble *E, int x, int fc, cudaEvent_t *ev) {
    const int y = x ^ 1;
    auto mark = [&](int q) {
        if (ev) cudaEventRecord(ev[q], E->st);
    };
    cudaMemsetAsync(E->d_next, 0, 7 * sizeof(int), E->st);
    if (!ev) { // captured: the ghost fill beside dt (independent; Phase1 waits for both)
        cudaEventRecord(E->fill_fork, E->st);
        cudaStreamWaitEvent(E->fill, E->fill_fork, 0);
        kb_wrap<<<grid_of(E, WL_WRAP), 128, 0, E->fill>>>(E->d_inst, E->d_jobs + (size_t)y * E->n, wl(E, WL_WRAP));
        cudaEventRecord(E->fill_join, E->fill);
        kb_finalize<<<E->n, 1024, 0, E->st>>>(E->d_inst, 1);
        cudaStreamWaitEvent(E->st, E->fill_join, 0);
    } else { // timed one launch after the other
        kb_finalize<<<E->n, 1024, 0, E->st>>>(E->d_inst, 1);
        mark(0);
        kb_wrap<<<grid_of(E, WL_WRAP), 128, 0, E->st>>>(E->d_inst, E->d_jobs + (size_t)y * E->n, wl(E, WL_WRAP));
        mark(1);
    }
    // every member of an ensemble runs the bulk forcing or none does (checked at creation)
    if (E->K[0].forcing)
        launch_p1<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX>(E, E->shape.march_a, y, x, fc);
    else
        launch_p1<P1_STRESS | P1_FORCES | P1_RMAX>(E, E->shape.march_a, y, x, fc);
    mark(2);
    // the x3 (and x1) sweeps folded in: their seam faces (read by the second Phase1 only) beside
    // the remaining sweeps when captured, in the folded sweeps' timed slots otherwise
    const bool fold = folds_x3(E->shape) && E->d_maps, fold1 = fold && folds_x1(E->shape) && E->d_seams;
    const bool beside = fold && !ev;
    auto zseams = [&](cudaStream_t s) {
        kb_sweep_z_seams<<<grid_of(E, WL_ZSEAMS), 128, 0, s>>>(E->d_inst, wl(E, WL_ZSEAMS), y, fc, E->d_next + 5);
    };
    auto xseams = [&](cudaStream_t s) {
        kb_sweep_x_seams<<<grid_of(E, WL_XSEAMS), 128, 0, s>>>(E->d_inst, E->d_seams, wl(E, WL_XSEAMS), y, fc, E->d_next + 6);
    };
    if (beside) {
        cudaEventRecord(E->seam_fork, E->st);
        cudaStreamWaitEvent(E->fill, E->seam_fork, 0);
        if (fold1) xseams(E->fill);
        zseams(E->fill);
        cudaEventRecord(E->seam_join, E->fill);
    }
    if (!fold1) kb_sweep_x<<<grid_of(E, WL_SWEEPX), 128, 0, E->st>>>(E->d_inst, wl(E, WL_SWEEPX), y, fc, E->d_next + 2);
    else if (!beside) xseams(E->st);
    mark(3);
    kb_sweep_col<1><<<grid_of(E, WL_COL1), 128, 0, E->st>>>(E->d_inst, wl(E, WL_COL1), y, fc, E->d_next + 3);
    mark(4);
    if (!fold) kb_sweep_col<2><<<grid_of(E, WL_COL2), 128, 0, E->st>>>(E->d_inst, wl(E, WL_COL2), y, fc, E->d_next + 4);
    else if (!beside) zseams(E->st);
    if (beside) cudaStreamWaitEvent(E->st, E->seam_join, 0);
    mark(5);
    launch_p1<P1_FORCES | P1_RSUM>(E, E->shape.march_b, x, y, fc ^ 1);
    mark(6);
}

void drop_graphs(ark_ensemble *E) {
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            if (E->graph[a][b]) {
                cudaGraphExecDestroy(E->graph[a][b]);
                E->graph[a][b] = nullptr;
            }
}

int ensure_parts(ark_ensemble *E) {
    if (E->parts_valid) return ARK_OK;
    for (int q = 0; q < E->n; ++q) {
        cudaMemsetAsync(E->S[q].part_max, 0, sizeof(unsigned long long) * 3 * kBuckets, E->st);
        cudaMemsetAsync(E->S[q].part_sum, 0, sizeof(long long) * kBuckets, E->st);
    }
    kb_reduce<<<grid_of(E, WL_TILES), dim3(kTileX, kTileY), 0, E->st>>>(E->d_inst, wl(E, WL_TILES), E->con);
    ENS_CUDA(cudaGetLastError());
    E->parts_valid = true;
    return ARK_OK;
}

int ensure_graph(ark_ensemble *E) {
    const int x = E->con, fc = E->fcur;
    if (E->graph[x][fc]) return ARK_OK;
    cudaGraph_t g = nullptr;
    ENS_CUDA(cudaStreamBeginCapture(E->st, cudaStreamCaptureModeThreadLocal));
    ens_step(E, x, fc, nullptr);
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(E->st, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return efail(ARK_ERR_CUDA, std::string("ensemble capture: ") + cudaGetErrorString(le != cudaSuccess ? le : ce));
    }
    cudaError_t ie = cudaGraphInstantiate(&E->graph[x][fc], g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
        E->graph[x][fc] = nullptr;
        return efail(ARK_ERR_CUDA, std::string("ensemble graph: ") + cudaGetErrorString(ie));
    }
    return ARK_OK;
}

int check_member(ark_ensemble *E, int q) {
    if (!E) return efail(ARK_ERR_PARAM, "ensemble is NULL");
    if (q < 0 || q >= E->n) return efail(ARK_ERR_PARAM, "member index out of range");
    return ARK_OK;
}

} // namespace

extern "C" {

const char *ark_ensemble_last_error(void) { return g_ens_error.c_str(); }

ark_ensemble *ark_ensemble_create(const ark_params *params, int n, int *status) {
    int dummy;
    if (!status) status = &dummy;
    *status = ARK_ERR_PARAM;
    if (!params || n < 1) {
        efail(ARK_ERR_PARAM, "need at least one member");
        return nullptr;
    }
    for (int q = 0; q < n; ++q) {
        const ark_params &p = params[q];
        if (p.precision != ARK_FP32) {
            *status = efail(ARK_ERR_UNSUPPORTED, "ensemble members are FP32 contexts");
            return nullptr;
        }
        if (p.n1_cells < 1 || p.n2_cells < 1 || p.n3_cells < 1 || !(p.sound > 0) || !(p.ro0 > 0) || !(p.cfl > 0) ||
            !(p.vis >= 0) || !(p.lx > 0) || !(p.ly > 0) || !(p.lz > 0) || p.device != params[0].device ||
            p.forcing != params[0].forcing) {
            efail(ARK_ERR_PARAM, "bad member parameters (or members on different devices / forcing modes)");
            return nullptr;
        }
        if (p.n1_cells > (1 << 28) ||
            (double)device_pitch(p.n1_cells) * (p.n2_cells + 3) * (p.n3_cells + 3) >= 2147483647.0) {
            efail(ARK_ERR_PARAM, "member grid too large for 32-bit indexing");
            return nullptr;
        }
    }
    if (cudaSetDevice(params[0].device) != cudaSuccess) {
        *status = efail(ARK_ERR_CUDA, "cudaSetDevice failed");
        return nullptr;
    }
    std::unique_ptr<ark_ensemble> E(new ark_ensemble());
    E->n = n;
    E->P.assign(params, params + n);
    E->S.resize(n);
    E->K.resize(n);
    E->cond_host.resize(n);
    E->uploaded.assign(n, 0);
    size_t maxf = 0;
    for (int q = 0; q < n; ++q) {
        E->K[q] = make_run_consts(params[q]);
        DS &S = E->S[q];
        std::memset(&S, 0, sizeof(S));
        S.g = geom_of(params[q]);
        S.k = E->K[q];
        if ((*status = alloc_member(E.get(), S))) return nullptr;
        maxf = std::max(maxf, (size_t)S.g.nface());
    }
    if ((*status = ens_alloc(E.get(), &E->d_inst, (size_t)n))) return nullptr;
    if (cudaMemcpy(E->d_inst, E->S.data(), sizeof(DS) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
        *status = efail(ARK_ERR_CUDA, "member table copy failed");
        return nullptr;
    }
    if ((*status = ens_alloc(E.get(), &E->stage, maxf))) return nullptr;
    { // the members' seam arrays for the folded x1 sweep (slots for any tile width; build_lists sets tw)
        size_t tot = 0;
        for (int q = 0; q < n; ++q) tot += 20 * (size_t)seam_slots(E->S[q].g, 32);
        float *pool = nullptr;
        if ((*status = ens_alloc(E.get(), &pool, tot))) return nullptr;
        E->seams.assign(n, XSeams{});
        size_t off = 0;
        for (int q = 0; q < n; ++q) {
            const size_t ns = (size_t)seam_slots(E->S[q].g, 32);
            XSeams &X = E->seams[q];
            for (int a = 0; a < 8; ++a) X.b[a] = pool + off + a * ns;
            for (int a = 0; a < 12; ++a) X.a[a] = pool + off + (8 + a) * ns;
            X.n = (int)ns;
            X.tw = 64;
            off += 20 * ns;
        }
        if ((*status = ens_alloc(E.get(), &E->d_seams, (size_t)n))) return nullptr;
    }
    if (cudaStreamCreateWithFlags(&E->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&E->fill, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&E->fill_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&E->fill_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&E->seam_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&E->seam_join, cudaEventDisableTiming) != cudaSuccess) {
        *status = efail(ARK_ERR_CUDA, "stream creation failed");
        return nullptr;
    }
    int dev = params[0].device, sms = 152, per = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kb_phase1<P1_FORCES | P1_RSUM, false>, kTileX * kTileY, 0);
    E->persist = sms * std::max(per, 1) * 2;
    E->persist_staged = prepare_staged_kernels(sms);
    stg::encode_tiled(); // looked up here, outside any stream capture
    if ((*status = build_lists(E.get())) || (*status = build_jobs(E.get())) || (*status = build_maps(E.get())) ||
        (*status = ens_alloc(E.get(), &E->d_next, 7)))
        return nullptr;
    cudaEventCreate(&E->ev0);
    cudaEventCreate(&E->ev1);
    *status = ARK_OK;
    return E.release();
}

int ark_ensemble_destroy(ark_ensemble *E) {
    if (!E) return ARK_OK;
    cudaStreamSynchronize(E->st);
    drop_graphs(E);
    for (void *p : E->allocs) cudaFree(p);
    if (E->ev0) cudaEventDestroy(E->ev0);
    if (E->ev1) cudaEventDestroy(E->ev1);
    if (E->st) cudaStreamDestroy(E->st);
    if (E->fill) {
        cudaStreamSynchronize(E->fill);
        cudaStreamDestroy(E->fill);
    }
    if (E->fill_fork) cudaEventDestroy(E->fill_fork);
    if (E->fill_join) cudaEventDestroy(E->fill_join);
    if (E->seam_fork) cudaEventDestroy(E->seam_fork);
    if (E->seam_join) cudaEventDestroy(E->seam_join);
    delete E;
    return ARK_OK;
}

int ark_ensemble_size(const ark_ensemble *E) { return E ? E->n : 0; }

int ark_ensemble_upload(ark_ensemble *E, int q, const ark_host_state *h) {
    if (int rc = check_member(E, q)) return rc;
    if (!h) return efail(ARK_ERR_PARAM, "host state is NULL");
    double *cells[8] = {h->roCon, h->u1Con, h->u2Con, h->u3Con, h->ronCon, h->u1nCon, h->u2nCon, h->u3nCon};
    double *faces[3][4] = {{h->p1, h->u11, h->u21, h->u31}, {h->p2, h->u12, h->u22, h->u32}, {h->p3, h->u13, h->u23, h->u33}};
    for (double *a : cells)
        if (!a) return efail(ARK_ERR_PARAM, "NULL cell array");
    for (auto &d : faces)
        for (double *a : d)
            if (!a) return efail(ARK_ERR_PARAM, "NULL face array");
    if (!h->condition) return efail(ARK_ERR_PARAM, "NULL condition");
    ENS_CUDA(cudaStreamSynchronize(E->st));
    DS &S = E->S[q];
    const size_t nc = (size_t)S.g.ncell(), nf = (size_t)S.g.nface();
    const double ro0 = E->P[q].ro0;
    // into the current roles of the levels and the current face generation (shared by all
    // members)
    const int lc = E->con, ln = E->con ^ 1;
    float *dcell[8] = {S.lv[lc].ro, S.lv[lc].u1, S.lv[lc].u2, S.lv[lc].u3,
                       S.lv[ln].ro, S.lv[ln].u1, S.lv[ln].u2, S.lv[ln].u3};
    for (int a = 0; a < 8; ++a) {
        const RowShape r = row_shape(S.g, 0);
        ENS_CUDA(cudaMemcpyAsync(E->stage, cells[a], sizeof(double) * r.w * r.rows, cudaMemcpyHostToDevice, E->st));
        rows_from_double<float>(dcell[a], E->stage, r.w, r.rows, r.pitch, (a % 4 == 0) ? ro0 : 0.0, E->st);
        ENS_CUDA(cudaStreamSynchronize(E->st));
    }
    for (int d = 0; d < 3; ++d) {
        const FaceSet<float> &F = S.fc[E->fcur][d];
        float *df[4] = {F.p, F.u[0], F.u[1], F.u[2]};
        for (int a = 0; a < 4; ++a) {
            const RowShape r = row_shape(S.g, 1);
            ENS_CUDA(cudaMemcpyAsync(E->stage, faces[d][a], sizeof(double) * r.w * r.rows, cudaMemcpyHostToDevice, E->st));
            rows_from_double<float>(df[a], E->stage, r.w, r.rows, r.pitch, 0.0, E->st);
            ENS_CUDA(cudaStreamSynchronize(E->st));
        }
    }
    const Geom hg = host_geom(S.g.C1, S.g.C2, S.g.C3);
    const size_t hnc = (size_t)hg.ncell();
    E->cond_host[q].assign(h->condition, h->condition + hnc);
    std::vector<uint8_t> fl(hnc);
    long long nfluid = 0;
    for (size_t c = 0; c < hnc; ++c) {
        const double v = h->condition[c];
        fl[c] = (uint8_t)((v < 0.5 ? FL_LT : 0) | (v > 0.5 ? FL_GT : 0) | (v == 0 ? FL_EQ0 : 0));
    }
    for (int k = 1; k <= hg.C3; ++k)
        for (int j = 1; j <= hg.C2; ++j)
            for (int i = 1; i <= hg.C1; ++i)
                if (fl[(size_t)hg.cell(i, j, k)] & FL_EQ0) ++nfluid;
    ENS_CUDA(copy_rows(S.flags, fl.data(), S.g, 0, 1, cudaMemcpyHostToDevice, E->st));
    ENS_CUDA(cudaStreamSynchronize(E->st));
    DevScalars sc;
    std::memset(&sc, 0, sizeof(sc));
    sc.nfluid = nfluid;
    ENS_CUDA(cudaMemcpy(S.sc, &sc, sizeof(sc), cudaMemcpyHostToDevice));
    E->uploaded[q] = 1;
    E->parts_valid = false;
    return ARK_OK;
}

int ark_ensemble_download(ark_ensemble *E, int q, ark_host_state *h) {
    if (int rc = check_member(E, q)) return rc;
    if (!h) return efail(ARK_ERR_PARAM, "host state is NULL");
    ENS_CUDA(cudaStreamSynchronize(E->st));
    DS &S = E->S[q];
    const size_t nc = (size_t)S.g.ncell(), nf = (size_t)S.g.nface();
    const double ro0 = E->P[q].ro0;
    const int c = E->con, n = E->con ^ 1, fc = E->fcur;
    double *cells[8] = {h->roCon, h->u1Con, h->u2Con, h->u3Con, h->ronCon, h->u1nCon, h->u2nCon, h->u3nCon};
    float *dcell[8] = {S.lv[c].ro, S.lv[c].u1, S.lv[c].u2, S.lv[c].u3, S.lv[n].ro, S.lv[n].u1, S.lv[n].u2, S.lv[n].u3};
    for (int a = 0; a < 8; ++a) {
        if (!cells[a]) continue;
        const RowShape r = row_shape(S.g, 0);
        rows_to_double<float>(E->stage, dcell[a], r.w, r.rows, r.pitch, (a % 4 == 0) ? ro0 : 0.0, E->st);
        ENS_CUDA(cudaMemcpyAsync(cells[a], E->stage, sizeof(double) * r.w * r.rows, cudaMemcpyDeviceToHost, E->st));
        ENS_CUDA(cudaStreamSynchronize(E->st));
    }
    double *faces[3][5] = {{h->p1, h->ro1, h->u11, h->u21, h->u31},
                           {h->p2, h->ro2, h->u12, h->u22, h->u32},
                           {h->p3, h->ro3, h->u13, h->u23, h->u33}};
    for (int d = 0; d < 3; ++d) {
        const FaceSet<float> &F = S.fc[fc][d];
        const float *df[5] = {F.p, nullptr, F.u[0], F.u[1], F.u[2]};
        for (int a = 0; a < 5; ++a) {
            if (!faces[d][a]) continue;
            const RowShape r = row_shape(S.g, 1);
            if (a == 1) rows_face_density<float>(E->stage, F.p, r.w, r.rows, r.pitch, E->K[q].ro0, E->K[q].rc2, E->st);
            else rows_to_double<float>(E->stage, df[a], r.w, r.rows, r.pitch, 0.0, E->st);
            ENS_CUDA(cudaMemcpyAsync(faces[d][a], E->stage, sizeof(double) * r.w * r.rows, cudaMemcpyDeviceToHost, E->st));
            ENS_CUDA(cudaStreamSynchronize(E->st));
        }
    }
    if (h->condition) std::memcpy(h->condition, E->cond_host[q].data(), sizeof(double) * E->cond_host[q].size());
    return ARK_OK;
}

int ark_ensemble_step(ark_ensemble *E, int nsteps) {
    if (!E) return efail(ARK_ERR_PARAM, "ensemble is NULL");
    for (char u : E->uploaded)
        if (!u) return efail(ARK_ERR_STATE, "every member needs a state before stepping");
    if (nsteps < 0) return efail(ARK_ERR_PARAM, "nsteps < 0");
    if (int rc = ensure_parts(E)) return rc;
    for (int s = 0; s < nsteps; ++s) {
        if (int rc = ensure_graph(E)) return rc;
        ENS_CUDA(cudaGraphLaunch(E->graph[E->con][E->fcur], E->st));
        E->fcur ^= 1;
    }
    return ARK_OK;
}

int ark_ensemble_sync(ark_ensemble *E) {
    if (!E) return efail(ARK_ERR_PARAM, "ensemble is NULL");
    ENS_CUDA(cudaStreamSynchronize(E->st));
    for (int q = 0; q < E->n; ++q) {
        int status = 0;
        ENS_CUDA(cudaMemcpy(&status, &E->S[q].sc->status, sizeof(int), cudaMemcpyDeviceToHost));
        if (status & STATUS_NONFINITE) return efail(ARK_ERR_NONFINITE, "non-finite velocity in member " + std::to_string(q));
    }
    return ARK_OK;
}

int ark_ensemble_time_steps(ark_ensemble *E, int nsteps, double *ms) {
    if (!E || !ms) return efail(ARK_ERR_PARAM, "NULL argument");
    if (int rc = ensure_parts(E)) return rc;
    if (int rc = ensure_graph(E)) return rc;
    E->fcur ^= 1;
    int rc2 = ensure_graph(E);
    E->fcur ^= 1;
    if (rc2) return rc2;
    ENS_CUDA(cudaStreamSynchronize(E->st));
    ENS_CUDA(cudaEventRecord(E->ev0, E->st));
    if (int rc = ark_ensemble_step(E, nsteps)) return rc;
    ENS_CUDA(cudaEventRecord(E->ev1, E->st));
    ENS_CUDA(cudaEventSynchronize(E->ev1));
    float f = 0.f;
    ENS_CUDA(cudaEventElapsedTime(&f, E->ev0, E->ev1));
    *ms = (double)f;
    return ark_ensemble_sync(E);
}

// The launches of a step in the order ark_kernel_name lists them (the same eight phases as
// the single-context step), each timed with events around it, averaged over nsteps.
const char *ark_ensemble_kernel_name(int index) {
    return index >= 0 && index < kEnsPhases ? kEnsKernels[index] : nullptr;
}
// The same for the ensemble's current shape (with the x3 sweep folded in, its seam kernel in the
// x3 sweep's place).
const char *ark_ensemble_step_kernel_name(const ark_ensemble *E, int index) {
    if (!E || index < 0 || index >= kEnsPhases) return nullptr;
    if (folds_x1(E->shape) && (index == 2 || index == 3)) return index == 2 ? "phase1_stress_sweep_x1_x3" : "sweep_x1_seams";
    if (folds_x3(E->shape) && (index == 2 || index == 5)) return index == 2 ? "phase1_stress_sweep_x3" : "sweep_x3_seams";
    return kEnsKernels[index];
}

int ark_ensemble_kernel_times(ark_ensemble *E, int nsteps, double *ms, int cap, int *count) {
    constexpr int kPhases = kEnsPhases;
    if (!E || !ms || !count || nsteps < 1) return efail(ARK_ERR_PARAM, "bad arguments");
    for (char u : E->uploaded)
        if (!u) return efail(ARK_ERR_STATE, "every member needs a state before stepping");
    *count = kPhases;
    if (int rc = ensure_parts(E)) return rc;
    cudaEvent_t ev[kPhases + 1] = {};
    for (auto &e : ev) ENS_CUDA(cudaEventCreate(&e));
    double acc[kPhases] = {};
    cudaError_t err = cudaSuccess;
    for (int s = 0; s < nsteps && err == cudaSuccess; ++s) {
        cudaEventRecord(ev[0], E->st);
        ens_step(E, E->con, E->fcur, ev + 1);
        E->fcur ^= 1;
        err = cudaGetLastError();
        if (err == cudaSuccess) err = cudaEventSynchronize(ev[kPhases]);
        for (int q = 0; q < kPhases && err == cudaSuccess; ++q) {
            float f = 0.f;
            cudaEventElapsedTime(&f, ev[q], ev[q + 1]);
            acc[q] += f;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (err != cudaSuccess) return efail(ARK_ERR_CUDA, std::string("kernel times: ") + cudaGetErrorString(err));
    for (int q = 0; q < kPhases && q < cap; ++q) ms[q] = acc[q] / nsteps;
    return ark_ensemble_sync(E);
}

int ark_ensemble_get_scalars(ark_ensemble *E, int q, ark_scalars *out) {
    if (int rc = check_member(E, q)) return rc;
    if (!out) return efail(ARK_ERR_PARAM, "out is NULL");
    DevScalars sc;
    ENS_CUDA(cudaStreamSynchronize(E->st));
    ENS_CUDA(cudaMemcpy(&sc, E->S[q].sc, sizeof(sc), cudaMemcpyDeviceToHost));
    out->dt = sc.dt;
    out->time = sc.time;
    out->nstep = sc.nstep;
    out->bulk_velocity = sc.ub;
    out->bulk_force = sc.G;
    return ARK_OK;
}

int ark_ensemble_mean_profile(ark_ensemble *E, int q, double *mean_u1, double *wall_shear) {
    if (int rc = check_member(E, q)) return rc;
    if (!mean_u1) return efail(ARK_ERR_PARAM, "mean_u1 is NULL");
    const DS &S = E->S[q];
    const int n = S.g.C2;
    long long *acc = nullptr;
    ENS_CUDA(cudaMalloc(&acc, sizeof(long long) * 2 * n));
    Launch<float>::mean_profile(S, E->con ^ 1, acc, E->st);
    std::vector<long long> h(2 * (size_t)n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(E->st);
    if (e == cudaSuccess) e = cudaMemcpy(h.data(), acc, sizeof(long long) * 2 * n, cudaMemcpyDeviceToHost);
    cudaFree(acc);
    if (e != cudaSuccess) return efail(ARK_ERR_CUDA, std::string("profile: ") + cudaGetErrorString(e));
    for (int j = 0; j < n; ++j)
        mean_u1[j] = h[2 * j + 1] > 0 ? ((double)h[2 * j] * (1.0 / 4294967296.0)) / (double)h[2 * j + 1] : 0.0;
    if (wall_shear) {
        wall_shear[0] = 2 * E->P[q].vis * mean_u1[0] / S.k.dx[1];
        wall_shear[1] = 2 * E->P[q].vis * mean_u1[n - 1] / S.k.dx[1];
    }
    return ARK_OK;
}

// Times every candidate shape for steps_per_candidate steps on the live state (the results do
// not depend on the shape) and keeps the fastest.  choice (4 ints, may be NULL) receives the
// chosen {march_a, march_b, segment target, ms per step x 1000}.
int ark_ensemble_autotune(ark_ensemble *E, int steps_per_candidate, int *choice) {
    if (!E) return efail(ARK_ERR_PARAM, "ensemble is NULL");
    if (steps_per_candidate < 1) return efail(ARK_ERR_PARAM, "steps_per_candidate < 1");
    for (char u : E->uploaded)
        if (!u) return efail(ARK_ERR_STATE, "every member needs a state before tuning");
    const Shape cands[] = {{1, 0, 32}, {0, 0, 32}, {1, 1, 32}, {0, 1, 32}, {1, 0, 16}, {1, 0, 64}, {0, 0, 16},
                           {0, 0, 64}, {2, 2, 32}, {2, 0, 32}, {0, 2, 32}, {2, 2, 64}, {2, 0, 64}, {4, 4, 32},
                           {4, 4, 64}, {4, 4, 16}, {4, 2, 32}, {2, 4, 32}, {4, 0, 32}, {5, 5, 32}, {5, 4, 32},
                           {4, 5, 32}, {5, 5, 64}, {7, 5, 32}, {6, 4, 32}, {7, 4, 32}, {6, 5, 32}, {7, 5, 16},
                           {7, 5, 64}, {9, 5, 32}, {8, 4, 32}, {9, 4, 32}, {9, 5, 64}};
    Shape best = E->shape;
    double best_ms = 1e300;
    if (int rc = ensure_parts(E)) return rc;
    for (const Shape &c : cands) {
        E->shape = c;
        if (int rc = build_lists(E)) return rc;
        drop_graphs(E);
        // one untimed step to build both graphs, then the timed ones
        if (int rc = ark_ensemble_step(E, 2)) return rc;
        double ms = 0;
        if (int rc = ark_ensemble_time_steps(E, steps_per_candidate, &ms)) return rc;
        if (ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    E->shape = best;
    drop_graphs(E);
    if (int rc = build_lists(E)) return rc;
    if (choice) {
        choice[0] = best.march_a;
        choice[1] = best.march_b;
        choice[2] = best.seg;
        choice[3] = (int)(1000.0 * best_ms / steps_per_candidate);
    }
    return ARK_OK;
}

int ark_ensemble_set_shape(ark_ensemble *E, int march_a, int march_b, int segment) {
    if (!E) return efail(ARK_ERR_PARAM, "ensemble is NULL");
    if (segment < 1) return efail(ARK_ERR_PARAM, "segment < 1");
    auto ok = [](int m) { return (m >= 0 && m <= 2) || m == 4 || m == 5; };
    if (!(ok(march_a) || (march_a >= 6 && march_a <= 9)) || !ok(march_b))
        return efail(ARK_ERR_PARAM, "march must be 0, 1, 2, 4 or 5 (and 6 to 9 for the Phase1 with stress)");
    E->shape = Shape{march_a, march_b, segment};
    drop_graphs(E);
    return build_lists(E);
}

} // extern "C"
