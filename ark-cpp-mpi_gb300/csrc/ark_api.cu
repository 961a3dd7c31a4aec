// C ABI of the GB300 CABARET step (include/ark_gpu.h): context, state transfer, the
// reference's step pieces and the fused, graph-captured time step.
#include <cuda_runtime.h>

#include <fcntl.h>
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/ark_gpu.h"
#include "ark_check.cuh"
#include "ark_ctx.h"

using namespace ark;

namespace {

thread_local std::string g_last_error;

int fail(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}

#define ARK_CUDA(call)                                                                            \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(e_ == cudaErrorMemoryAllocation ? ARK_ERR_NOMEM : ARK_ERR_CUDA,           \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                      \
    } while (0)

// Field names of the host state, in struct order, and whether each is a face array.
struct FieldRef {
    const char *name;
    double *ark_host_state::*member;
    int face;
};
const FieldRef kFields[] = {
    {"roCon", &ark_host_state::roCon, 0},   {"u1Con", &ark_host_state::u1Con, 0},
    {"u2Con", &ark_host_state::u2Con, 0},   {"u3Con", &ark_host_state::u3Con, 0},
    {"ronCon", &ark_host_state::ronCon, 0}, {"u1nCon", &ark_host_state::u1nCon, 0},
    {"u2nCon", &ark_host_state::u2nCon, 0}, {"u3nCon", &ark_host_state::u3nCon, 0},
    {"condition", &ark_host_state::condition, 0},
    {"p1", &ark_host_state::p1, 1},  {"ro1", &ark_host_state::ro1, 1}, {"u11", &ark_host_state::u11, 1},
    {"u21", &ark_host_state::u21, 1}, {"u31", &ark_host_state::u31, 1},
    {"p2", &ark_host_state::p2, 1},  {"ro2", &ark_host_state::ro2, 1}, {"u12", &ark_host_state::u12, 1},
    {"u22", &ark_host_state::u22, 1}, {"u32", &ark_host_state::u32, 1},
    {"p3", &ark_host_state::p3, 1},  {"ro3", &ark_host_state::ro3, 1}, {"u13", &ark_host_state::u13, 1},
    {"u23", &ark_host_state::u23, 1}, {"u33", &ark_host_state::u33, 1},
};

Geom make_geom(const ark_params &p) { return device_geom(p.n1_cells, p.n2_cells, p.n3_cells); }

template <class T> void fill_kt(const Consts &k, KT<T> &t) {
    for (int d = 0; d < 3; ++d) {
        t.dx[d] = (T)k.dx[d];
        t.rdx[d] = (T)k.rdx[d];
        t.vrdx[d] = (T)(k.vis * k.rdx[d]);
        t.ds[d] = (T)k.ds[d];
    }
    t.dvc = (T)k.dvc;
    t.rdvc = (T)(1.0 / k.dvc);
    t.vis = (T)k.vis;
    t.two_vis = (T)k.two_vis;
    t.sound = (T)k.sound;
    t.ro0 = (T)k.ro0;
    t.c2 = (T)k.c2;
    t.rc2 = (T)k.rc2;
    t.roc = (T)k.roc;
    t.rroc = (T)k.rroc;
    for (int d = 0; d < 3; ++d) t.q_dx[d] = make_qrecip(k.dx[d]);
    t.q_dvc = make_qrecip(k.dvc);
    t.q_roc = make_qrecip(k.roc);
    t.q_c2 = make_qrecip(k.c2);
}

// Run constants, evaluated exactly as the reference evaluates them: grid steps as
// InitializeData forms them (main.cpp:284-290, domain [0,lx] x [-ly/2,ly/2] x [0,lz]),
// areas and volume as Phase1 (main.cpp:456-462), dt numerators as TimeStepSize.
Consts make_consts(const ark_params &p) {
    Consts k;
    k.dx[0] = (p.lx - 0.) / (double)p.n1_cells;
    k.dx[1] = (0.5 * p.ly - -0.5 * p.ly) / (double)p.n2_cells;
    k.dx[2] = (p.lz - 0.) / (double)p.n3_cells;
    for (int d = 0; d < 3; ++d) {
        k.rdx[d] = 1.0 / k.dx[d];
        k.cfl_dx[d] = p.cfl * k.dx[d];
    }
    k.ds[0] = k.dx[1] * k.dx[2];
    k.ds[1] = k.dx[0] * k.dx[2];
    k.ds[2] = k.dx[0] * k.dx[1];
    k.dvc = k.dx[0] * k.dx[1] * k.dx[2];
    k.vis = p.vis;
    k.two_vis = 2 * p.vis;
    k.sound = p.sound;
    k.ro0 = p.ro0;
    k.c2 = p.sound * p.sound;
    k.rc2 = 1.0 / k.c2;
    k.roc = p.ro0 * p.sound;
    k.rroc = 1.0 / k.roc;
    if (p.vis > 1e-16) {
        const double dtv1 = p.cfl * k.dx[0] * k.dx[0] / (2. * p.vis);
        const double dtv2 = p.cfl * k.dx[1] * k.dx[1] / (2. * p.vis);
        const double dtv3 = p.cfl * k.dx[2] * k.dx[2] / (2. * p.vis);
        double m = dtv1 > dtv2 ? dtv2 : dtv1;
        k.dtv = m > dtv3 ? dtv3 : m;
    } else {
        k.dtv = 1e16;
    }
    k.u_target = p.u_target;
    k.forcing = p.forcing;
    k.periodic_x = p.periodic_x != 0;
    k.periodic_z = p.periodic_z != 0;
    k.ext_z = 0;
    fill_kt(k, k.kd);
    fill_kt(k, k.kf);
    return k;
}

// The launches of one fused step, in order (ark_kernel_times reports them in this order).
const char *const kStepKernels[] = {"finalize_dt", "wrap_con", "phase1_stress_forces", "wrap_phase2",
                                    "sweep_x1",    "sweep_x2", "sweep_x3",             "phase1_forces"};
constexpr int kNumStepKernels = 8;

} // namespace

namespace ark {
// Run constants of a parameter set (shared with the ensemble code).
Consts make_run_consts(const ark_params &p) { return make_consts(p); }
int api_fail(int status, const std::string &msg) { return fail(status, msg); }

// The bounds-check records of the translation units built with -DARK_CHECK (none otherwise).
static std::vector<CheckReader> &check_readers() {
    static std::vector<CheckReader> r;
    return r;
}
int check_register(CheckReader reader) {
    check_readers().push_back(reader);
    return (int)check_readers().size();
}
} // namespace ark

extern "C" int ark_bounds_check(int reset, long long *out) {
    if (!out) return fail(ARK_ERR_PARAM, "out is NULL");
    if (ark::check_readers().empty())
        return fail(ARK_ERR_UNSUPPORTED, "not a bounds-checked build (compile with -DARK_CHECK)");
    out[0] = out[1] = out[2] = out[3] = 0;
    if (cudaError_t e = cudaDeviceSynchronize()) return fail(ARK_ERR_CUDA, std::string("ark_bounds_check: ") + cudaGetErrorString(e));
    for (ark::CheckReader r : ark::check_readers()) {
        ark::CheckRecord c;
        if (r(&c, reset)) return fail(ARK_ERR_CUDA, "could not read a bounds-check record");
        if (c.hits && !out[0]) {
            out[1] = c.value;
            out[2] = c.bound;
            out[3] = c.line;
        }
        out[0] += (long long)c.hits;
    }
    return ARK_OK;
}

namespace {

// up to four destinations of get_block
template <class T> struct U_ptrs {
    T **p[4];
    T **&operator[](int q) { return p[q]; }
};

// The device address of a page-locked (cudaHostAlloc / cudaHostRegister) host array, which
// kernels may read and write in place; null for pageable memory.
static const void *mapped_host(const void *host) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError(); // pageable memory on older drivers: not an error of the caller's
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// The flag bits of every cell from the condition array (host layout hg, device memory) into the
// padded device rows (dg), and the count of interior fluid cells (condition == 0) into *nfluid
// (atomic integer adds: the count does not depend on their order).
__global__ void k_condition_flags(const double *__restrict__ cond, uint8_t *__restrict__ flags, Geom hg, Geom dg,
                                  unsigned long long *nfluid) {
    __shared__ unsigned int cnt;
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    const int64_t n = hg.ncell(), plane = hg.cs2;
    unsigned int mine = 0;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(c / plane), rem = (int)(c - (int64_t)k * plane);
        const int j = rem / (int)hg.cs1, i = rem - j * (int)hg.cs1;
        const double v = cond[c];
        const uint8_t f = (uint8_t)((v < 0.5 ? FL_LT : 0) | (v > 0.5 ? FL_GT : 0) | (v == 0 ? FL_EQ0 : 0));
        flags[dg.cell(i, j, k)] = f;
        if ((f & FL_EQ0) && i >= 1 && i <= hg.C1 && j >= 1 && j <= hg.C2 && k >= 1 && k <= hg.C3) ++mine;
    }
    if (mine) atomicAdd(&cnt, mine);
    __syncthreads();
    if (threadIdx.x == 0 && cnt) atomicAdd(nfluid, (unsigned long long)cnt);
}

template <class T> struct EngineT : Engine {
    ark_ctx *ctx;
    DevState<T> S;
    XSeams seams = {};   // FP32: the folded x1 sweep's tile seams (Phase2 form 4)
    std::vector<void *> allocs;

    explicit EngineT(ark_ctx *c) : ctx(c) { std::memset(&S, 0, sizeof(S)); }
    ~EngineT() override {
        for (void *p : allocs) cudaFree(p);
    }

    template <class U> int get(U **out, size_t n) {
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, n * sizeof(U));
        if (e != cudaSuccess) return fail(ARK_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        allocs.push_back(p);
        cudaMemset(p, 0, n * sizeof(U));
        *out = (U *)p;
        return ARK_OK;
    }

    // n arrays of `each` elements in one allocation, array q at out[q] = base + q * each (the
    // staged Phase1 reads a level's four arrays, a face set's four or the three forces as one
    // 4-D tensor: arrays a fixed stride apart)
    int get_block(U_ptrs<T> out, int n, size_t each) {
        T *base = nullptr;
        if (int rc = get(&base, each * n)) return rc;
        for (int q = 0; q < n; ++q) *out[q] = base + each * q;
        return ARK_OK;
    }

    int alloc() override {
        S.g = ctx->g;
        S.k = ctx->k;
        const size_t nc = (size_t)S.g.ncell(), nf = (size_t)S.g.nface();
        int rc = 0;
        for (int l = 0; l < 2; ++l) rc |= get_block({&S.lv[l].ro, &S.lv[l].u1, &S.lv[l].u2, &S.lv[l].u3}, 4, nc);
        if (Storage<T>::deviation) { // FP32: the level the one-kernel Phase2 + second Phase1 writes
            rc |= get_block({&S.spare.ro, &S.spare.u1, &S.spare.u2, &S.spare.u3}, 4, nc);
            // the seam arrays of Phase1 + stress with the x1 sweep folded in (any tile width)
            const size_t ns = (size_t)seam_slots(S.g, 32);
            float *sb = nullptr;
            rc |= get(&sb, 20 * ns);
            if (sb) {
                for (int q = 0; q < 8; ++q) seams.b[q] = sb + q * ns;
                for (int q = 0; q < 12; ++q) seams.a[q] = sb + (8 + q) * ns;
                seams.n = (int)ns;
            }
        }
        rc |= get_block({&S.f[0], &S.f[1], &S.f[2], nullptr}, 3, nc);
        for (int gen = 0; gen < 2; ++gen)
            for (int d = 0; d < 3; ++d) {
                FaceSet<T> &F = S.fc[gen][d];
                rc |= get_block({&F.p, &F.u[0], &F.u[1], &F.u[2]}, 4, nf);
                if (Storage<T>::deviation) F.ro = nullptr; // derived from p
                else rc |= get(&F.ro, nf);
            }
        for (int d = 0; d < 3; ++d)
            for (int m = 0; m < 3; ++m) {
                if (ctx->P.keep_stress) rc |= get(&S.sig[d][m], nf);
                else S.sig[d][m] = nullptr;
            }
        rc |= get(&S.flags, nc);
        rc |= get(&S.sc, 1);
        rc |= get(&S.part_max, 3 * (size_t)kBuckets);
        rc |= get(&S.part_sum, (size_t)kBuckets);
        if (rc) return ARK_ERR_NOMEM;
        return ARK_OK;
    }

    // which: index into kFields (0..23), levels resolved through ctx->con
    T *dev_of(int which) {
        const int con = ctx->con, ncon = con ^ 1;
        switch (which) {
        case 0: return S.lv[con].ro;
        case 1: return S.lv[con].u1;
        case 2: return S.lv[con].u2;
        case 3: return S.lv[con].u3;
        case 4: return S.lv[ncon].ro;
        case 5: return S.lv[ncon].u1;
        case 6: return S.lv[ncon].u2;
        case 7: return S.lv[ncon].u3;
        default: break;
        }
        if (which >= 9 && which < 24) {
            const int d = (which - 9) / 5, v = (which - 9) % 5;
            FaceSet<T> &F = S.fc[ctx->fcur][d];
            return v == 0 ? F.p : v == 1 ? F.ro : F.u[v - 2];
        }
        return nullptr;
    }

    // Host arrays in the Arr3d layout <-> device arrays with padded rows, through the contiguous
    // double staging buffer: one plain copy across the bus, then a kernel moves the rows (and
    // converts for FP32 contexts, whose density fields hold rho - ro0).
    // A page-locked host array is read or written in place by the row kernels over the host
    // link (one pass); pageable memory goes through the device staging buffer.
    int copy_in(T *dev, const double *host, int face, double offset) {
        const RowShape r = row_shape(S.g, face);
        const double *m = (const double *)mapped_host(host);
        if (m && ((uintptr_t)m & 15) == 0) {
            flat_from_host<T>(dev, m, r.w, r.rows, r.pitch, offset, ctx->st);
        } else if (m) {
            rows_from_double<T>(dev, m, r.w, r.rows, r.pitch, offset, ctx->st);
        } else {
            ARK_CUDA(cudaMemcpyAsync(ctx->stage, host, sizeof(double) * r.w * r.rows, cudaMemcpyHostToDevice, ctx->st));
            rows_from_double<T>(dev, ctx->stage, r.w, r.rows, r.pitch, offset, ctx->st);
        }
        ARK_CUDA(cudaStreamSynchronize(ctx->st));
        return ARK_OK;
    }

    int copy_out(double *host, const T *dev, int face, double offset) {
        const RowShape r = row_shape(S.g, face);
        double *m = (double *)mapped_host(host);
        if (m && ((uintptr_t)m & 15) == 0) {
            flat_to_host<T>(m, dev, r.w, r.rows, r.pitch, offset, ctx->st);
        } else if (m) {
            rows_to_double<T>(m, dev, r.w, r.rows, r.pitch, offset, ctx->st);
        } else {
            rows_to_double<T>(ctx->stage, dev, r.w, r.rows, r.pitch, offset, ctx->st);
            ARK_CUDA(cudaMemcpyAsync(host, ctx->stage, sizeof(double) * r.w * r.rows, cudaMemcpyDeviceToHost, ctx->st));
        }
        ARK_CUDA(cudaStreamSynchronize(ctx->st));
        return ARK_OK;
    }

    static bool is_cell_density(int which) { return which == 0 || which == 4; }
    static bool is_face_density(int which) { return which >= 9 && which < 24 && (which - 9) % 5 == 1; }

    int upload_field(int which, int face, const double *host) override {
        if (Storage<T>::deviation && is_face_density(which)) return ARK_OK; // derived from p
        const double off = (Storage<T>::deviation && is_cell_density(which)) ? ctx->P.ro0 : 0.0;
        return copy_in(dev_of(which), host, face, off);
    }
    int download_field(int which, int face, double *host) override {
        if (Storage<T>::deviation && is_face_density(which)) {
            const int d = (which - 9) / 5;
            const RowShape r = row_shape(S.g, 1);
            double *m = (double *)mapped_host(host);
            rows_face_density<T>(m ? m : ctx->stage, S.fc[ctx->fcur][d].p, r.w, r.rows, r.pitch, ctx->k.ro0, ctx->k.rc2,
                                 ctx->st);
            if (!m)
                ARK_CUDA(cudaMemcpyAsync(host, ctx->stage, sizeof(double) * r.w * r.rows, cudaMemcpyDeviceToHost, ctx->st));
            ARK_CUDA(cudaStreamSynchronize(ctx->st));
            return ARK_OK;
        }
        const double off = (Storage<T>::deviation && is_cell_density(which)) ? ctx->P.ro0 : 0.0;
        return copy_out(host, dev_of(which), face, off);
    }
    int download_raw(void *p, int face, double *host) override { return copy_out(host, (const T *)p, face, 0.0); }
    int upload_raw(void *p, int face, const double *host) override { return copy_in((T *)p, host, face, 0.0); }

    void *field_ptr(const char *name, int *face) override {
        for (int w = 0; w < 24; ++w)
            if (w != 8 && std::strcmp(name, kFields[w].name) == 0) {
                *face = kFields[w].face;
                return dev_of(w);
            }
        if (std::strcmp(name, "nut") == 0 && S.nut) {
            *face = 0;
            return S.nut;
        }
        if (name[0] == 'f' && name[1] >= '1' && name[1] <= '3' && name[2] == 0) {
            *face = 0;
            return S.f[name[1] - '1'];
        }
        if (std::strncmp(name, "sigm", 4) == 0 && name[4] >= '1' && name[4] <= '3' && name[5] >= '1' &&
            name[5] <= '3' && name[6] == 0) {
            *face = 1;
            return S.sig[name[5] - '1'][name[4] - '1'];
        }
        return nullptr;
    }

    void clear_parts() {
        cudaMemsetAsync(S.part_max, 0, sizeof(unsigned long long) * 3 * kBuckets, ctx->st);
        cudaMemsetAsync(S.part_sum, 0, sizeof(long long) * kBuckets, ctx->st);
    }
    void time_step_size(int con, int advance) override {
        clear_parts();
        Launch<T>::reduce_start(S, con, ctx->st);
        Launch<T>::finalize_dt(S, advance, ctx->st);
    }
    void reduce(int con) override {
        clear_parts();
        Launch<T>::reduce_start(S, con, ctx->st);
    }
    void phase1(int src, int dst, int fcur, int mode) override {
        Launch<T>::phase1(S, src, dst, fcur, mode, ctx->march[0], ctx->st, ctx->p1_chunk);
    }
    void stress(int con, int bulk) override {
        Launch<T>::wrap_con(S, con, 0, ctx->st);
        if (S.sig[0][0]) {
            for (int d = 0; d < 3; ++d)
                for (int m = 0; m < 3; ++m)
                    cudaMemsetAsync(S.sig[d][m], 0, sizeof(T) * (size_t)S.g.nface(), ctx->st);
        }
        Launch<T>::stress(S, con, bulk, ctx->st);
    }
    void use_forces(int ncon) override { Launch<T>::use_forces(S, ncon, ctx->st); }
    void phase2(int con, int fcur) override {
        Launch<T>::wrap_phase2(S, con, fcur, ctx->st);
        for (int ax = 0; ax < 3; ++ax) Launch<T>::sweep(S, con, fcur, ax, ctx->st, ctx->seg_target, ctx->x1_lines);
    }
    // One full step of main.cpp:82-91 with "Con" = level x at entry and exit, reading the
    // dt / bulk-flow partials of the current state and leaving those of the next one.  With
    // ev given, an event is recorded after each of the step_launches() launches.
    void step(int x, int fcur, cudaEvent_t *ev) override {
        const int y = x ^ 1;
        cudaStream_t st = ctx->st;
        int nmark = 0;
        auto mark = [&]() {
            if (ev) cudaEventRecord(ev[nmark], st);
            ++nmark;
        };
        int mode = P1_STRESS | P1_FORCES | P1_RMAX | (ctx->k.forcing ? P1_BULK : 0);
        if (ctx->closure_net) {
            // the learned closure: nu_t of the level the stress reads, on a branch beside dt and
            // the ghost fill (it reads only that level's interior and the flags)
            cudaEventRecord(ctx->fork, st);
            cudaStreamWaitEvent(ctx->side, ctx->fork, 0);
            closure_nut<T>(S, y, ctx->closure_net, ctx->closure_scale, ctx->side);
            cudaEventRecord(ctx->join, ctx->side);
            mode |= P1_NUT;
        }
        // the one-kernel Phase2 forms read x and z ghosts; the sweep kernels read the ghost
        // positions from the cells and faces they stand for (x1: xcell; x3: zcell, unless the
        // z ghosts are a slab's halo), so with them the Phase2 ghost fill has nothing to do and
        // the Con level's density needs no ghosts
        const int xg = ctx->p2mode >= 1 && ctx->p2mode <= 3 ? 1 : 0;
        const bool nofill = skip_phase2_fill();
        if (!ev) {
            // captured: the ghost fill (the "Con" level's ghosts) beside dt (the partial slots
            // and the scalars): independent work, both done before Phase1
            cudaEventRecord(ctx->fill_fork, st);
            cudaStreamWaitEvent(ctx->fill, ctx->fill_fork, 0);
            Launch<T>::wrap_con(S, y, xg ? 2 : nofill ? 0 : 1, ctx->fill);
            cudaEventRecord(ctx->fill_join, ctx->fill);
            Launch<T>::finalize_dt(S, 1, st);
            cudaStreamWaitEvent(st, ctx->fill_join, 0);
        } else { // timed one launch after the other
            Launch<T>::finalize_dt(S, 1, st);
            mark();
            Launch<T>::wrap_con(S, y, xg ? 2 : nofill ? 0 : 1, st);
            mark();
        }
        if (ctx->closure_net) cudaStreamWaitEvent(st, ctx->join, 0);
        // Phase2 form 4: the x1 sweep folded into Phase1 + stress (TMA-staged FP32 shapes; the
        // seam kernel takes the x1 sweep's launch), else Phase1 + stress alone (should the folded
        // form be unavailable, the x1 sweep follows in the same timed slot)
        const bool fold = folds_x1(), fold3 = fold && ctx->p2mode == 5;
        const bool xs =
            fold && Launch<T>::phase1_sweep_x(S, y, x, fcur, mode, ctx->march[0], st, ctx->p1_chunk, seams, fold3 ? 3 : 1);
        const bool zs = xs && fold3; // form 5: the x3 sweep folded in too
        if (!xs) Launch<T>::phase1(S, y, x, fcur, mode, ctx->march[0], st, ctx->p1_chunk);
        if (fold && !xs) Launch<T>::sweep(S, y, fcur, 0, st, ctx->seg_target, ctx->x1_lines);
        mark();
        if (!nofill) {
            Launch<T>::wrap_phase2(S, y, fcur, st, xg);
            mark();
        }
        if (use_step2()) {
            // Phase2 and the second Phase1 in one kernel; the new level goes to the spare, which
            // after_step swaps in as "nCon"
            Launch<T>::phase2_phase1(S, y, fcur, S.spare, st, ctx->p2mode == 3);
            mark();
            if (ctx->averaging) {
                DevState<T> Sn = S;
                Sn.lv[y] = S.spare;
                output_average_add<T>(Sn, y, ctx->avg, st);
            }
            return;
        }
        if (ctx->p2mode == 1) { // one kernel for the three sweeps: timed in the first sweep's slot
            Launch<T>::phase2_fused(S, y, fcur, st);
            for (int ax = 0; ax < 3; ++ax) mark();
        } else {
            // the seam faces of the folded sweeps: only the second Phase1 reads the x and z faces,
            // so (captured) they are written beside the x2 sweep (and the x3 sweep), on the second
            // stream
            const bool beside = xs && !ev;
            if (beside) {
                cudaEventRecord(ctx->seam_fork, st);
                cudaStreamWaitEvent(ctx->fill, ctx->seam_fork, 0);
                Launch<T>::sweep_x_seams(S, y, fcur, seams, ctx->fill);
                if (zs) Launch<T>::sweep_z_seams(S, y, fcur, seams.kch, ctx->fill);
                cudaEventRecord(ctx->seam_join, ctx->fill);
            }
            for (int ax = 0; ax < 3; ++ax) {
                if (ax == 0 && xs) {
                    if (!beside) Launch<T>::sweep_x_seams(S, y, fcur, seams, st);
                } else if (ax == 2 && zs) {
                    if (!beside) Launch<T>::sweep_z_seams(S, y, fcur, seams.kch, st);
                } else if (ax > 0 || !fold) {
                    Launch<T>::sweep(S, y, fcur, ax, st, ctx->seg_target, ctx->x1_lines);
                }
                mark();
            }
            if (beside) cudaStreamWaitEvent(st, ctx->seam_join, 0);
        }
        Launch<T>::phase1(S, x, y, fcur ^ 1, P1_FORCES | P1_RSUM, ctx->march[1], st, ctx->p1_chunk);
        mark();
        // AverageValues after the step (main.cpp:93-96 when enabled), outside the timed marks
        if (ctx->averaging) output_average_add<T>(S, y, ctx->avg, st);
    }
    int staging_unmet(int x, int fcur) override { return Launch<T>::staging_unmet(S, x ^ 1, x, fcur, ctx->st); }
    void boundary_fill(int ncon, int axis, int periodic) override {
        Launch<T>::boundary_fill(S, ncon, axis, periodic, ctx->st);
    }
    void sums(int ncon) override { Launch<T>::sums(S, ncon, ctx->st); }
    void mean_profile(int ncon, long long *acc) override { Launch<T>::mean_profile(S, ncon, acc, ctx->st); }
    void pack(int ncon, int fcur, const CellPack &a) override { output_pack<T>(S, ncon, fcur, a, ctx->st); }
    int alloc_nut() override { return S.nut ? ARK_OK : get(&S.nut, (size_t)S.g.ncell()); }
    void plane_stats(int ncon, double *out) override { output_plane_stats<T>(S, ncon, out, ctx->st); }
    void gather(int lvl, double *u0, double *u1, double *u2) override { closure_gather<T>(S, lvl, u0, u1, u2, ctx->st); }
    void average_add(int ncon) override { output_average_add<T>(S, ncon, ctx->avg, ctx->st); }
    void energy(int ncon, double *scratch, double *out) override { output_energy<T>(S, ncon, scratch, out, ctx->st); }
    DevScalars *scalars() override { return S.sc; }
    uint8_t *flags() override { return S.flags; }
    bool use_step2() const { return (ctx->p2mode == 2 || ctx->p2mode == 3) && S.spare.ro; }
    // the three sweep kernels (or the x1 sweep folded into Phase1) of a context whose z ghosts
    // are its own: no Phase2 ghost fill
    bool skip_phase2_fill() const { return (ctx->p2mode == 0 || ctx->p2mode >= 4) && !S.k.ext_z; }
    // Phase2 forms 4 and 5 where the Phase1 shape allows them (FP32, TMA-staged Phase1 + stress)
    bool folds_x1() const {
        return (ctx->p2mode == 4 || ctx->p2mode == 5) && seams.b[0] && ctx->march[0] >= 4 && ctx->march[0] <= 6 &&
               !ctx->closure_net && !S.k.ext_z;
    }
    int step_launches() override { return use_step2() ? 5 : skip_phase2_fill() ? kNumStepKernels - 1 : kNumStepKernels; }
    const char *step_kernel_name(int q) override {
        if (q < 0 || q >= step_launches()) return "";
        if (skip_phase2_fill() && q >= 3) ++q; // no wrap_phase2
        if (use_step2() && q == 4) return "phase2_phase1_forces";
        if (folds_x1() && ctx->p2mode == 5 && (q == 2 || q == 6))
            return q == 2 ? "phase1_stress_sweep_x1_x3" : "sweep_x3_seams";
        if (folds_x1() && (q == 2 || q == 4)) return q == 2 ? "phase1_stress_sweep_x1" : "sweep_x1_seams";
        return kStepKernels[q];
    }
    void after_step(int con) override {
        if (use_step2()) std::swap(S.lv[con ^ 1], S.spare);
    }
    const void *level_ptr(int l) override { return l < 2 ? (const void *)S.lv[l].ro : (const void *)S.spare.ro; }

    void set_consts(const Consts &k) override { S.k = k; }
    void share_scalars(DevScalars *sc, unsigned long long *part_max, long long *part_sum) override {
        S.sc = sc;
        S.part_max = part_max;
        S.part_sum = part_sum;
    }
    void reduce_into(int con) override { Launch<T>::reduce_start(S, con, ctx->st); }
    // the launches of step() in the same order, cut where a slab group exchanges halos
    void stage(int q, int x, int fcur) override {
        const int y = x ^ 1;
        cudaStream_t st = ctx->st;
        switch (q) {
        case 0: Launch<T>::finalize_dt(S, 1, st); break;
        case 1: Launch<T>::wrap_con(S, y, 1, st); break;
        case 2:
            Launch<T>::phase1(S, y, x, fcur, P1_STRESS | P1_FORCES | P1_RMAX | (ctx->k.forcing ? P1_BULK : 0),
                              ctx->march[0], st, ctx->p1_chunk);
            break;
        case 3: Launch<T>::wrap_phase2(S, y, fcur, st); break;
        default:
            for (int ax = 0; ax < 3; ++ax) Launch<T>::sweep(S, y, fcur, ax, st, ctx->seg_target, ctx->x1_lines);
            Launch<T>::phase1(S, x, y, fcur ^ 1, P1_FORCES | P1_RSUM, ctx->march[1], st, ctx->p1_chunk);
            break;
        }
    }
    int halo_arrays(int exchange, int x, int fcur, void **ptrs, int *face) override {
        const int y = x ^ 1;
        int n = 0;
        auto add = [&](T *a, int f) {
            if (!a) return; // FP32 contexts keep no face density
            ptrs[n] = a;
            face[n] = f;
            ++n;
        };
        if (exchange == 0) { // wrap_con(y, with_ro = 1) along z
            const Level<T> &L = S.lv[y];
            add(L.u1, 0);
            add(L.u2, 0);
            add(L.u3, 0);
            add(L.ro, 0);
        } else { // wrap_phase2(y) along z
            const Level<T> &Ln = S.lv[x], &Lc = S.lv[y];
            add(Ln.u1, 0);
            add(Ln.u2, 0);
            add(Ln.u3, 0);
            add(Ln.ro, 0);
            add(Lc.ro, 0);
            const FaceSet<T> &Z = S.fc[fcur][2];
            add(Z.p, 1);
            add(Z.u[0], 1);
            add(Z.u[1], 1);
            add(Z.u[2], 1);
            add(Z.ro, 1);
        }
        return n;
    }
    void halo_exchange(const HaloJob *jobs, int njobs) override { Launch<T>::halo_exchange(S.g, jobs, njobs, ctx->st); }
};

int check_params(const ark_params *p) {
    if (!p) return fail(ARK_ERR_PARAM, "params is NULL");
    if (p->n1_cells < 1 || p->n2_cells < 1 || p->n3_cells < 1) return fail(ARK_ERR_PARAM, "need at least one cell per axis");
    const double faces = (double)device_pitch(p->n1_cells) * (p->n2_cells + 3) * (p->n3_cells + 3);
    if (p->n1_cells > (1 << 28) || faces >= 2147483647.0) return fail(ARK_ERR_PARAM, "grid too large: arrays are indexed with 32 bits");
    if (!(p->lx > 0) || !(p->ly > 0) || !(p->lz > 0)) return fail(ARK_ERR_PARAM, "domain extents must be > 0");
    if (!(p->sound > 0) || !(p->ro0 > 0) || !(p->cfl > 0) || !(p->vis >= 0))
        return fail(ARK_ERR_PARAM, "sound, ro0, cfl must be > 0 and vis >= 0");
    if (p->precision != ARK_FP64 && p->precision != ARK_FP32) return fail(ARK_ERR_PARAM, "unknown precision");
    return ARK_OK;
}

// dt and the copies the kernels read (1/dt, and both rounded to FP32)
void set_dt_fields(DevScalars &sc, double dt) {
    sc.dt = dt;
    sc.rdt = 1.0 / dt;
    sc.dtf = (float)dt;
    sc.rdtf = (float)(1.0 / dt);
    sc.qdt = make_qrecip(dt);
}

int check_ctx(ark_ctx *ctx, bool need_state) {
    if (!ctx) return fail(ARK_ERR_PARAM, "context is NULL");
    if (need_state && !ctx->uploaded) return fail(ARK_ERR_STATE, "no state uploaded");
    return ARK_OK;
}

int launch_status(ark_ctx *ctx) {
    (void)ctx;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ARK_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return ARK_OK;
}

} // namespace

extern "C" {

const char *ark_last_error(void) { return g_last_error.c_str(); }

const char *ark_status_string(int s) {
    switch (s) {
    case ARK_OK: return "ok";
    case ARK_ERR_PARAM: return "bad parameter";
    case ARK_ERR_CUDA: return "CUDA error";
    case ARK_ERR_NONFINITE: return "non-finite value in the velocity field";
    case ARK_ERR_STATE: return "call out of order";
    case ARK_ERR_NOMEM: return "device allocation failed";
    case ARK_ERR_UNSUPPORTED: return "unsupported configuration";
    case ARK_ERR_IO: return "file could not be opened or written";
    default: return "unknown status";
    }
}

size_t ark_cell_count(const ark_params *p) {
    return p ? (size_t)(p->n1_cells + 2) * (p->n2_cells + 2) * (p->n3_cells + 2) : 0;
}
size_t ark_face_count(const ark_params *p) {
    return p ? (size_t)(p->n1_cells + 3) * (p->n2_cells + 3) * (p->n3_cells + 3) : 0;
}

ark_ctx *ark_create(const ark_params *params, int *status) {
    int dummy;
    if (!status) status = &dummy;
    *status = check_params(params);
    if (*status) return nullptr;
    if (cudaSetDevice(params->device) != cudaSuccess) {
        *status = fail(ARK_ERR_CUDA, "cudaSetDevice failed (no usable GPU?)");
        return nullptr;
    }
    std::unique_ptr<ark_ctx> ctx(new ark_ctx());
    ctx->P = *params;
    ctx->g = make_geom(*params);
    ctx->k = make_consts(*params);
    // the step's stream at the highest priority, so that work on lower-priority branches (the
    // learned closure's inference) only takes SMs the step's kernels leave idle
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (cudaStreamCreateWithPriority(&ctx->st, cudaStreamNonBlocking, prio_high) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->fill, cudaStreamNonBlocking, prio_high) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->fill_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->fill_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->seam_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->seam_join, cudaEventDisableTiming) != cudaSuccess) {
        *status = fail(ARK_ERR_CUDA, "cudaStreamCreate failed");
        return nullptr;
    }
    if (params->precision == ARK_FP64) ctx->eng.reset(new EngineT<double>(ctx.get()));
    else ctx->eng.reset(new EngineT<float>(ctx.get()));
    *status = ctx->eng->alloc();
    if (*status) return nullptr;
    // the transfer staging buffer: one host face array (the largest host array)
    if (cudaMalloc(&ctx->stage, sizeof(double) * ark_face_count(params)) != cudaSuccess) {
        *status = fail(ARK_ERR_NOMEM, "staging allocation failed");
        return nullptr;
    }
    // Phase1 kernel shapes measured fastest on GB300 at the benchmark sizes: FP32 stages its
    // planes in shared memory with TMA tensor copies (Phase1 + stress 0.558 ms against 0.611
    // with cp.async copies, 0.70 one cell per thread and 1.10 marching at 512x256x256; second
    // Phase1 0.507 against 0.540); FP64 computes each face's quantities once (1.94 vs 2.37 ms
    // and 1.10 vs 1.18 ms one cell per thread at 256x128x128).  ark_autotune picks per grid.
    ctx->march[0] = params->precision == ARK_FP32 ? 4 : 3;
    if (params->precision == ARK_FP32) {
        // FP32: the x1 and x3 sweeps folded into Phase1 + stress (Phase2 form 5), on 128 x 2
        // tiles where lines are long enough to fill them (a tile seam every 128 cells): at
        // 512x256x256 the step takes 1.980 ms against 2.130 with the x1 sweep alone folded in
        // (form 4) and 2.210 with the separate sweeps (form 0); Phase1 + stress with both sweeps
        // 1.032 ms and the seams 0.055 + 0.029 ms, against 0.538 + 0.421 + 0.374 for the three
        // kernels.  On 64 x 4 tiles: 2.012 ms.  Smaller grids (form 5 on 64 x 4 / 128 x 2 tiles
        // against form 0, ms per step): 256x128x128 0.329 / 0.324 against 0.353, 128x64x64
        // 0.0606 / 0.0595 against 0.0734, 64x48x48 0.0451 / 0.0461 against 0.0522
        ctx->p2mode = 5;
        if (params->n1_cells >= 128) ctx->march[0] = 6;
    }
    // x2/x3 segments: 20 faces for FP64 (0.531 / 0.508 -> 0.513 / 0.492 ms at 256x128x128 against
    // 32), 16 for FP32 (what the autotuner picks at 512x256x256)
    ctx->seg_target = params->precision == ARK_FP32 ? 16 : 20;
    ctx->march[1] = params->precision == ARK_FP32 ? 4 : 3;
    if (const char *e = std::getenv("ARK_PHASE1_MARCH")) { // "ab": a for Phase1 with stress, b without
        // 0: one cell per thread, 1: marching, 2: planes staged in shared memory (FP32 only),
        // 3: face quantities computed once (FP64 only), 4: staged with TMA copies (FP32 only),
        // 5: the same on 32 x 8 tiles, 6: on 128 x 2 tiles
        auto ok = [&](char ch) {
            return ch >= '0' && ch <= '1' ? true : (params->precision == ARK_FP32 ? ch == '2' || (ch >= '4' && ch <= '6') : ch == '3');
        };
        if (ok(e[0])) ctx->march[0] = e[0] - '0';
        if (e[0] && ok(e[1])) ctx->march[1] = e[1] - '0';
    }
    if (const char *e = std::getenv("ARK_PHASE2_FUSED"))
        if (e[0] >= '0' && e[0] <= '5' && (e[0] < '2' || params->precision == ARK_FP32)) ctx->p2mode = e[0] - '0';
    Launch<float>::prepare();
    Launch<double>::prepare();
    cudaEventCreate(&ctx->ev0);
    cudaEventCreate(&ctx->ev1);
    *status = ARK_OK;
    return ctx.release();
}

int ark_destroy(ark_ctx *ctx) {
    if (!ctx) return ARK_OK;
    cudaStreamSynchronize(ctx->st);
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            if (ctx->graph[a][b]) cudaGraphExecDestroy(ctx->graph[a][b]);
    ctx->eng.reset();
    if (ctx->stage) cudaFree(ctx->stage);
    if (ctx->cond_dev) cudaFree(ctx->cond_dev);
    for (double *a : ctx->avg.a)
        if (a) cudaFree(a);
    if (ctx->closure_net) cudaFree(ctx->closure_net);
    if (ctx->side) {
        cudaStreamSynchronize(ctx->side);
        cudaStreamDestroy(ctx->side);
    }
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    if (ctx->join) cudaEventDestroy(ctx->join);
    if (ctx->fill) {
        cudaStreamSynchronize(ctx->fill);
        cudaStreamDestroy(ctx->fill);
    }
    if (ctx->fill_fork) cudaEventDestroy(ctx->fill_fork);
    if (ctx->fill_join) cudaEventDestroy(ctx->fill_join);
    if (ctx->seam_fork) cudaEventDestroy(ctx->seam_fork);
    if (ctx->seam_join) cudaEventDestroy(ctx->seam_join);
    for (int b = 0; b < 2; ++b) {
        if (ctx->io_dev[b]) cudaFree(ctx->io_dev[b]);
        if (ctx->io_host[b]) cudaFreeHost(ctx->io_host[b]);
    }
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
    return ARK_OK;
}

int ark_upload(ark_ctx *ctx, const ark_host_state *h) {
    if (int rc = check_ctx(ctx, false)) return rc;
    if (!h) return fail(ARK_ERR_PARAM, "host state is NULL");
    for (const FieldRef &f : kFields)
        if (!(h->*f.member) && !(f.member == &ark_host_state::condition && ctx->uploaded))
            return fail(ARK_ERR_PARAM, std::string("host array ") + f.name + " is NULL");
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    ctx->con = 0;
    ctx->fcur = 0;
    ctx->parts_valid = false;
    for (int w = 0; w < 24; ++w) {
        if (w == 8) continue;
        if (int rc = ctx->eng->upload_field(w, kFields[w].face, h->*kFields[w].member)) return rc;
    }
    if (!h->condition) return ARK_OK; // keep the condition (and the scalars) of the last upload
    // condition: a device copy in the host layout (for download), turned into flag bits and the
    // fluid-cell count on the device; the scalars start from zero
    const Geom hg = host_geom(ctx->g.C1, ctx->g.C2, ctx->g.C3);
    const size_t nc = (size_t)hg.ncell();
    if (!ctx->cond_dev && cudaMalloc(&ctx->cond_dev, sizeof(double) * nc) != cudaSuccess) {
        ctx->cond_dev = nullptr;
        return fail(ARK_ERR_NOMEM, "condition array allocation failed");
    }
    ARK_CUDA(cudaMemcpyAsync(ctx->cond_dev, h->condition, sizeof(double) * nc, cudaMemcpyHostToDevice, ctx->st));
    DevScalars *sc = ctx->eng->scalars();
    ARK_CUDA(cudaMemsetAsync(sc, 0, sizeof(DevScalars), ctx->st));
    const int blocks = (int)std::min<size_t>((nc + 255) / 256, 152 * 16);
    k_condition_flags<<<blocks, 256, 0, ctx->st>>>(ctx->cond_dev, ctx->eng->flags(), hg, ctx->g,
                                                    (unsigned long long *)&sc->nfluid);
    ARK_CUDA(cudaGetLastError());
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    ctx->uploaded = true;
    return ARK_OK;
}

int ark_download(ark_ctx *ctx, ark_host_state *h) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!h) return fail(ARK_ERR_PARAM, "host state is NULL");
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    for (int w = 0; w < 24; ++w) {
        double *dst = h->*kFields[w].member;
        if (!dst) continue;
        if (w == 8) {
            ARK_CUDA(cudaMemcpyAsync(dst, ctx->cond_dev, sizeof(double) * (size_t)host_geom(ctx->g.C1, ctx->g.C2, ctx->g.C3).ncell(),
                                     cudaMemcpyDeviceToHost, ctx->st));
            continue;
        }
        if (int rc = ctx->eng->download_field(w, kFields[w].face, dst)) return rc;
    }
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    return ARK_OK;
}

// "averageU1".."averageU3" -> 1..3, anything else -> 0
static int average_name(const char *name) {
    if (std::strncmp(name, "averageU", 8) == 0 && name[8] >= '1' && name[8] <= '3' && name[9] == 0) return name[8] - '0';
    return 0;
}

// The averageU arrays, allocated and zeroed on first use.
static int ensure_averages(ark_ctx *ctx) {
    if (ctx->avg.a[0]) return ARK_OK;
    const size_t n = (size_t)avg_count(ctx->g);
    for (int m = 0; m < 3; ++m) {
        cudaError_t e = cudaMalloc(&ctx->avg.a[m], sizeof(double) * n);
        if (e != cudaSuccess) {
            for (double *&a : ctx->avg.a) {
                if (a) cudaFree(a);
                a = nullptr;
            }
            return fail(ARK_ERR_NOMEM, std::string("averageU: ") + cudaGetErrorString(e));
        }
        ARK_CUDA(cudaMemset(ctx->avg.a[m], 0, sizeof(double) * n));
    }
    return ARK_OK;
}

int ark_get_array(ark_ctx *ctx, const char *name, double *host) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!name || !host) return fail(ARK_ERR_PARAM, "NULL name or buffer");
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    if (std::strcmp(name, "condition") == 0) {
        ARK_CUDA(cudaMemcpy(host, ctx->cond_dev, sizeof(double) * (size_t)host_geom(ctx->g.C1, ctx->g.C2, ctx->g.C3).ncell(),
                            cudaMemcpyDeviceToHost));
        return ARK_OK;
    }
    for (int w = 0; w < 24; ++w)
        if (w != 8 && std::strcmp(name, kFields[w].name) == 0) return ctx->eng->download_field(w, kFields[w].face, host);
    if (int m = average_name(name)) {
        if (int rc = ensure_averages(ctx)) return rc;
        ARK_CUDA(cudaMemcpy(host, ctx->avg.a[m - 1], sizeof(double) * avg_count(ctx->g), cudaMemcpyDeviceToHost));
        return ARK_OK;
    }
    int face = 0;
    void *p = ctx->eng->field_ptr(name, &face);
    if (!p) return fail(ARK_ERR_PARAM, std::string("no device array named ") + name);
    return ctx->eng->download_raw(p, face, host);
}

int ark_put_array(ark_ctx *ctx, const char *name, const double *host) {
    if (int rc = check_ctx(ctx, true)) return rc;
    ctx->parts_valid = false;
    if (!name || !host) return fail(ARK_ERR_PARAM, "NULL name or buffer");
    if (std::strcmp(name, "condition") == 0) return fail(ARK_ERR_PARAM, "condition is set by ark_upload");
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    for (int w = 0; w < 24; ++w)
        if (w != 8 && std::strcmp(name, kFields[w].name) == 0) return ctx->eng->upload_field(w, kFields[w].face, host);
    if (int m = average_name(name)) {
        if (int rc = ensure_averages(ctx)) return rc;
        ARK_CUDA(cudaMemcpy(ctx->avg.a[m - 1], host, sizeof(double) * avg_count(ctx->g), cudaMemcpyHostToDevice));
        return ARK_OK;
    }
    int face = 0;
    void *p = ctx->eng->field_ptr(name, &face);
    if (!p) return fail(ARK_ERR_PARAM, std::string("no device array named ") + name);
    return ctx->eng->upload_raw(p, face, host);
}

int ark_time_step_size(ark_ctx *ctx) {
    if (int rc = check_ctx(ctx, true)) return rc;
    ctx->eng->time_step_size(ctx->con, 0);
    return launch_status(ctx);
}

int ark_phase1(ark_ctx *ctx) {
    if (int rc = check_ctx(ctx, true)) return rc;
    ctx->parts_valid = false;
    // "Con" <- "nCon" is a relabelling: the old nCon level is read as Con and the new
    // nCon values are written over the old Con level.
    const int src = ctx->con ^ 1, dst = ctx->con;
    ctx->eng->phase1(src, dst, ctx->fcur, P1_PLAIN);
    ctx->con = src;
    return launch_status(ctx);
}

int ark_stress_tensor(ark_ctx *ctx) {
    if (int rc = check_ctx(ctx, true)) return rc;
    ctx->parts_valid = false;
    ctx->eng->stress(ctx->con, ctx->k.forcing);
    return launch_status(ctx);
}

int ark_use_forces(ark_ctx *ctx) {
    if (int rc = check_ctx(ctx, true)) return rc;
    ctx->parts_valid = false;
    ctx->eng->use_forces(ctx->con ^ 1);
    return launch_status(ctx);
}

int ark_phase2(ark_ctx *ctx) {
    if (int rc = check_ctx(ctx, true)) return rc;
    ctx->parts_valid = false;
    ctx->eng->phase2(ctx->con, ctx->fcur);
    ctx->fcur ^= 1; // the sweeps wrote the other face generation
    return launch_status(ctx);
}

int ark_boundary_fill(ark_ctx *ctx, int axis) {
    if (int rc = check_ctx(ctx, true)) return rc;
    ctx->parts_valid = false;
    if (axis < 1 || axis > 3) return fail(ARK_ERR_PARAM, "axis must be 1, 2 or 3");
    const int periodic = axis == 2 ? 0 : axis == 3 ? ctx->P.periodic_z : 0;
    ctx->eng->boundary_fill(ctx->con ^ 1, axis, periodic);
    return launch_status(ctx);
}

int ark_boundary_conditions(ark_ctx *ctx, int axis, int x1_period, int x2_period, int x3_period) {
    (void)x1_period; // BoundaryConditions::alongX1 never reads it (source/BoundaryConditions.cpp:22-42)
    if (int rc = check_ctx(ctx, true)) return rc;
    ctx->parts_valid = false;
    if (axis < 1 || axis > 3) return fail(ARK_ERR_PARAM, "axis must be 1, 2 or 3");
    const int periodic = axis == 2 ? (x2_period != 0) : axis == 3 ? (x3_period != 0) : 0;
    ctx->eng->boundary_fill(ctx->con ^ 1, axis, periodic);
    return launch_status(ctx);
}

int ark_set_dt(ark_ctx *ctx, double dt) {
    if (int rc = check_ctx(ctx, true)) return rc;
    DevScalars sc;
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    ARK_CUDA(cudaMemcpy(&sc, ctx->eng->scalars(), sizeof(sc), cudaMemcpyDeviceToHost));
    set_dt_fields(sc, dt);
    ARK_CUDA(cudaMemcpy(ctx->eng->scalars(), &sc, sizeof(sc), cudaMemcpyHostToDevice));
    return ARK_OK;
}

// Captures the fused step for the current role of the two cell levels (once per role).  A graph
// holds the level buffers it was captured with; when the one-kernel Phase2 + second Phase1
// rotates them through the spare, each face generation meets its own buffers again every
// other step, and a graph that meets other buffers is captured again.
static int ensure_graph(ark_ctx *ctx) {
    const int x = ctx->con, fc = ctx->fcur;
    const void *lv[3] = {ctx->eng->level_ptr(0), ctx->eng->level_ptr(1), ctx->eng->level_ptr(2)};
    if (ctx->graph[x][fc] && std::memcmp(ctx->graph_levels[x][fc], lv, sizeof lv) != 0) {
        cudaGraphExecDestroy(ctx->graph[x][fc]);
        ctx->graph[x][fc] = nullptr;
    }
    if (!ctx->graph[x][fc]) {
        std::memcpy(ctx->graph_levels[x][fc], lv, sizeof lv);
        cudaGraph_t graph = nullptr;
        ARK_CUDA(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
        ctx->eng->step(x, fc, nullptr);
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(ctx->st, &graph);
        if (le != cudaSuccess || ce != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return fail(ARK_ERR_CUDA, std::string("step capture: ") +
                                          cudaGetErrorString(le != cudaSuccess ? le : ce));
        }
        cudaError_t ie = cudaGraphInstantiate(&ctx->graph[x][fc], graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            ctx->graph[x][fc] = nullptr;
            return fail(ARK_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        }
    }
    return ARK_OK;
}

int ark_step(ark_ctx *ctx, int nsteps) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (nsteps < 0) return fail(ARK_ERR_PARAM, "nsteps < 0");
    if (nsteps == 0) return ARK_OK;
    if (!ctx->parts_valid) {
        ctx->eng->reduce(ctx->con);
        ctx->parts_valid = true;
    }
    // each step flips the face generation; the graph of each parity is captured once
    for (int s = 0; s < nsteps; ++s) {
        if (int rc = ensure_graph(ctx)) return rc;
        ARK_CUDA(cudaGraphLaunch(ctx->graph[ctx->con][ctx->fcur], ctx->st));
        ctx->fcur ^= 1;
        ctx->eng->after_step(ctx->con);
    }
    return ARK_OK;
}

int ark_sync(ark_ctx *ctx) {
    if (int rc = check_ctx(ctx, false)) return rc;
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    int status = 0;
    ARK_CUDA(cudaMemcpy(&status, &ctx->eng->scalars()->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (status & STATUS_NONFINITE) return fail(ARK_ERR_NONFINITE, "non-finite velocity detected on the device");
    if (status & STATUS_STAGING) return fail(ARK_ERR_CUDA, "a staged Phase1 block gave up waiting for its TMA copies");
    return ARK_OK;
}

int ark_time_steps(ark_ctx *ctx, int nsteps, double *ms) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!ms) return fail(ARK_ERR_PARAM, "ms is NULL");
    // both face-generation graphs are built outside the timed region (each with the level
    // buffers the step will meet; after_step is its own inverse)
    if (int rc = ensure_graph(ctx)) return rc;
    ctx->fcur ^= 1;
    ctx->eng->after_step(ctx->con);
    int rc2 = ensure_graph(ctx);
    ctx->fcur ^= 1;
    ctx->eng->after_step(ctx->con);
    if (rc2) return rc2;
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    ARK_CUDA(cudaEventRecord(ctx->ev0, ctx->st));
    if (int rc = ark_step(ctx, nsteps)) return rc;
    ARK_CUDA(cudaEventRecord(ctx->ev1, ctx->st));
    ARK_CUDA(cudaEventSynchronize(ctx->ev1));
    float f = 0.f;
    ARK_CUDA(cudaEventElapsedTime(&f, ctx->ev0, ctx->ev1));
    *ms = (double)f;
    return ark_sync(ctx);
}

int ark_kernel_times(ark_ctx *ctx, int nsteps, double *ms, int cap, int *count) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!ms || !count || nsteps < 1) return fail(ARK_ERR_PARAM, "bad arguments");
    const int nk = ctx->eng->step_launches();
    *count = nk;
    std::vector<cudaEvent_t> ev(kNumStepKernels + 1);
    for (auto &e : ev) ARK_CUDA(cudaEventCreate(&e));
    std::vector<double> acc(kNumStepKernels, 0.0);
    int rc = ARK_OK;
    if (!ctx->parts_valid) {
        ctx->eng->reduce(ctx->con);
        ctx->parts_valid = true;
    }
    for (int s = 0; s < nsteps && rc == ARK_OK; ++s) {
        cudaEventRecord(ev[0], ctx->st);
        ctx->eng->step(ctx->con, ctx->fcur, ev.data() + 1);
        ctx->fcur ^= 1;
        ctx->eng->after_step(ctx->con);
        if ((rc = launch_status(ctx))) break;
        if (cudaEventSynchronize(ev[nk]) != cudaSuccess) {
            rc = fail(ARK_ERR_CUDA, "event synchronize failed");
            break;
        }
        for (int q = 0; q < nk; ++q) {
            float f = 0.f;
            cudaEventElapsedTime(&f, ev[q], ev[q + 1]);
            acc[q] += f;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int q = 0; q < nk && q < cap; ++q) ms[q] = acc[q] / nsteps;
    if (rc) return rc;
    return ark_sync(ctx);
}

const char *ark_kernel_name(int index) {
    return index >= 0 && index < kNumStepKernels ? kStepKernels[index] : nullptr;
}

const char *ark_step_kernel_name(ark_ctx *ctx, int index) {
    if (!ctx || !ctx->eng || index < 0 || index >= ctx->eng->step_launches()) return nullptr;
    return ctx->eng->step_kernel_name(index);
}

int ark_alloc_host_state(const ark_params *p, ark_host_state *out) {
    if (!p || !out) return fail(ARK_ERR_PARAM, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    const size_t nc = ark_cell_count(p), nf = ark_face_count(p);
    for (const FieldRef &f : kFields) {
        void *ptr = nullptr;
        const size_t bytes = sizeof(double) * (f.face ? nf : nc);
        cudaError_t e = cudaHostAlloc(&ptr, bytes, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            ark_free_host_state(out);
            return fail(ARK_ERR_NOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
        }
        std::memset(ptr, 0, bytes);
        out->*f.member = (double *)ptr;
    }
    return ARK_OK;
}

int ark_free_host_state(ark_host_state *h) {
    if (!h) return ARK_OK;
    for (const FieldRef &f : kFields) {
        if (h->*f.member) cudaFreeHost(h->*f.member);
        h->*f.member = nullptr;
    }
    return ARK_OK;
}

int ark_get_scalars(ark_ctx *ctx, ark_scalars *out) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!out) return fail(ARK_ERR_PARAM, "out is NULL");
    DevScalars sc;
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    ARK_CUDA(cudaMemcpy(&sc, ctx->eng->scalars(), sizeof(sc), cudaMemcpyDeviceToHost));
    out->dt = sc.dt;
    out->time = sc.time;
    out->nstep = sc.nstep;
    out->bulk_velocity = sc.ub;
    out->bulk_force = sc.G;
    return ARK_OK;
}

int ark_set_scalars(ark_ctx *ctx, const ark_scalars *in) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!in) return fail(ARK_ERR_PARAM, "in is NULL");
    DevScalars sc;
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    ARK_CUDA(cudaMemcpy(&sc, ctx->eng->scalars(), sizeof(sc), cudaMemcpyDeviceToHost));
    set_dt_fields(sc, in->dt);
    sc.time = in->time;
    sc.nstep = in->nstep;
    sc.ub = in->bulk_velocity;
    sc.G = in->bulk_force;
    sc.Gf = (float)in->bulk_force;
    ARK_CUDA(cudaMemcpy(ctx->eng->scalars(), &sc, sizeof(sc), cudaMemcpyHostToDevice));
    return ARK_OK;
}

int ark_conservation_sums(ark_ctx *ctx, ark_sums *out) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!out) return fail(ARK_ERR_PARAM, "out is NULL");
    DevScalars *dsc = ctx->eng->scalars();
    ARK_CUDA(cudaMemsetAsync(&dsc->sums[0], 0, sizeof(long long) * 6, ctx->st));
    ctx->eng->sums(ctx->con ^ 1);
    if (int rc = launch_status(ctx)) return rc;
    long long v[6];
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    ARK_CUDA(cudaMemcpy(v, &dsc->sums[0], sizeof(v), cudaMemcpyDeviceToHost));
    const double q = 1.0 / 4294967296.0;
    out->mass = (double)v[0] * q;
    out->momentum1 = (double)v[1] * q;
    out->momentum2 = (double)v[2] * q;
    out->momentum3 = (double)v[3] * q;
    out->kinetic = (double)v[4] * q;
    out->cells = v[5];
    return ARK_OK;
}

int ark_selftest_staging_timeout(ark_ctx *ctx) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (ctx->P.precision != ARK_FP32) return fail(ARK_ERR_UNSUPPORTED, "the TMA staging runs in FP32 contexts");
    if (!ctx->eng->staging_unmet(ctx->con, ctx->fcur)) return fail(ARK_ERR_UNSUPPORTED, "no TMA staging for this grid");
    ARK_CUDA(cudaGetLastError());
    return ARK_OK;
}

int ark_selftest_division(long long n, unsigned long long seed, long long *mismatches) {
    if (!mismatches || n < 0) return fail(ARK_ERR_PARAM, "bad arguments");
    unsigned long long *bad = nullptr;
    ARK_CUDA(cudaMalloc(&bad, sizeof(unsigned long long)));
    cudaMemset(bad, 0, sizeof(unsigned long long));
    const int rc = selftest_division(n, seed, bad, 0);
    cudaError_t e = cudaGetLastError();
    if (rc && e == cudaSuccess) e = cudaErrorMemoryAllocation;
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(bad);
    if (e != cudaSuccess) return fail(ARK_ERR_CUDA, std::string("selftest: ") + cudaGetErrorString(e));
    *mismatches = (long long)h;
    return ARK_OK;
}

int ark_mean_profile(ark_ctx *ctx, double *mean_u1, double *wall_shear) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!mean_u1) return fail(ARK_ERR_PARAM, "mean_u1 is NULL");
    const int n = ctx->g.C2;
    long long *acc = nullptr;
    ARK_CUDA(cudaMallocAsync((void **)&acc, sizeof(long long) * 2 * n, ctx->st));
    ctx->eng->mean_profile(ctx->con ^ 1, acc);
    int rc = launch_status(ctx);
    std::vector<long long> h(2 * (size_t)n);
    if (!rc && cudaMemcpyAsync(h.data(), acc, sizeof(long long) * 2 * n, cudaMemcpyDeviceToHost, ctx->st) != cudaSuccess)
        rc = fail(ARK_ERR_CUDA, "profile copy failed");
    cudaFreeAsync(acc, ctx->st);
    if (!rc) ARK_CUDA(cudaStreamSynchronize(ctx->st));
    if (rc) return rc;
    for (int j = 0; j < n; ++j)
        mean_u1[j] = h[2 * j + 1] > 0 ? ((double)h[2 * j] * (1.0 / 4294967296.0)) / (double)h[2 * j + 1] : 0.0;
    if (wall_shear) {
        // one-sided wall form of StressTensor (main.cpp:924-927): 2*VIS*u_c/dx2 at both walls
        wall_shear[0] = 2 * ctx->P.vis * mean_u1[0] / ctx->k.dx[1];
        wall_shear[1] = 2 * ctx->P.vis * mean_u1[n - 1] / ctx->k.dx[1];
    }
    return ARK_OK;
}

} // extern "C"

// ---- output and statistics -------------------------------------------------------------

namespace {

void drop_graphs(ark_ctx *ctx) {
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            if (ctx->graph[a][b]) {
                cudaGraphExecDestroy(ctx->graph[a][b]);
                ctx->graph[a][b] = nullptr;
            }
}

// The two slab buffers (device and pinned host) of at least n doubles each.
int ensure_io(ark_ctx *ctx, size_t n) {
    if (ctx->io_cap >= n) return ARK_OK;
    for (int b = 0; b < 2; ++b) {
        if (ctx->io_dev[b]) cudaFree(ctx->io_dev[b]);
        if (ctx->io_host[b]) cudaFreeHost(ctx->io_host[b]);
        ctx->io_dev[b] = ctx->io_host[b] = nullptr;
    }
    ctx->io_cap = 0;
    for (int b = 0; b < 2; ++b) {
        if (cudaMalloc(&ctx->io_dev[b], n * sizeof(double)) != cudaSuccess ||
            cudaMallocHost(&ctx->io_host[b], n * sizeof(double)) != cudaSuccess)
            return fail(ARK_ERR_NOMEM, "output slab buffers");
    }
    ctx->io_cap = n;
    return ARK_OK;
}

bool write_all(int fd, const void *buf, size_t n, off_t off) {
    const char *p = (const char *)buf;
    while (n > 0) {
        const ssize_t w = pwrite(fd, p, n, off);
        if (w <= 0) return false;
        p += w;
        n -= (size_t)w;
        off += w;
    }
    return true;
}

void put_be64(std::string &s, double v) {
    unsigned char b[8];
    std::memcpy(b, &v, 8);
    // host byte order is little-endian on every supported host (x86-64, aarch64)
    for (int q = 7; q >= 0; --q) s.push_back((char)b[q]);
}

// Everything before the first data block of the reference's VTK files (main.cpp:2585-2645):
// headers and node coordinates (i-1)*dx with n_g = C + 1 nodes per axis.
std::string vtk_head(const ark_ctx *ctx) {
    const Geom &g = ctx->g;
    const int ng[3] = {g.C1 + 1, g.C2 + 1, g.C3 + 1};
    char buf[256];
    std::string s = "# vtk DataFile Version 3.0\nvtk output\nBINARY\n";
    std::snprintf(buf, sizeof buf, "DATASET RECTILINEAR_GRID\nDIMENSIONS %d %d %d", ng[0], ng[1], ng[2]);
    s += buf;
    const char axis[3] = {'X', 'Y', 'Z'};
    for (int d = 0; d < 3; ++d) {
        std::snprintf(buf, sizeof buf, "\n%c_COORDINATES %d double\n", axis[d], ng[d]);
        s += buf;
        for (int i = 1; i <= ng[d]; ++i) put_be64(s, (i - 1) * ctx->k.dx[d]);
    }
    std::snprintf(buf, sizeof buf, "\nCELL_DATA %d\nVECTORS U double\n", g.C1 * g.C2 * g.C3);
    s += buf;
    return s;
}

enum BlockKind { BK_U, BK_PC, BK_R, BK_AVG };
struct Block {
    const char *header;
    int comps;
    BlockKind kind;
};

// Writes head + blocks to path.  Slabs of k planes are packed on the device into one of two
// buffers and copied to pinned memory while the host writes the previous slab.
int write_vtk_blocks(ark_ctx *ctx, const char *path, int layout, const Block *blocks, int nb, double avg_div) {
    if (!path) return fail(ARK_ERR_PARAM, "path is NULL");
    if (layout != ARK_VTK_FULL && layout != ARK_VTK_REFERENCE) return fail(ARK_ERR_PARAM, "unknown VTK layout");
    const Geom &g = ctx->g;
    const int64_t plane = (int64_t)g.C1 * g.C2, ncell = plane * g.C3;
    int comps = 0;
    for (int b = 0; b < nb; ++b) comps += blocks[b].comps;
    // slabs of about 2^20 cells; the reference layout writes only the last plane
    const int kslab = layout == ARK_VTK_REFERENCE ? 1 : (int)std::max<int64_t>(1, std::min<int64_t>(g.C3, (1 << 20) / std::max<int64_t>(plane, 1)));
    if (int rc = ensure_io(ctx, (size_t)(kslab * plane * comps))) return rc;

    const std::string head = vtk_head(ctx);
    std::vector<off_t> data_off(nb);
    const int fd = open(path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) return fail(ARK_ERR_IO, std::string("cannot open ") + path);
    bool ok = write_all(fd, head.data(), head.size(), 0);
    off_t off = (off_t)head.size();
    for (int b = 0; b < nb && ok; ++b) {
        const size_t hl = std::strlen(blocks[b].header);
        ok = write_all(fd, blocks[b].header, hl, off);
        off += (off_t)hl;
        data_off[b] = off;
        off += (off_t)(ncell * blocks[b].comps * 8);
    }
    cudaEvent_t ev[2] = {nullptr, nullptr};
    for (auto &e : ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    const int kfirst = layout == ARK_VTK_REFERENCE ? g.C3 : 1;
    struct Slab {
        int k0, k1;
    } pending[2] = {{0, 0}, {0, 0}};
    int rc = ARK_OK;
    auto flush = [&](int buf) {
        const Slab sl = pending[buf];
        if (sl.k1 <= sl.k0) return;
        if (cudaEventSynchronize(ev[buf]) != cudaSuccess) {
            rc = fail(ARK_ERR_CUDA, "output copy failed");
            return;
        }
        const int64_t ns = (int64_t)(sl.k1 - sl.k0) * plane;
        const double *h = ctx->io_host[buf];
        for (int b = 0; b < nb && ok; ++b) {
            const off_t at = layout == ARK_VTK_REFERENCE ? data_off[b] : data_off[b] + (off_t)((sl.k0 - 1) * plane * blocks[b].comps * 8);
            ok = write_all(fd, h, (size_t)(ns * blocks[b].comps * 8), at);
            h += ns * blocks[b].comps;
        }
        pending[buf] = Slab{0, 0};
    };
    int buf = 0;
    for (int k0 = kfirst; k0 <= g.C3 && ok && rc == ARK_OK; k0 += kslab, buf ^= 1) {
        const int k1 = std::min(g.C3 + 1, k0 + kslab);
        flush(buf); // the buffer about to be reused
        const int64_t ns = (int64_t)(k1 - k0) * plane;
        double *d = ctx->io_dev[buf];
        CellPack a;
        std::memset(&a, 0, sizeof a);
        a.k0 = k0;
        a.k1 = k1;
        a.swap = 1;
        a.avg_div = avg_div;
        for (int m = 0; m < 3; ++m) a.avg[m] = ctx->avg.a[m];
        for (int b = 0; b < nb; ++b) {
            switch (blocks[b].kind) {
            case BK_U: a.u = d; break;
            case BK_PC: a.pc = d; break;
            case BK_R: a.r = d; break;
            case BK_AVG: a.avg_out = d; break;
            }
            d += ns * blocks[b].comps;
        }
        ctx->eng->pack(ctx->con ^ 1, ctx->fcur, a);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(ctx->io_host[buf], ctx->io_dev[buf], (size_t)(ns * comps) * sizeof(double),
                            cudaMemcpyDeviceToHost, ctx->st) != cudaSuccess) {
            rc = fail(ARK_ERR_CUDA, "output pack failed");
            break;
        }
        cudaEventRecord(ev[buf], ctx->st);
        pending[buf] = Slab{k0, k1};
    }
    flush(buf ^ 1);
    flush(buf);
    for (auto &e : ev) cudaEventDestroy(e);
    if (close(fd) != 0) ok = false;
    if (rc) return rc;
    if (!ok) return fail(ARK_ERR_IO, std::string("write failed: ") + path);
    return ARK_OK;
}

} // namespace

extern "C" {

// Times the candidate kernel shapes on the live state (results do not depend on the shape)
// one setting at a time: the shape of the Phase1 with stress, then of the second Phase1, then
// the three sweeps separate or fused, then (separate) the x2/x3 sweep segment (8, 16, 32, 64
// faces, and 12, 20, 24, 48), the x1 sweep's lines per warp (1 to 4) and the staged Phase1's
// planes per block.
// choice (may be NULL): {shape 1, shape 2, segment, microseconds per step, fused}.
int ark_autotune(ark_ctx *ctx, int steps_per_candidate, int *choice) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (steps_per_candidate < 1) return fail(ARK_ERR_PARAM, "steps_per_candidate < 1");
    // Phase1 shapes: one cell per thread, marching, and the precision's own (staged with
    // cp.async or TMA copies for FP32, face-centric for FP64)
    const bool fp32 = ctx->P.precision == ARK_FP32;
    const int shapes[5] = {0, 1, fp32 ? 2 : 3, 4, 6};
    // best of three timings of steps_per_candidate steps each
    auto measure = [&](double *us) -> int {
        ARK_CUDA(cudaStreamSynchronize(ctx->st));
        drop_graphs(ctx);
        if (int rc = ark_step(ctx, 2)) return rc; // captures both face-generation graphs
        *us = 1e300;
        for (int rep = 0; rep < 3; ++rep) {
            double ms = 0.0;
            if (int rc = ark_time_steps(ctx, steps_per_candidate, &ms)) return rc;
            *us = std::min(*us, 1000.0 * ms / steps_per_candidate);
        }
        return ARK_OK;
    };
    double best = 0.0;
    if (int rc = measure(&best)) return rc;
    auto set = [&](int which, int v) {
        if (which < 2) ctx->march[which] = v;
        else if (which == 2) ctx->p2mode = v;
        else if (which == 3) ctx->seg_target = v;
        else if (which == 4) ctx->x1_lines = v;
        else ctx->p1_chunk = v;
    };
    if (ctx->x1_lines <= 0) ctx->x1_lines = x_lines_per_warp(ctx->g, !fp32);
    for (int which = 0; which < 6; ++which) {
        // segment lengths: the steps between also move the blocks' last wave
        const int segs[8] = {8, 12, 16, 20, 24, 32, 48, 64};
        const int lines[4] = {1, 2, 3, 4}; // x1 sweep lines per warp
        // planes per block of the staged / face-centric Phase1 (0: the default rule); the count
        // sets how evenly the blocks fill the GPU's waves against the halo planes per block
        const int chunks[16] = {0, 2, 3, 4, 6, 8, 12, 16, 22, 24, 29, 32, 37, 43, 48, 64};
        if (which == 5) {
            const bool staged = (ctx->march[0] >= 2 || ctx->march[1] >= 2);
            if (!staged) continue;
            int keep = ctx->p1_chunk;
            for (int v : chunks) {
                if (v == keep || v > ctx->g.C3) continue;
                set(which, v);
                double us = 0.0;
                if (int rc = measure(&us)) return rc;
                if (us < best) {
                    best = us;
                    keep = v;
                }
            }
            set(which, keep);
            continue;
        }
        // Phase2 forms: the three sweep kernels, or (FP32) one kernel for the sweeps and the
        // second Phase1, or (FP32) the x1 sweep folded into Phase1 + stress.  The one-kernel
        // Phase2 alone (mode 1) is correct but slower at every size measured: left to
        // ARK_PHASE2_FUSED=1, not tried here.
        const int p2cand[5] = {0, 2, 3, 4, 5};
        if (which == 2 && !fp32) continue;
        const int ncand = which < 2 ? (fp32 ? 5 : 3) : which == 2 ? 5 : which == 3 ? 8 : 4;
        int keep = which < 2 ? ctx->march[which] : which == 2 ? ctx->p2mode : which == 3 ? ctx->seg_target : ctx->x1_lines;
        // the one-kernel forms have no segments and no x1 sweep; the folded forms no x1 sweep
        if (which >= 3 && ctx->p2mode != 0 && !(which == 3 && ctx->p2mode >= 4)) continue;
        for (int c = 0; c < ncand; ++c) {
            const int v = which < 2 ? shapes[c] : which == 2 ? p2cand[c] : which == 3 ? segs[c] : lines[c];
            if (v == keep) continue;
            set(which, v);
            double us = 0.0;
            if (int rc = measure(&us)) return rc;
            if (us < best) {
                best = us;
                keep = v;
            }
        }
        set(which, keep);
    }
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    drop_graphs(ctx);
    if (choice) {
        choice[0] = ctx->march[0];
        choice[1] = ctx->march[1];
        choice[2] = ctx->seg_target;
        choice[3] = (int)std::lround(best);
        choice[4] = ctx->p2mode;
    }
    return ARK_OK;
}

int ark_set_closure(ark_ctx *ctx, const ark_mlp *mlp, double u_tau) {
    if (int rc = check_ctx(ctx, false)) return rc;
    if (mlp && ctx->P.precision != ARK_FP32) return fail(ARK_ERR_UNSUPPORTED, "the learned closure runs in FP32 contexts");
    if (mlp && !(u_tau > 0)) return fail(ARK_ERR_PARAM, "u_tau must be > 0");
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    if (mlp)
        if (int rc = ctx->eng->alloc_nut()) return rc;
    if (ctx->closure_net) {
        cudaFree(ctx->closure_net);
        ctx->closure_net = nullptr;
    }
    if (mlp && !ctx->side) {
        int prio_low = 0, prio_high = 0;
        ARK_CUDA(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
        ARK_CUDA(cudaStreamCreateWithPriority(&ctx->side, cudaStreamNonBlocking, prio_low));
        ARK_CUDA(cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
        ARK_CUDA(cudaEventCreateWithFlags(&ctx->join, cudaEventDisableTiming));
    }
    if (mlp) {
        ARK_CUDA(cudaMalloc(&ctx->closure_net, mlp_bytes()));
        if (mlp_snapshot_device(mlp, ctx->closure_net) != ARK_OK) {
            cudaFree(ctx->closure_net);
            ctx->closure_net = nullptr;
            return fail(ARK_ERR_CUDA, "could not copy the network");
        }
    }
    ctx->closure_scale = mlp ? (float)(u_tau / ctx->P.vis) : 0.f;
    drop_graphs(ctx);
    return ARK_OK;
}

int ark_closure_sample(ark_ctx *ctx, ark_closure_data *data, int sx, int sz, int ox, int oz, double u_tau) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!data) return fail(ARK_ERR_PARAM, "dataset is NULL");
    const Geom &g = ctx->g;
    if (!ctx->P.periodic_x || !ctx->P.periodic_z) return fail(ARK_ERR_UNSUPPORTED, "closure samples need periodic x and z");
    DevScalars sc;
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    ARK_CUDA(cudaMemcpy(&sc, ctx->eng->scalars(), sizeof sc, cudaMemcpyDeviceToHost));
    if (sc.nfluid != (long long)g.C1 * g.C2 * g.C3) return fail(ARK_ERR_UNSUPPORTED, "closure samples need a channel without solids");
    const long long count = closure_count(g.C1, g.C2, g.C3, sx, sz, ox, oz);
    if (count < 0) return fail(ARK_ERR_PARAM, "bad sampling lattice");
    if (count > closure_room(data)) return fail(ARK_ERR_PARAM, "dataset full");
    double *u = nullptr;
    const long long cells = (long long)g.C1 * g.C2 * g.C3;
    if (int rc = closure_scratch(data, cells, &u)) return fail(rc, ark_closure_last_error());
    ctx->eng->gather(ctx->con ^ 1, u, u + cells, u + 2 * cells);
    if (int rc = closure_sample(data, g.C1, g.C2, g.C3, ctx->P.lx, ctx->P.ly, ctx->P.lz, ctx->P.vis, sx, sz, ox, oz, u_tau,
                                ctx->st))
        return fail(rc, ark_closure_last_error());
    return ARK_OK;
}

int ark_write_vtk(ark_ctx *ctx, const char *path, int layout) {
    if (int rc = check_ctx(ctx, true)) return rc;
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    const Block blocks[3] = {{"", 3, BK_U},
                             {"\nscalars PC double\nLOOKUP_TABLE default\n", 1, BK_PC},
                             {"\nVECTORS R double\n", 3, BK_R}};
    return write_vtk_blocks(ctx, path, layout, blocks, 3, 1.0);
}

int ark_average_values(ark_ctx *ctx) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (int rc = ensure_averages(ctx)) return rc;
    ctx->eng->average_add(ctx->con ^ 1);
    return launch_status(ctx);
}

int ark_set_averaging(ark_ctx *ctx, int on) {
    if (int rc = check_ctx(ctx, false)) return rc;
    if (on)
        if (int rc = ensure_averages(ctx)) return rc;
    if ((on != 0) != ctx->averaging) {
        ARK_CUDA(cudaStreamSynchronize(ctx->st));
        drop_graphs(ctx);
        ctx->averaging = on != 0;
    }
    return ARK_OK;
}

int ark_write_average_vtk(ark_ctx *ctx, const char *path, double start_time, int layout) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (int rc = ensure_averages(ctx)) return rc;
    DevScalars sc;
    ARK_CUDA(cudaStreamSynchronize(ctx->st));
    ARK_CUDA(cudaMemcpy(&sc, ctx->eng->scalars(), sizeof sc, cudaMemcpyDeviceToHost));
    const Block blocks[1] = {{"", 3, BK_AVG}};
    return write_vtk_blocks(ctx, path, layout, blocks, 1, sc.time - start_time);
}

int ark_kinetic_energy(ark_ctx *ctx, double *energy) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!energy) return fail(ARK_ERR_PARAM, "energy is NULL");
    const int np = energy_scratch_count(ctx->g);
    double *scratch = nullptr;
    ARK_CUDA(cudaMallocAsync((void **)&scratch, sizeof(double) * (np + 1), ctx->st));
    ctx->eng->energy(ctx->con ^ 1, scratch + 1, scratch);
    int rc = launch_status(ctx);
    double sum = 0.0;
    if (!rc && cudaMemcpyAsync(&sum, scratch, sizeof(double), cudaMemcpyDeviceToHost, ctx->st) != cudaSuccess)
        rc = fail(ARK_ERR_CUDA, "energy copy failed");
    cudaFreeAsync(scratch, ctx->st);
    if (!rc) ARK_CUDA(cudaStreamSynchronize(ctx->st));
    if (rc) return rc;
    // allEnergy *= (x3_t - x3_b) * (x2_n - x2_s) * (x1_e - x1_w)  (main.cpp:2869-2870)
    const double volume = ctx->P.lz * ctx->P.ly * ctx->P.lx;
    *energy = sum * volume;
    return ARK_OK;
}

int ark_write_energy(ark_ctx *ctx, const char *path) {
    if (!path) return fail(ARK_ERR_PARAM, "path is NULL");
    double e = 0.0;
    if (int rc = ark_kinetic_energy(ctx, &e)) return rc;
    DevScalars sc;
    ARK_CUDA(cudaMemcpy(&sc, ctx->eng->scalars(), sizeof sc, cudaMemcpyDeviceToHost));
    FILE *fd = std::fopen(path, "a");
    if (!fd) return fail(ARK_ERR_IO, std::string("cannot open ") + path);
    const bool ok = std::fprintf(fd, "(%f; %f) ", sc.time, e) > 0;
    if (std::fclose(fd) != 0 || !ok) return fail(ARK_ERR_IO, std::string("write failed: ") + path);
    return ARK_OK;
}

int ark_plane_stats(ark_ctx *ctx, double *out) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!out) return fail(ARK_ERR_PARAM, "out is NULL");
    const size_t n = 9 * (size_t)ctx->g.C2;
    double *d = nullptr;
    ARK_CUDA(cudaMallocAsync((void **)&d, sizeof(double) * n, ctx->st));
    ctx->eng->plane_stats(ctx->con ^ 1, d);
    int rc = launch_status(ctx);
    if (!rc && cudaMemcpyAsync(out, d, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->st) != cudaSuccess)
        rc = fail(ARK_ERR_CUDA, "plane statistics copy failed");
    cudaFreeAsync(d, ctx->st);
    if (!rc) ARK_CUDA(cudaStreamSynchronize(ctx->st));
    return rc;
}

int ark_vorticity(ark_ctx *ctx, double *out) {
    if (int rc = check_ctx(ctx, true)) return rc;
    if (!out) return fail(ARK_ERR_PARAM, "out is NULL");
    const size_t n = (size_t)ctx->g.C1 * ctx->g.C2 * ctx->g.C3 * 3;
    double *d = nullptr;
    ARK_CUDA(cudaMallocAsync((void **)&d, sizeof(double) * n, ctx->st));
    CellPack a;
    std::memset(&a, 0, sizeof a);
    a.r = d;
    a.k0 = 1;
    a.k1 = ctx->g.C3 + 1;
    ctx->eng->pack(ctx->con ^ 1, ctx->fcur, a);
    int rc = launch_status(ctx);
    if (!rc && cudaMemcpyAsync(out, d, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->st) != cudaSuccess)
        rc = fail(ARK_ERR_CUDA, "vorticity copy failed");
    cudaFreeAsync(d, ctx->st);
    if (!rc) ARK_CUDA(cudaStreamSynchronize(ctx->st));
    return rc;
}

} // extern "C"
