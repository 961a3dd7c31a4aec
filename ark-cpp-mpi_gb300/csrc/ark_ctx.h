// Internal: the context behind the C ABI's ark_ctx and its precision-independent engine
// interface, shared by the ABI (ark_api.cu) and the slab groups (ark_slabs.cu).
#pragma once
#include <memory>
#include <vector>

#include "../../include/ark_gpu.h"
#include "ark_state.h"

namespace ark {

// Precision-independent engine interface.
struct Engine {
    virtual ~Engine() {}
    virtual int alloc() = 0;
    virtual int upload_field(int which, int face, const double *host) = 0;
    virtual int download_field(int which, int face, double *host) = 0;
    virtual void *field_ptr(const char *name, int *face) = 0;
    virtual int download_raw(void *p, int face, double *host) = 0;
    virtual int upload_raw(void *p, int face, const double *host) = 0;
    virtual void time_step_size(int con, int advance) = 0;
    virtual void reduce(int con) = 0;
    virtual void phase1(int src, int dst, int fcur, int mode) = 0;
    virtual void stress(int con, int bulk) = 0;
    virtual void use_forces(int ncon) = 0;
    virtual void phase2(int con, int fcur) = 0;
    virtual void step(int con, int fcur, cudaEvent_t *ev) = 0;
    virtual void boundary_fill(int ncon, int axis, int periodic) = 0;
    virtual void sums(int ncon) = 0;
    virtual void mean_profile(int ncon, long long *acc) = 0;
    virtual void pack(int ncon, int fcur, const CellPack &a) = 0;
    virtual int alloc_nut() = 0;
    virtual void plane_stats(int ncon, double *out) = 0;
    virtual void gather(int lvl, double *u0, double *u1, double *u2) = 0;
    virtual void average_add(int ncon) = 0;
    virtual void energy(int ncon, double *scratch, double *out) = 0;
    virtual DevScalars *scalars() = 0;
    virtual uint8_t *flags() = 0;
    // launches of one step in the current configuration, and their names
    virtual int step_launches() = 0;
    virtual const char *step_kernel_name(int q) = 0;
    // after each step: the level the step wrote into the spare takes the place of "nCon"
    virtual void after_step(int con) = 0;
    // identity of the cell-level buffers (0, 1: the two levels, 2: the spare), for graph reuse
    virtual const void *level_ptr(int l) = 0;

    // ---- slab groups (ark_slabs.cu) ----
    // run constants (a slab takes the whole domain's, with ext_z set)
    virtual void set_consts(const Consts &k) = 0;
    // the scalar block and the dt / bulk-flow partial slots: one set shared by all slabs
    virtual void share_scalars(DevScalars *sc, unsigned long long *part_max, long long *part_sum) = 0;
    // the partials of the step start into the shared slots (not cleared here)
    virtual void reduce_into(int con) = 0;
    // stage q of the fused step with "Con" = level x at entry (the three separate Phase2
    // sweeps): 0 dt and bulk force, 1 ghost fill of the "Con" level, 2 Phase1 with stress and
    // forces, 3 the ghost fill before Phase2, 4 the sweeps and the second Phase1
    virtual void stage(int q, int x, int fcur) = 0;
    // the arrays a z split exchanges before the stress (exchange 0: u1, u2, u3 and ro of the
    // level Phase1 reads) or before Phase2 (1: u1, u2, u3, ro of the level Phase1 wrote, ro of
    // the other level, and the faces normal to z); *face[q] says which are face arrays.
    // Returns the count.
    virtual int halo_arrays(int exchange, int x, int fcur, void **ptrs, int *face) = 0;
    virtual void halo_exchange(const HaloJob *jobs, int njobs) = 0;
    // the TMA staging's bounded-wait check (Launch<T>::staging_unmet): 1 launched, 0 unavailable
    virtual int staging_unmet(int x, int fcur) = 0;
};


} // namespace ark

struct ark_ctx {
    ark_params P;
    ark::Geom g;
    ark::Consts k;
    cudaStream_t st = nullptr;
    std::unique_ptr<ark::Engine> eng;
    double *cond_dev = nullptr; // the last uploaded condition array (host layout), on the device
    int con = 0;  // the cell level holding "Con"
    int fcur = 0; // the current face generation
    bool uploaded = false;
    bool parts_valid = false; // the dt / bulk-flow partials describe the current state
    int march[2] = {1, 0};    // Phase1 kernel shape of the two Phase1 launches of a step
    cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}}; // [con][fcur]
    const void *graph_levels[2][2][3] = {};  // the level buffers each graph was captured with
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double *stage = nullptr; // contiguous double staging for host transfers
    ark::AvgArrays avg = {{nullptr, nullptr, nullptr}}; // averageU1..3 (FP64, reference layout)
    bool averaging = false;  // AverageValues at the end of every step
    void *closure_net = nullptr;          // learned closure: the network's constants (device copy)
    cudaStream_t side = nullptr;          // the closure's branch of the step
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaStream_t fill = nullptr;          // the captured step's ghost fill, beside dt
    cudaEvent_t fill_fork = nullptr, fill_join = nullptr;
    cudaEvent_t seam_fork = nullptr, seam_join = nullptr; // the seam kernel on `fill`, beside the x2 and x3 sweeps
    float closure_scale = 0.f;            // u_tau / vis for the y+ feature
    int seg_target = 32;                  // x2/x3 sweep segment length (faces)
    int x1_lines = 0;                     // x1 sweep lines per warp (0: x_lines_per_warp's choice)
    int p1_chunk = 0;                     // planes per block of the staged / face-centric Phase1 (0: default)
    int p2mode = 0; // Phase2: 0 three sweep kernels, 1 one kernel for the three sweeps, 2 (FP32)
                    // one kernel for the three sweeps and the second Phase1, 3 (FP32) the same
                    // with TMA tensor copies, 4 (FP32, TMA-staged Phase1 + stress) the x1 sweep
                    // folded into Phase1 + stress (a seam kernel finishes it), then the x2 and
                    // x3 sweeps, 5 the x1 and x3 sweeps folded in (two seam kernels), then the
                    // x2 sweep
    // output streaming: two device and two pinned host slab buffers of io_cap doubles
    double *io_dev[2] = {nullptr, nullptr};
    double *io_host[2] = {nullptr, nullptr};
    size_t io_cap = 0;
};

