// Slab groups: one channel split along z into slabs, each an ark_ctx of its own, stepped
// together with the reference's two halo exchanges per step and one shared set of reductions.
//
// The reference decomposes its domain over MPI ranks (main.cpp:53-67, MPI_Cart_create) and
// exchanges one-plane halos at two points of every step: u1Con, u2Con, u3Con before the stress
// (main.cpp:601-801) and the twelve fields before Phase2 (main.cpp:1049-1631), with dt reduced
// by MPI_Allreduce(MIN) (main.cpp:412).  Here a slab keeps its x wrap (and its y walls) as a
// single context does, and leaves its z ghosts to the group: before the stress the "Con"
// velocities and density, before Phase2 the half-step level, the old density and the faces
// normal to z are copied plane by plane from the neighbouring slabs (periodic z wraps around
// the group; a bounded z copies zero-gradient at the group's ends), as k_wrap does for one
// domain.  The reductions are exact: every slab folds max |u| (as integer bit patterns) and the
// fixed-point u1 sum into one shared set of partial slots, so dt and the bulk force are those of
// the whole domain, and the group's result is the single context's bit for bit.
//
// All slabs live on one device and one stream, and a step is one CUDA graph (one per face
// generation).  The halo copies read the neighbours' interior planes and write ghost planes
// only, so one kernel launch performs a whole exchange.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "ark_ctx.h"

using namespace ark;

namespace ark {
Consts make_run_consts(const ark_params &p); // ark_api.cu
}

struct ark_slabs {
    ark_params P; // the whole domain
    int n = 0;
    std::vector<ark_ctx *> ctx;
    std::vector<SlabRange> R;
    cudaStream_t st = nullptr;
    DevScalars *sc = nullptr;
    unsigned long long *part_max = nullptr;
    long long *part_sum = nullptr;
    HaloJob *jobs[2][2][2] = {};    // [x][fcur][exchange], device tables
    int njobs[2][2][2] = {};
    cudaGraphExec_t graph[2][2] = {}; // [x][fcur]
    int con = 0, fcur = 0;
    bool uploaded = false, parts_valid = false;
    long long nfluid = 0;
    std::vector<double> cond_host;
};

namespace {

int slabs_fail(int status, const std::string &msg) { return api_fail(status, "slabs: " + msg); }

#define SLAB_CUDA(call)                                                                          \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) return slabs_fail(ARK_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

size_t cell_plane(const ark_params &p) { return (size_t)(p.n1_cells + 2) * (p.n2_cells + 2); }
size_t face_plane(const ark_params &p) { return (size_t)(p.n1_cells + 3) * (p.n2_cells + 3); }

// Member q of a host state: its 24 pointers in declaration order, the 9 cell arrays first.
double **member(ark_host_state &h, int q) { return &(&h.roCon)[q]; }

// The slab's window of a whole-domain host state: cell planes k_first-1 .. k_last+1 and face
// planes k_first-1 .. k_last+2 are contiguous in the Arr3d layout (k slowest).
ark_host_state window(const ark_slabs *G, const ark_host_state &h, int s) {
    ark_host_state v = h;
    const size_t off_c = (size_t)(G->R[s].k_first - 1) * cell_plane(G->P);
    const size_t off_f = (size_t)(G->R[s].k_first - 1) * face_plane(G->P);
    for (int q = 0; q < 24; ++q) {
        double **m = member(v, q);
        if (*m) *m += q < 9 ? off_c : off_f;
    }
    return v;
}

// Job tables of both exchanges for "Con" = level x and face generation fc.
int build_jobs(ark_slabs *G, int x, int fc) {
    for (int e = 0; e < 2; ++e) {
        std::vector<HaloJob> jobs;
        std::vector<std::vector<void *>> arrays(G->n, std::vector<void *>(16));
        std::vector<std::vector<int>> faces(G->n, std::vector<int>(16));
        int na = -1;
        for (int s = 0; s < G->n; ++s) {
            const int m = G->ctx[s]->eng->halo_arrays(e, x, fc, arrays[s].data(), faces[s].data());
            if (na >= 0 && m != na) return slabs_fail(ARK_ERR_STATE, "slabs list different halo arrays");
            na = m;
        }
        for (int s = 0; s < G->n; ++s) {
            const int c3 = G->R[s].k_last - G->R[s].k_first + 1;
            for (int side = 0; side < 2; ++side) {
                const int nb = side ? G->R[s].above : G->R[s].below;
                const bool bounded = nb < 0;
                const int src = bounded ? s : nb;
                const int c3_src = G->R[src].k_last - G->R[src].k_first + 1;
                for (int q = 0; q < na; ++q) {
                    const HaloPlanes hp = halo_planes(faces[s][q], side, c3, c3_src, bounded);
                    HaloJob j;
                    j.dst = arrays[s][q];
                    j.src = arrays[src][q];
                    j.dst_plane = hp.dst;
                    j.src_plane = hp.src;
                    j.face = faces[s][q];
                    j.dst_planes = c3 + 2 + faces[s][q];
                    j.src_planes = c3_src + 2 + faces[s][q];
                    j.pad = 0;
                    jobs.push_back(j);
                }
            }
        }
        if (G->jobs[x][fc][e]) cudaFree(G->jobs[x][fc][e]);
        G->jobs[x][fc][e] = nullptr;
        SLAB_CUDA(cudaMalloc(&G->jobs[x][fc][e], sizeof(HaloJob) * std::max<size_t>(1, jobs.size())));
        SLAB_CUDA(cudaMemcpy(G->jobs[x][fc][e], jobs.data(), sizeof(HaloJob) * jobs.size(), cudaMemcpyHostToDevice));
        G->njobs[x][fc][e] = (int)jobs.size();
    }
    return ARK_OK;
}

// One step of the group, in the order of main.cpp:82-91, with the two exchanges.
void enqueue_step(ark_slabs *G, int x, int fc) {
    Engine *e0 = G->ctx[0]->eng.get();
    e0->stage(0, x, fc); // dt and the bulk force of the whole domain (shared slots and scalars)
    for (ark_ctx *c : G->ctx) c->eng->stage(1, x, fc);
    e0->halo_exchange(G->jobs[x][fc][0], G->njobs[x][fc][0]);
    for (ark_ctx *c : G->ctx) c->eng->stage(2, x, fc);
    for (ark_ctx *c : G->ctx) c->eng->stage(3, x, fc);
    e0->halo_exchange(G->jobs[x][fc][1], G->njobs[x][fc][1]);
    for (ark_ctx *c : G->ctx) c->eng->stage(4, x, fc);
}

int ensure_graph(ark_slabs *G) {
    const int x = G->con, fc = G->fcur;
    if (G->graph[x][fc]) return ARK_OK;
    if (int rc = build_jobs(G, x, fc)) return rc;
    cudaGraph_t graph = nullptr;
    SLAB_CUDA(cudaStreamBeginCapture(G->st, cudaStreamCaptureModeThreadLocal));
    enqueue_step(G, x, fc);
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(G->st, &graph);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return slabs_fail(ARK_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString(le != cudaSuccess ? le : ce));
    }
    cudaError_t ie = cudaGraphInstantiate(&G->graph[x][fc], graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        G->graph[x][fc] = nullptr;
        return slabs_fail(ARK_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
    }
    return ARK_OK;
}

void sync_ctx_levels(ark_slabs *G) {
    for (ark_ctx *c : G->ctx) {
        c->con = G->con;
        c->fcur = G->fcur;
    }
}

} // namespace

extern "C" {

int ark_slab_plan(int n3_cells, int nslabs, int slab, int periodic_z, int *k_first, int *k_last, int *below,
                  int *above) {
    if (n3_cells < 1 || nslabs < 1 || nslabs > n3_cells || slab < 0 || slab >= nslabs || !k_first || !k_last ||
        !below || !above)
        return api_fail(ARK_ERR_PARAM, "ark_slab_plan: bad arguments");
    const SlabRange R = slab_range(n3_cells, nslabs, slab, periodic_z != 0);
    *k_first = R.k_first;
    *k_last = R.k_last;
    *below = R.below;
    *above = R.above;
    return ARK_OK;
}

int ark_slab_halo_planes(int face, int side, int c3, int c3_src, int bounded, int *dst_plane, int *src_plane) {
    if (c3 < 1 || c3_src < 1 || side < 0 || side > 1 || !dst_plane || !src_plane)
        return api_fail(ARK_ERR_PARAM, "ark_slab_halo_planes: bad arguments");
    const HaloPlanes h = halo_planes(face != 0, side, c3, c3_src, bounded != 0);
    *dst_plane = h.dst;
    *src_plane = h.src;
    return ARK_OK;
}

int ark_slabs_destroy(ark_slabs *G) {
    if (!G) return ARK_OK;
    if (G->st) cudaStreamSynchronize(G->st);
    for (auto &a : G->graph)
        for (auto &g : a)
            if (g) cudaGraphExecDestroy(g);
    for (auto &a : G->jobs)
        for (auto &b : a)
            for (HaloJob *j : b)
                if (j) cudaFree(j);
    for (ark_ctx *c : G->ctx) {
        if (!c) continue;
        c->st = nullptr; // the group's stream, destroyed below
        ark_destroy(c);
    }
    if (G->sc) cudaFree(G->sc);
    if (G->part_max) cudaFree(G->part_max);
    if (G->part_sum) cudaFree(G->part_sum);
    if (G->st) cudaStreamDestroy(G->st);
    delete G;
    return ARK_OK;
}

ark_slabs *ark_slabs_create(const ark_params *params, int nslabs, int *status) {
    int dummy;
    if (!status) status = &dummy;
    if (!params) {
        *status = slabs_fail(ARK_ERR_PARAM, "params is NULL");
        return nullptr;
    }
    if (nslabs < 1 || nslabs > params->n3_cells) {
        *status = slabs_fail(ARK_ERR_PARAM, "need 1 <= nslabs <= n3_cells");
        return nullptr;
    }
    ark_slabs *G = new ark_slabs();
    G->P = *params;
    G->n = nslabs;
    auto bail = [&](int rc) {
        *status = rc;
        ark_slabs_destroy(G);
        return (ark_slabs *)nullptr;
    };
    if (cudaSetDevice(params->device) != cudaSuccess) return bail(slabs_fail(ARK_ERR_CUDA, "cudaSetDevice failed"));
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (cudaStreamCreateWithPriority(&G->st, cudaStreamNonBlocking, hi) != cudaSuccess)
        return bail(slabs_fail(ARK_ERR_CUDA, "cudaStreamCreate failed"));
    if (cudaMalloc(&G->sc, sizeof(DevScalars)) != cudaSuccess ||
        cudaMalloc(&G->part_max, sizeof(unsigned long long) * 3 * kBuckets) != cudaSuccess ||
        cudaMalloc(&G->part_sum, sizeof(long long) * kBuckets) != cudaSuccess)
        return bail(slabs_fail(ARK_ERR_NOMEM, "shared scalars"));
    cudaMemset(G->sc, 0, sizeof(DevScalars));
    cudaMemset(G->part_max, 0, sizeof(unsigned long long) * 3 * kBuckets);
    cudaMemset(G->part_sum, 0, sizeof(long long) * kBuckets);
    // the whole domain's run constants (dx3 = lz / C3, not a slab's own), z ghosts from outside
    Consts K = make_run_consts(*params);
    K.ext_z = 1;
    for (int s = 0; s < nslabs; ++s) {
        G->R.push_back(slab_range(params->n3_cells, nslabs, s, params->periodic_z != 0));
        ark_params ps = *params;
        ps.n3_cells = G->R[s].k_last - G->R[s].k_first + 1;
        ps.lz = params->lz * ps.n3_cells / params->n3_cells;
        ps.keep_stress = 0;
        int rc = ARK_OK;
        ark_ctx *c = ark_create(&ps, &rc);
        if (!c) return bail(rc);
        G->ctx.push_back(c);
        c->k = K;
        c->eng->set_consts(K);
        c->p2mode = 0; // the three sweep kernels (the one-kernel forms rotate levels per launch)
        if (c->march[0] == 6) c->march[0] = 4; // 128 x 2 tiles pay off only with the x1 sweep folded in
        cudaStreamDestroy(c->st);
        c->st = G->st;
        c->eng->share_scalars(G->sc, G->part_max, G->part_sum);
    }
    *status = ARK_OK;
    return G;
}

int ark_slabs_count(const ark_slabs *G) { return G ? G->n : 0; }

int ark_slabs_upload(ark_slabs *G, const ark_host_state *host) {
    if (!G || !host) return slabs_fail(ARK_ERR_PARAM, "NULL argument");
    if (!host->condition) return slabs_fail(ARK_ERR_PARAM, "host->condition is NULL");
    for (int s = 0; s < G->n; ++s) {
        const ark_host_state v = window(G, *host, s);
        if (int rc = ark_upload(G->ctx[s], &v)) return rc;
    }
    // fluid cells of the whole domain (each slab's upload counted its own)
    const Geom hg = host_geom(G->P.n1_cells, G->P.n2_cells, G->P.n3_cells);
    long long nfluid = 0;
    for (int k = 1; k <= hg.C3; ++k)
        for (int j = 1; j <= hg.C2; ++j)
            for (int i = 1; i <= hg.C1; ++i)
                if (host->condition[hg.cell(i, j, k)] == 0) ++nfluid;
    G->nfluid = nfluid;
    G->cond_host.assign(host->condition, host->condition + (size_t)hg.ncell());
    DevScalars sc;
    std::memset(&sc, 0, sizeof sc);
    sc.nfluid = nfluid;
    SLAB_CUDA(cudaMemcpy(G->sc, &sc, sizeof sc, cudaMemcpyHostToDevice));
    G->con = G->fcur = 0;
    sync_ctx_levels(G);
    G->uploaded = true;
    G->parts_valid = false;
    return ARK_OK;
}

int ark_slabs_download(ark_slabs *G, ark_host_state *host) {
    if (!G || !host) return slabs_fail(ARK_ERR_PARAM, "NULL argument");
    if (!G->uploaded) return slabs_fail(ARK_ERR_STATE, "no state uploaded");
    SLAB_CUDA(cudaStreamSynchronize(G->st));
    sync_ctx_levels(G);
    const size_t cp = cell_plane(G->P), fp = face_plane(G->P);
    for (int s = 0; s < G->n; ++s) {
        const int c3 = G->R[s].k_last - G->R[s].k_first + 1;
        // the slab's own arrays, downloaded whole, then its planes placed into the domain's
        std::vector<std::vector<double>> tmp(24);
        ark_host_state t;
        std::memset(&t, 0, sizeof t);
        for (int q = 0; q < 24; ++q) {
            if (q == 8 || !*member(*host, q)) continue;
            tmp[q].resize((q < 9 ? cp * (c3 + 2) : fp * (c3 + 3)));
            *member(t, q) = tmp[q].data();
        }
        if (int rc = ark_download(G->ctx[s], &t)) return rc;
        const int kf = G->R[s].k_first;
        const bool first = s == 0, last = s == G->n - 1;
        for (int q = 0; q < 24; ++q) {
            if (q == 8 || !*member(*host, q)) continue;
            double *dst = *member(*host, q);
            const size_t pl = q < 9 ? cp : fp;
            const int lo = first ? 0 : 1;                              // local planes kept
            const int hi = last ? (q < 9 ? c3 + 1 : c3 + 2) : c3;
            std::memcpy(dst + (size_t)(kf - 1 + lo) * pl, tmp[q].data() + (size_t)lo * pl, sizeof(double) * pl * (hi - lo + 1));
        }
    }
    if (host->condition) std::memcpy(host->condition, G->cond_host.data(), sizeof(double) * G->cond_host.size());
    return ARK_OK;
}

int ark_slabs_step(ark_slabs *G, int nsteps) {
    if (!G) return slabs_fail(ARK_ERR_PARAM, "NULL group");
    if (!G->uploaded) return slabs_fail(ARK_ERR_STATE, "no state uploaded");
    if (nsteps < 0) return slabs_fail(ARK_ERR_PARAM, "nsteps < 0");
    if (!G->parts_valid) {
        SLAB_CUDA(cudaMemsetAsync(G->part_max, 0, sizeof(unsigned long long) * 3 * kBuckets, G->st));
        SLAB_CUDA(cudaMemsetAsync(G->part_sum, 0, sizeof(long long) * kBuckets, G->st));
        sync_ctx_levels(G);
        for (ark_ctx *c : G->ctx) c->eng->reduce_into(G->con);
        G->parts_valid = true;
    }
    for (int s = 0; s < nsteps; ++s) {
        if (int rc = ensure_graph(G)) return rc;
        SLAB_CUDA(cudaGraphLaunch(G->graph[G->con][G->fcur], G->st));
        G->fcur ^= 1;
    }
    sync_ctx_levels(G);
    return ARK_OK;
}

int ark_slabs_sync(ark_slabs *G) {
    if (!G) return slabs_fail(ARK_ERR_PARAM, "NULL group");
    SLAB_CUDA(cudaStreamSynchronize(G->st));
    int status = 0;
    SLAB_CUDA(cudaMemcpy(&status, &G->sc->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (status & STATUS_NONFINITE) return slabs_fail(ARK_ERR_NONFINITE, "non-finite velocity detected on the device");
    return ARK_OK;
}

int ark_slabs_time_steps(ark_slabs *G, int nsteps, double *ms) {
    if (!G || !ms) return slabs_fail(ARK_ERR_PARAM, "NULL argument");
    if (!G->uploaded) return slabs_fail(ARK_ERR_STATE, "no state uploaded");
    // both face-generation graphs outside the timed region
    if (int rc = ensure_graph(G)) return rc;
    G->fcur ^= 1;
    int rc2 = ensure_graph(G);
    G->fcur ^= 1;
    if (rc2) return rc2;
    if (int rc = ark_slabs_step(G, 0)) return rc;
    cudaEvent_t a, b;
    SLAB_CUDA(cudaEventCreate(&a));
    SLAB_CUDA(cudaEventCreate(&b));
    cudaStreamSynchronize(G->st);
    cudaEventRecord(a, G->st);
    int rc = ark_slabs_step(G, nsteps);
    cudaEventRecord(b, G->st);
    cudaEventSynchronize(b);
    float f = 0.f;
    cudaEventElapsedTime(&f, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = f;
    if (rc) return rc;
    return ark_slabs_sync(G);
}

int ark_slabs_get_scalars(ark_slabs *G, ark_scalars *out) {
    if (!G || !out) return slabs_fail(ARK_ERR_PARAM, "NULL argument");
    if (!G->uploaded) return slabs_fail(ARK_ERR_STATE, "no state uploaded");
    return ark_get_scalars(G->ctx[0], out); // the shared scalar block
}

int ark_slabs_conservation_sums(ark_slabs *G, ark_sums *out) {
    if (!G || !out) return slabs_fail(ARK_ERR_PARAM, "NULL argument");
    if (!G->uploaded) return slabs_fail(ARK_ERR_STATE, "no state uploaded");
    SLAB_CUDA(cudaMemsetAsync(&G->sc->sums[0], 0, sizeof(long long) * 6, G->st));
    for (ark_ctx *c : G->ctx) c->eng->sums(G->con ^ 1); // every slab adds into the shared sums
    SLAB_CUDA(cudaGetLastError());
    long long v[6];
    SLAB_CUDA(cudaStreamSynchronize(G->st));
    SLAB_CUDA(cudaMemcpy(v, &G->sc->sums[0], sizeof v, cudaMemcpyDeviceToHost));
    const double q = 1.0 / 4294967296.0;
    out->mass = (double)v[0] * q;
    out->momentum1 = (double)v[1] * q;
    out->momentum2 = (double)v[2] * q;
    out->momentum3 = (double)v[3] * q;
    out->kinetic = (double)v[4] * q;
    out->cells = v[5];
    return ARK_OK;
}

} // extern "C"
