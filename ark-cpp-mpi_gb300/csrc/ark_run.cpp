// ark_run: the reference's main() time loop (source/main.cpp:53-116) on the GPU library.
//
//   ark_run [--grid C1 C2 C3] [--steps N] [--print P] [--re RE] [--sound C] [--cfl CFL]
//           [--fp32] [--seed S] [--amp A] [--no-forcing] [--per-phase]
//
// Sets up the seeded channel (periodic x/z, walls in y) instead of the reference's hard-coded
// backward-facing step (Input/InitializeData, main.cpp:118-372), advances N steps and prints
// the reference's step line (main.cpp:102) every P steps and its "Program time" line
// (main.cpp:111), plus throughput.  --per-phase calls the step pieces one by one, in the
// order of main.cpp:82-91, instead of the fused graph step.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ark_gpu.h"

namespace {

struct HostState {
    std::vector<std::vector<double>> store;
    ark_host_state s{};
    explicit HostState(const ark_params &p) {
        const size_t nc = ark_cell_count(&p), nf = ark_face_count(&p);
        double **cells[] = {&s.roCon, &s.u1Con, &s.u2Con, &s.u3Con, &s.ronCon, &s.u1nCon, &s.u2nCon, &s.u3nCon,
                            &s.condition};
        double **faces[] = {&s.p1, &s.ro1, &s.u11, &s.u21, &s.u31, &s.p2, &s.ro2, &s.u12,
                            &s.u22, &s.u32, &s.p3, &s.ro3, &s.u13, &s.u23, &s.u33};
        store.reserve(24);
        for (double **c : cells) {
            store.emplace_back(nc);
            *c = store.back().data();
        }
        for (double **f : faces) {
            store.emplace_back(nf);
            *f = store.back().data();
        }
    }
};

int die(const char *what, int rc) {
    std::fprintf(stderr, "%s: %s (%s)\n", what, ark_status_string(rc), ark_last_error());
    return 1;
}

} // namespace

int main(int argc, char **argv) {
    ark_params p{};
    p.n1_cells = 64;
    p.n2_cells = 32;
    p.n3_cells = 32;
    p.lx = 2 * M_PI;
    p.ly = 2.0;
    p.lz = M_PI;
    double re = 2800.0;
    p.sound = 10.0;
    p.ro0 = 1.0;
    p.cfl = 0.2;
    p.periodic_x = p.periodic_z = 1;
    p.precision = ARK_FP64;
    p.forcing = 1;
    p.u_target = 1.0;
    int steps = 100, nprint = 10, per_phase = 0;
    unsigned long long seed = 12345;
    double amp = 0.1;
    for (int a = 1; a < argc; ++a) {
        if (!std::strcmp(argv[a], "--grid") && a + 3 < argc) {
            p.n1_cells = std::atoi(argv[++a]);
            p.n2_cells = std::atoi(argv[++a]);
            p.n3_cells = std::atoi(argv[++a]);
        } else if (!std::strcmp(argv[a], "--steps") && a + 1 < argc) steps = std::atoi(argv[++a]);
        else if (!std::strcmp(argv[a], "--print") && a + 1 < argc) nprint = std::atoi(argv[++a]);
        else if (!std::strcmp(argv[a], "--re") && a + 1 < argc) re = std::atof(argv[++a]);
        else if (!std::strcmp(argv[a], "--sound") && a + 1 < argc) p.sound = std::atof(argv[++a]);
        else if (!std::strcmp(argv[a], "--cfl") && a + 1 < argc) p.cfl = std::atof(argv[++a]);
        else if (!std::strcmp(argv[a], "--seed") && a + 1 < argc) seed = std::strtoull(argv[++a], nullptr, 10);
        else if (!std::strcmp(argv[a], "--amp") && a + 1 < argc) amp = std::atof(argv[++a]);
        else if (!std::strcmp(argv[a], "--fp32")) p.precision = ARK_FP32;
        else if (!std::strcmp(argv[a], "--no-forcing")) p.forcing = 0;
        else if (!std::strcmp(argv[a], "--per-phase")) per_phase = 1;
        else {
            std::fprintf(stderr, "unknown or incomplete argument: %s\n", argv[a]);
            return 2;
        }
    }
    p.vis = 1.0 / re;
    if (nprint < 1) nprint = 1;

    HostState hs(p);
    int rc = ark_channel_init(&p, seed, amp, &hs.s);
    if (rc) return die("ark_channel_init", rc);
    ark_ctx *ctx = ark_create(&p, &rc);
    if (!ctx) return die("ark_create", rc);
    if ((rc = ark_upload(ctx, &hs.s))) return die("ark_upload", rc);

    const auto t0 = std::chrono::steady_clock::now();
    int done = 0;
    while (done < steps) {
        const int n = std::min(nprint, steps - done);
        if (per_phase) {
            ark_scalars sc;
            for (int s = 0; s < n; ++s) {
                if ((rc = ark_get_scalars(ctx, &sc))) return die("ark_get_scalars", rc);
                if ((rc = ark_time_step_size(ctx))) return die("ark_time_step_size", rc);
                double dt_now;
                {
                    ark_scalars t;
                    ark_get_scalars(ctx, &t);
                    dt_now = t.dt;
                    t.nstep = sc.nstep + 1;
                    t.time = sc.time + 0.5 * dt_now;
                    ark_set_scalars(ctx, &t);
                }
                if ((rc = ark_phase1(ctx))) return die("ark_phase1", rc);
                if ((rc = ark_stress_tensor(ctx))) return die("ark_stress_tensor", rc);
                if ((rc = ark_use_forces(ctx))) return die("ark_use_forces", rc);
                if ((rc = ark_phase2(ctx))) return die("ark_phase2", rc);
                if ((rc = ark_phase1(ctx))) return die("ark_phase1", rc);
                if ((rc = ark_use_forces(ctx))) return die("ark_use_forces", rc);
                ark_scalars t;
                ark_get_scalars(ctx, &t);
                t.time += 0.5 * dt_now;
                ark_set_scalars(ctx, &t);
            }
        } else if ((rc = ark_step(ctx, n))) {
            return die("ark_step", rc);
        }
        if ((rc = ark_sync(ctx))) return die("ark_sync", rc);
        done += n;
        ark_scalars sc;
        ark_get_scalars(ctx, &sc);
        ark_sums sums;
        ark_conservation_sums(ctx, &sums);
        std::printf("step: %lld dt:%E time:%8.4f U_b:%.12f mass:%.12e\n", sc.nstep, sc.dt, sc.time,
                    sc.bulk_velocity, sums.mass);
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const double cells = (double)p.n1_cells * p.n2_cells * p.n3_cells;
    std::printf("Program time: %8.3f\n", secs);
    std::printf("Mcell-steps/s: %.2f\n", cells * steps / secs / 1e6);
    ark_destroy(ctx);
    return 0;
}
