// Host-only helpers of libark_gb300.so (no GPU needed): the seeded channel-flow initial
// state.  The reference builds its initial state in InitializeData (main.cpp:280-372) for
// its backward-facing-step case; the channel below is this project's own definition,
// shared bit-for-bit by the GPU runs and the CPU oracle runs it is compared with.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/ark_gpu.h"

namespace {

// Vigna's splitmix64: state += golden gamma, then two xor-shift-multiply rounds.
struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    uint64_t next() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // top 53 bits scaled to [0, 1)
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

} // namespace

extern "C" int ark_channel_init(const ark_params *p, uint64_t seed, double amp, ark_host_state *out) {
    if (!p || !out) return ARK_ERR_PARAM;
    const int C1 = p->n1_cells, C2 = p->n2_cells, C3 = p->n3_cells;
    if (C1 < 1 || C2 < 1 || C3 < 1) return ARK_ERR_PARAM;
    double *all[] = {out->roCon, out->u1Con, out->u2Con, out->u3Con, out->ronCon, out->u1nCon, out->u2nCon,
                     out->u3nCon, out->condition, out->p1, out->ro1, out->u11, out->u21, out->u31,
                     out->p2, out->ro2, out->u12, out->u22, out->u32, out->p3, out->ro3, out->u13,
                     out->u23, out->u33};
    for (double *a : all)
        if (!a) return ARK_ERR_PARAM;
    const int64_t N1 = C1 + 2, N2 = C2 + 2, M1 = C1 + 3, M2 = C2 + 3;
    const size_t nc = (size_t)N1 * N2 * (C3 + 2), nf = (size_t)M1 * M2 * (C3 + 3);
    auto cell = [&](int i, int j, int k) { return ((size_t)k * N2 + j) * N1 + i; };
    auto face = [&](int i, int j, int k) { return ((size_t)k * M2 + j) * M1 + i; };

    std::vector<double> u[3];
    for (int m = 0; m < 3; ++m) u[m].assign(nc, 0.0);
    std::vector<double> ro(nc, p->ro0);
    const double ub = p->u_target, ly = p->ly;
    const double dy = (0.5 * ly - -0.5 * ly) / C2;
    SplitMix64 rng(seed);
    for (int k = 1; k <= C3; ++k)
        for (int j = 1; j <= C2; ++j) {
            const double y = -0.5 * ly + ((double)j - 0.5) * dy;
            const double base = 1.5 * ub * (1.0 - y * y);
            for (int i = 1; i <= C1; ++i) {
                const double r1 = rng.uniform(), r2 = rng.uniform(), r3 = rng.uniform();
                const size_t c = cell(i, j, k);
                u[0][c] = base + amp * (2.0 * r1 - 1.0);
                u[1][c] = amp * (2.0 * r2 - 1.0);
                u[2][c] = amp * (2.0 * r3 - 1.0);
            }
        }
    // periodic ghost copies in x, then z
    std::vector<double> *fields[4] = {&u[0], &u[1], &u[2], &ro};
    for (auto *a : fields) {
        std::vector<double> &v = *a;
        for (int k = 1; k <= C3; ++k)
            for (int j = 1; j <= C2; ++j) {
                v[cell(0, j, k)] = v[cell(C1, j, k)];
                v[cell(C1 + 1, j, k)] = v[cell(1, j, k)];
            }
        for (int j = 1; j <= C2; ++j)
            for (int i = 1; i <= C1; ++i) {
                v[cell(i, j, 0)] = v[cell(i, j, C3)];
                v[cell(i, j, C3 + 1)] = v[cell(i, j, 1)];
            }
    }
    for (int lvl = 0; lvl < 2; ++lvl) {
        double *r = lvl ? out->ronCon : out->roCon;
        double *a = lvl ? out->u1nCon : out->u1Con;
        double *b = lvl ? out->u2nCon : out->u2Con;
        double *c = lvl ? out->u3nCon : out->u3Con;
        std::memcpy(r, ro.data(), nc * sizeof(double));
        std::memcpy(a, u[0].data(), nc * sizeof(double));
        std::memcpy(b, u[1].data(), nc * sizeof(double));
        std::memcpy(c, u[2].data(), nc * sizeof(double));
    }
    for (size_t c = 0; c < nc; ++c) out->condition[c] = 0.0;
    for (int k = 0; k < C3 + 2; ++k)
        for (int i = 0; i < C1 + 2; ++i) {
            out->condition[cell(i, 0, k)] = 1.0;
            out->condition[cell(i, C2 + 1, k)] = 1.0;
        }

    double *P[3] = {out->p1, out->p2, out->p3};
    double *R[3] = {out->ro1, out->ro2, out->ro3};
    double *U[3][3] = {{out->u11, out->u21, out->u31}, {out->u12, out->u22, out->u32}, {out->u13, out->u23, out->u33}};
    for (int d = 0; d < 3; ++d) {
        std::memset(P[d], 0, nf * sizeof(double));
        std::memset(R[d], 0, nf * sizeof(double));
        for (int m = 0; m < 3; ++m) std::memset(U[d][m], 0, nf * sizeof(double));
    }
    // faces normal to x1: i = 1..C1+1 between cells i-1 and i
    for (int k = 1; k <= C3; ++k)
        for (int j = 1; j <= C2; ++j)
            for (int i = 1; i <= C1 + 1; ++i) {
                const size_t f = face(i, j, k);
                R[0][f] = p->ro0;
                for (int m = 0; m < 3; ++m) U[0][m][f] = 0.5 * (u[m][cell(i - 1, j, k)] + u[m][cell(i, j, k)]);
            }
    // faces normal to x2: j = 1..C2+1, walls at j = 1 and C2+1 keep u = 0
    for (int k = 1; k <= C3; ++k)
        for (int j = 1; j <= C2 + 1; ++j)
            for (int i = 1; i <= C1; ++i) {
                const size_t f = face(i, j, k);
                R[1][f] = p->ro0;
                if (j == 1 || j == C2 + 1) continue;
                for (int m = 0; m < 3; ++m) U[1][m][f] = 0.5 * (u[m][cell(i, j - 1, k)] + u[m][cell(i, j, k)]);
            }
    // faces normal to x3: k = 1..C3+1 between cells k-1 and k
    for (int k = 1; k <= C3 + 1; ++k)
        for (int j = 1; j <= C2; ++j)
            for (int i = 1; i <= C1; ++i) {
                const size_t f = face(i, j, k);
                R[2][f] = p->ro0;
                for (int m = 0; m < 3; ++m) U[2][m][f] = 0.5 * (u[m][cell(i, j, k - 1)] + u[m][cell(i, j, k)]);
            }
    return ARK_OK;
}
