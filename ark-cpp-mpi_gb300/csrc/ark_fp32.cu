// FP32 instantiation of the step kernels (built with --fmad=false like FP64), plus the
// double <-> float conversions used when FP32 contexts exchange Arr3d (double) arrays.
#include "ark_kernels.cuh"

namespace ark {
template struct Launch<float>;
template void rows_from_double<float>(float *, const double *, int, int64_t, int, double, cudaStream_t);
template void rows_to_double<float>(double *, const float *, int, int64_t, int, double, cudaStream_t);
template void flat_from_host<float>(float *, const double *, int, int64_t, int, double, cudaStream_t);
template void flat_to_host<float>(double *, const float *, int, int64_t, int, double, cudaStream_t);
template void rows_face_density<float>(double *, const float *, int, int64_t, int, double, double, cudaStream_t);

} // namespace ark

// ---- host check of the staged Phase1's copy plan ----
#include <cstdio>
#include <string>
#include <vector>

namespace ark {
namespace {

// Fake array bases, 2^40 bytes apart: a byte's "address" tells its array and offset.
constexpr long long kSpan = 1ll << 40;
enum { A_CU = 0, A_CR = 3, A_FL = 4, A_FC = 5, A_FF = 17, A_N = 20 };

// Array numbers of the fake bases: u1 (u2, u3 follow), ro, flags, faces (12 follow), forces.
struct Ids {
    int cu, cr, fl, fc, ff;
};

// Every shared-memory read a thread of tile column (tx, ty) makes for cell (i, j, k) of a
// staged Phase1 with stage layout L, as want(plane, stage byte, bytes, expected address of the
// first byte); addr(a, e, elem) is the fake address of element e of array a.
template <int MODE, class L, class Want, class Addr>
void staged_reads(const Geom &g, const Ids &id, Want &&want, Addr &&addr, int tx, int ty, int i, int j, int k) {
    const int cr = ty - L::CROW0, cx = tx + 1;
    auto cell = [&](int ii, int jj, int kk) { return g.cell(ii, jj, kk); };
    auto face = [&](int ii, int jj, int kk) { return g.face(ii, jj, kk); };
    want(k, L::flag(cr, cx), 1, addr(id.fl, cell(i, j, k), 1));
    want(k, L::ro(ty, cx) * 4, 4, addr(id.cr, cell(i, j, k), 4));
    for (int m = 0; m < 3; ++m) want(k, L::cu(m, cr, cx) * 4, 4, addr(id.cu + m, cell(i, j, k), 4));
    for (int a = 0; a < 4; ++a) {
        want(k, L::face(0, a, ty, cx) * 4, 4, addr(id.fc + a, face(i, j, k), 4));
        want(k, L::face(0, a, ty, cx + 1) * 4, 4, addr(id.fc + a, face(i + 1, j, k), 4));
        want(k, L::face(1, a, ty, cx) * 4, 4, addr(id.fc + 4 + a, face(i, j, k), 4));
        want(k, L::face(1, a, ty + 1, cx) * 4, 4, addr(id.fc + 4 + a, face(i, j + 1, k), 4));
        want(k, L::face(2, a, ty, cx) * 4, 4, addr(id.fc + 8 + a, face(i, j, k), 4));
        want(k + 1, L::face(2, a, ty, cx) * 4, 4, addr(id.fc + 8 + a, face(i, j, k + 1), 4));
    }
    if (L::STRESS) {
        const int di[4] = {-1, 1, 0, 0}, dj[4] = {0, 0, -1, 1};
        for (int q = 0; q < 4; ++q) {
            want(k, L::flag(cr + dj[q], cx + di[q]), 1, addr(id.fl, cell(i + di[q], j + dj[q], k), 1));
            for (int m = 0; m < 3; ++m)
                want(k, L::cu(m, cr + dj[q], cx + di[q]) * 4, 4, addr(id.cu + m, cell(i + di[q], j + dj[q], k), 4));
        }
        for (int dk = -1; dk <= 1; dk += 2) {
            want(k + dk, L::flag(cr, cx), 1, addr(id.fl, cell(i, j, k + dk), 1));
            for (int m = 0; m < 3; ++m) want(k + dk, L::cu(m, cr, cx) * 4, 4, addr(id.cu + m, cell(i, j, k + dk), 4));
        }
    }
    if (L::FIN)
        for (int m = 0; m < 3; ++m) want(k, L::ff(m, ty, cx) * 4, 4, addr(id.ff + m, cell(i, j, k), 4));
}

template <int MODE> struct PlanCheck {
    using L = stg::Layout<MODE>;
    const Geom g;
    long long size[A_N];
    std::string err;
    int bad = 0;

    explicit PlanCheck(const Geom &gg) : g(gg) {
        for (int a = 0; a < A_N; ++a) size[a] = g.ncell() * 4;
        size[A_FL] = g.ncell();
        for (int a = A_FC; a < A_FC + 12; ++a) size[a] = g.nface() * 4;
    }
    void fail(const char *what, int bx, int by, int p, long long x) {
        if (bad++ == 0) {
            char b[256];
            std::snprintf(b, sizeof b, "mode %d tile (%d,%d) plane %d: %s (%lld)", MODE, bx, by, p, what, x);
            err = b;
        }
    }
    stg::Bases bases() const {
        stg::Bases b;
        for (int m = 0; m < 3; ++m) b.cu[m] = (const void *)((A_CU + m) * kSpan);
        b.cr = (const void *)(A_CR * kSpan);
        b.fl = (const void *)(A_FL * kSpan);
        for (int d = 0; d < 3; ++d)
            for (int a = 0; a < 4; ++a) b.fc[d][a] = (const void *)((A_FC + 4 * d + a) * kSpan);
        for (int m = 0; m < 3; ++m) b.ff[m] = (const void *)((A_FF + m) * kSpan);
        return b;
    }
    // expected "address" of element e (elements of elem bytes) of array a
    static long long addr(int a, long long e, int elem) { return a * kSpan + e * elem; }

    void run(int kch) {
        const dim3 grid = stg::staged_grid(g, kch);
        stg::Group G[stg::kMaxGroups];
        const stg::Bases b = bases();
        std::vector<std::vector<long long>> map;
        for (int bz = 0; bz < (int)grid.z; ++bz)
            for (int by = 0; by < (int)grid.y; ++by)
                for (int bx = 0; bx < (int)grid.x; ++bx) {
                    const int n = stg::build_groups<MODE>(G, g, b, bx, by);
                    if (n > stg::kMaxGroups) fail("too many groups", bx, by, 0, n);
                    const int k0 = bz * kch + 1, k1 = std::min(k0 + kch - 1, g.C3);
                    stg::Row fr[stg::kMaxRows], gr[stg::kMaxFlagRows];
                    int nfr = 0, ngr = 0;
                    if (n <= stg::kMaxGroups) stg::expand_rows(G, n, fr, nfr, gr, ngr);
                    if (nfr > stg::kMaxRows || ngr > stg::kMaxFlagRows) fail("too many rows", bx, by, 0, nfr);
                    const int pfirst = L::STRESS ? k0 - 1 : k0, plast = k1 + 1;
                    map.assign(plast - pfirst + 1, std::vector<long long>(L::STAGE, -1));
                    for (int p = pfirst; p <= plast; ++p) {
                        const unsigned kind = p < k0 ? stg::DOWN : (p > k1 ? stg::TOP : stg::MID);
                        unsigned total = 0;
                        std::vector<long long> &M = map[p - pfirst];
                        for (int fg = 0; fg < 2; ++fg)
                            for (int R = 0; R < (fg ? ngr : nfr); ++R) {
                                const stg::Row &w = fg ? gr[R] : fr[R];
                                if (!((w.dw >> 24) & kind)) continue;
                                const int chunks = fg ? stg::kFlagChunks : stg::kChunks;
                                for (int c = 0; c < chunks; ++c) {
                                    const long long src = (long long)w.src + (long long)p * w.plane + 16 * c;
                                    const long long dst = (w.dw & 0xFFFFFFu) + 16ll * c;
                                    const int arr = (int)(src / kSpan);
                                    const long long off = src % kSpan;
                                    total += 16;
                                    if (arr < 0 || arr >= A_N) {
                                        fail("copy from no array", bx, by, p, src);
                                        continue;
                                    }
                                    if (src % 16 || dst % 16) fail("unaligned copy", bx, by, p, src);
                                    if (off < 0 || off + 16 > size[arr]) fail("copy outside its array", bx, by, p, off);
                                    if (dst < 0 || dst + 16 > L::STAGE) fail("copy outside its stage", bx, by, p, dst);
                                    for (int y = 0; y < 16 && dst + y < L::STAGE; ++y) {
                                        if (M[dst + y] != -1) fail("two copies into one byte", bx, by, p, dst + y);
                                        M[dst + y] = src + y;
                                    }
                                }
                            }
                        if (total != stg::plan_bytes(G, n, kind)) fail("byte count", bx, by, p, total);
                    }
                    for (int ty = 0; ty < stg::SY; ++ty)
                        for (int tx = 0; tx < stg::SX; ++tx) {
                            const int i = bx * stg::SX + tx + 1, j = by * stg::SY + ty + 1;
                            if (i > g.C1 || j > g.C2) continue;
                            for (int k = k0; k <= k1; ++k) reads(map, pfirst, bx, by, tx, ty, i, j, k);
                        }
                }
    }
    void want(const std::vector<std::vector<long long>> &map, int pfirst, int bx, int by, int p, int off_bytes,
              int nbytes, long long expect) {
        if (p - pfirst < 0 || p - pfirst >= (int)map.size()) {
            fail("read of a plane not staged", bx, by, p, off_bytes);
            return;
        }
        const std::vector<long long> &M = map[p - pfirst];
        for (int y = 0; y < nbytes; ++y)
            if (off_bytes + y >= L::STAGE || M[off_bytes + y] != expect + y) {
                fail("shared-memory read maps to the wrong element", bx, by, p, off_bytes);
                return;
            }
    }
    void reads(const std::vector<std::vector<long long>> &map, int pfirst, int bx, int by, int tx, int ty, int i, int j,
               int k) {
        const Ids id = {A_CU, A_CR, A_FL, A_FC, A_FF};
        staged_reads<MODE, L>(
            g, id, [&](int p, int off, int nb, long long e) { want(map, pfirst, bx, by, p, off, nb, e); }, addr, tx, ty, i, j, k);
    }
};

// The tensor-copy rules for a launch's boxes (stage bytes each): fail(what, box).
template <class Fail> void check_boxes(const stg::TmaBox *B, int n, int stage, Fail &&fail) {
    for (int q = 0; q < n; ++q) {
        const stg::TmaBox &x = B[q];
        if ((long long)x.box[0] * x.elem % 16) fail("box row not a multiple of 16 bytes", q);
        for (int d = 0; d < 4; ++d)
            if (x.box[d] < 1 || x.box[d] > 256) fail("box size outside 1..256", q);
        for (int d = 0; d < 3; ++d)
            if (x.stride[d] % 16 || x.stride[d] >= (1ll << 40)) fail("global stride", q);
        if (x.dst % 128) fail("destination not 128-byte aligned", q);
        if ((long long)x.dst + stg::box_bytes(x) > stage) fail("box outside its stage", q);
    }
}
// The boxes of kind `kind` for plane p of the tile at column x0, row j0, byte by byte as the
// copy engine lays them out: M[stage byte] = fake source address (-2: zero fill past the end of
// a row or past the last row: a 128-wide tile's box may reach past a narrow grid's rows, and
// the reads below then show that no thread uses those bytes); fail(what, value).
template <class Fail>
void expand_boxes(const stg::TmaBox *B, int n, unsigned kind, int x0, int j0, int p, std::vector<long long> &M, Fail &&fail) {
    const long long stage = (long long)M.size();
    if ((long long)x0 * 4 % 16) fail("x offset not a multiple of 16 bytes", x0);
    for (int q = 0; q < n; ++q) {
        const stg::TmaBox &x = B[q];
        if (!(x.when & kind)) continue;
        if (p < 0 || p >= x.dim[2]) fail("plane outside its array", q);
        if (j0 + x.row0 < 0) fail("box starts at a negative row", q);
        if (x0 >= x.dim[0]) fail("box starts past the end of its row", q);
        for (int a = 0; a < x.box[3]; ++a)
            for (int r = 0; r < x.box[1]; ++r)
                for (int e = 0; e < x.box[0]; ++e) {
                    const long long y = j0 + x.row0 + r;
                    const long long dst = x.dst + ((long long)(a * x.box[1] + r) * x.box[0] + e) * x.elem;
                    const long long src =
                        (long long)x.base + a * x.stride[2] + p * x.stride[1] + y * x.stride[0] + (long long)(x0 + e) * x.elem;
                    for (int c = 0; c < x.elem; ++c) {
                        if (dst + c >= stage) continue;
                        if (M[dst + c] != -1) fail("two boxes into one byte", dst + c);
                        M[dst + c] = y < x.dim[1] && x0 + e < x.dim[0] ? src + c : -2;
                    }
                }
    }
}

// The TMA form's plan, checked the same way: the boxes of tma_boxes (from fake bases whose
// blocks of arrays are a fixed stride apart) are expanded byte by byte as the copy engine
// lays them out (rows past a block's last row as zero fill), with the tensor copies' rules
// checked (16-byte global strides, x offsets and box rows; 128-byte aligned destinations; box
// sizes at most 256), then every read of every thread as above.
template <int MODE, int TSX, int TSY> struct TmaCheck {
    using L = stg::TLayout<MODE, TSX, TSY>;
    static constexpr long long kS = 1ll << 36; // fake array spacing (tensor-map strides stay below 2^40)
    enum { T_CR = 0, T_CU = 1, T_FL = 4, T_FC = 5, T_FF = 17, T_N = 20 };
    const Geom g;
    std::string err;
    int bad = 0;
    explicit TmaCheck(const Geom &gg) : g(gg) {}
    void fail(const char *what, int bx, int by, int p, long long x) {
        if (bad++ == 0) {
            char b[256];
            std::snprintf(b, sizeof b, "TMA mode %d tile (%d,%d) plane %d: %s (%lld)", MODE, bx, by, p, what, x);
            err = b;
        }
    }
    static long long addr(int a, long long e, int elem) { return a * kS + e * elem; }
    void run(int kch) {
        stg::Bases b;
        b.cr = (const void *)(T_CR * kS);
        for (int m = 0; m < 3; ++m) b.cu[m] = (const void *)((T_CU + m) * kS);
        b.fl = (const void *)(T_FL * kS);
        for (int d = 0; d < 3; ++d)
            for (int a = 0; a < 4; ++a) b.fc[d][a] = (const void *)((T_FC + 4 * d + a) * kS);
        for (int m = 0; m < 3; ++m) b.ff[m] = (const void *)((T_FF + m) * kS);
        stg::TmaBox B[stg::kMaxBoxes];
        const int n = stg::tma_boxes<MODE, TSX, TSY>(B, g, b);
        if (n <= 0) {
            fail("no TMA plan for these arrays", 0, 0, 0, n);
            return;
        }
        check_boxes(B, n, L::STAGE, [&](const char *w, long long v) { fail(w, 0, 0, 0, v); });
        const dim3 grid = stg::tile_grid<TSX, TSY>(g, kch);
        std::vector<std::vector<long long>> map;
        for (int bz = 0; bz < (int)grid.z; ++bz)
            for (int by = 0; by < (int)grid.y; ++by)
                for (int bx = 0; bx < (int)grid.x; ++bx) {
                    const int k0 = bz * kch + 1, k1 = std::min(k0 + kch - 1, g.C3);
                    const int pfirst = L::STRESS ? k0 - 1 : k0, plast = k1 + 1;
                    map.assign(plast - pfirst + 1, std::vector<long long>(L::STAGE, -1));
                    for (int p = pfirst; p <= plast; ++p) {
                        const unsigned kind = p < k0 ? stg::DOWN : (p > k1 ? stg::TOP : stg::MID);
                        expand_boxes(B, n, kind, bx * TSX, by * TSY + 1, p, map[p - pfirst],
                                     [&](const char *w, long long v) { fail(w, bx, by, p, v); });
                    }
                    for (int ty = 0; ty < TSY; ++ty)
                        for (int tx = 0; tx < TSX; ++tx) {
                            const int i = bx * TSX + tx + 1, j = by * TSY + ty + 1;
                            if (i > g.C1 || j > g.C2) continue;
                            const Ids id = {T_CU, T_CR, T_FL, T_FC, T_FF};
                            for (int k = k0; k <= k1; ++k)
                                staged_reads<MODE, L>(
                                    g, id,
                                    [&](int p, int off, int nb, long long want) {
                                        if (p - pfirst < 0 || p - pfirst >= (int)map.size()) {
                                            fail("read of a plane not staged", bx, by, p, off);
                                            return;
                                        }
                                        const std::vector<long long> &M = map[p - pfirst];
                                        for (int y = 0; y < nb; ++y)
                                            if (off + y >= L::STAGE || M[off + y] != want + y) {
                                                fail("shared-memory read maps to the wrong element", bx, by, p, off);
                                                return;
                                            }
                                    },
                                    addr, tx, ty, i, j, k);
                        }
                }
    }
};

// The copy plan of the one-kernel Phase2 + second Phase1 (s2), checked the same way: every
// copy, then every shared-memory read the kernel makes (the thread's own cell for the three
// sweeps, the halo jobs, the old tangential face values, the bounded-x edge flag) against the
// element of the global arrays that the separate sweep kernels read for it.
struct Plan2Check {
    enum { B_CELL = 0, B_FL = 8, B_FX = 9, B_FY = 13, B_N = 17 };
    const Geom g;
    const bool tma;     // check the TMA form's boxes instead of the cp.async rows
    const long long sp; // fake array spacing (below 2^40 for the tensor maps' strides)
    long long size[B_N];
    std::string err;
    int bad = 0;
    explicit Plan2Check(const Geom &gg, bool t = false) : g(gg), tma(t), sp(t ? 1ll << 36 : kSpan) {
        for (int a = 0; a < B_N; ++a) size[a] = a < B_FL ? g.ncell() * 4 : (a == B_FL ? g.ncell() : g.nface() * 4);
    }
    void fail(const char *what, int bx, int by, int p, long long x) {
        if (bad++ == 0) {
            char b[256];
            std::snprintf(b, sizeof b, "phase2+phase1%s tile (%d,%d) plane %d: %s (%lld)", tma ? " (TMA)" : "", bx, by, p,
                          what, x);
            err = b;
        }
    }
    long long addr(int a, long long e, int elem) const { return a * sp + e * elem; }
    void run(int kch) {
        using namespace s2;
        const dim3 grd = s2::grid(g, kch);
        s2::Bases b;
        for (int q = 0; q < 8; ++q) b.cell[q] = (const void *)((B_CELL + q) * sp);
        b.fl = (const void *)(B_FL * sp);
        for (int a = 0; a < 4; ++a) {
            b.fx[a] = (const void *)((B_FX + a) * sp);
            b.fy[a] = (const void *)((B_FY + a) * sp);
        }
        stg::Group G[s2::kMaxGroups];
        std::vector<std::vector<long long>> map;
        stg::TmaBox TB[stg::kMaxBoxes];
        const int nb = tma ? s2::tma_boxes(TB, g, b) : 0;
        if (tma) {
            if (nb <= 0) fail("no TMA plan for these arrays", 0, 0, 0, nb);
            check_boxes(TB, nb, STAGE, [&](const char *w, long long v) { fail(w, 0, 0, 0, v); });
        }
        for (int bz = 0; bz < (int)grd.z; ++bz)
            for (int by = 0; by < (int)grd.y; ++by)
                for (int bx = 0; bx < (int)grd.x; ++bx) {
                    if (tma) {
                        const int k0 = bz * kch + 1, k1 = std::min(k0 + kch - 1, g.C3);
                        const int pfirst = k0 - 1, plast = k1 + 1;
                        map.assign(plast - pfirst + 1, std::vector<long long>(STAGE, -1));
                        for (int p = pfirst; p <= plast; ++p)
                            expand_boxes(TB, nb, (p < k0 || p > k1) ? EDGE : MID, bx * SX, by * SY + 1, p, map[p - pfirst],
                                         [&](const char *w, long long v) { fail(w, bx, by, p, v); });
                        reads(map, pfirst, k0, k1, bx, by);
                        continue;
                    }
                    const int n = s2::build_groups(G, g, b, bx, by);
                    if (n > s2::kMaxGroups) {
                        fail("too many groups", bx, by, 0, n);
                        continue;
                    }
                    stg::Row fr[stg::kMaxRows], gr[stg::kMaxFlagRows];
                    int nfr = 0, ngr = 0;
                    stg::expand_rows(G, n, fr, nfr, gr, ngr);
                    if (nfr > stg::kMaxRows || ngr > stg::kMaxFlagRows) fail("too many rows", bx, by, 0, nfr);
                    const int k0 = bz * kch + 1, k1 = std::min(k0 + kch - 1, g.C3);
                    const int pfirst = k0 - 1, plast = k1 + 1;
                    map.assign(plast - pfirst + 1, std::vector<long long>(STAGE, -1));
                    for (int p = pfirst; p <= plast; ++p) {
                        const unsigned kind = (p < k0 || p > k1) ? EDGE : MID;
                        std::vector<long long> &M = map[p - pfirst];
                        unsigned total = 0;
                        for (int fg = 0; fg < 2; ++fg)
                            for (int R = 0; R < (fg ? ngr : nfr); ++R) {
                                const stg::Row &w = fg ? gr[R] : fr[R];
                                if (!((w.dw >> 24) & kind)) continue;
                                const int chunks = fg ? stg::kFlagChunks : stg::kChunks;
                                for (int c = 0; c < chunks; ++c) {
                                    const long long src = (long long)w.src + (long long)p * w.plane + 16 * c;
                                    const long long dst = (w.dw & 0xFFFFFFu) + 16ll * c;
                                    const int arr = (int)(src / sp);
                                    const long long off = src % sp;
                                    total += 16;
                                    if (arr < 0 || arr >= B_N) {
                                        fail("copy from no array", bx, by, p, src);
                                        continue;
                                    }
                                    if (src % 16 || dst % 16) fail("unaligned copy", bx, by, p, src);
                                    if (off < 0 || off + 16 > size[arr]) fail("copy outside its array", bx, by, p, off);
                                    if (dst < 0 || dst + 16 > STAGE) fail("copy outside its stage", bx, by, p, dst);
                                    for (int y = 0; y < 16 && dst + y < STAGE; ++y) {
                                        if (M[dst + y] != -1) fail("two copies into one byte", bx, by, p, dst + y);
                                        M[dst + y] = src + y;
                                    }
                                }
                            }
                        if (total != stg::plan_bytes(G, n, kind)) fail("byte count", bx, by, p, total);
                    }
                    reads(map, pfirst, k0, k1, bx, by);
                }
    }
    void want(const std::vector<std::vector<long long>> &map, int pfirst, int bx, int by, int p, int off_bytes,
              int nbytes, long long expect) {
        if (p - pfirst < 0 || p - pfirst >= (int)map.size()) {
            fail("read of a plane not staged", bx, by, p, off_bytes);
            return;
        }
        const std::vector<long long> &M = map[p - pfirst];
        for (int y = 0; y < nbytes; ++y)
            if (off_bytes + y >= s2::STAGE || M[off_bytes + y] != expect + y) {
                fail("shared-memory read maps to the wrong element", bx, by, p, off_bytes);
                return;
            }
    }
    // all eight cell values and the flag of cell (ic, jc) read at stage row r, column x
    void cell_at(const std::vector<std::vector<long long>> &map, int pfirst, int bx, int by, int p, int r, int x,
                 int ic, int jc) {
        for (int q = 0; q < 8; ++q)
            want(map, pfirst, bx, by, p, s2::off_cell(q, r, x) * 4, 4, addr(B_CELL + q, g.cell(ic, jc, p), 4));
        want(map, pfirst, bx, by, p, s2::off_flag(r, x), 1, addr(B_FL, g.cell(ic, jc, p), 1));
    }
    void fx_at(const std::vector<std::vector<long long>> &map, int pfirst, int bx, int by, int p, int r, int x, int ic,
               int jc) {
        for (int a = 0; a < 4; ++a)
            want(map, pfirst, bx, by, p, s2::off_fx(a, r, x) * 4, 4, addr(B_FX + a, g.face(ic, jc, p), 4));
    }
    void fy_at(const std::vector<std::vector<long long>> &map, int pfirst, int bx, int by, int p, int r, int x, int ic,
               int jc) {
        for (int a = 0; a < 4; ++a)
            want(map, pfirst, bx, by, p, s2::off_fy(a, r, x) * 4, 4, addr(B_FY + a, g.face(ic, jc, p), 4));
    }
    void reads(const std::vector<std::vector<long long>> &map, int pfirst, int k0, int k1, int bx, int by) {
        using namespace s2;
        const int i0 = bx * SX + 1, j0 = by * SY + 1;
        const int tx_last = std::min(SX - 1, g.C1 - i0), ty_last = std::min(SY - 1, g.C2 - j0);
        for (int p = pfirst; p <= k1 + 1; ++p)
            for (int ty = 0; ty <= ty_last; ++ty)
                for (int tx = 0; tx <= tx_last; ++tx) {
                    const int i = i0 + tx, j = j0 + ty;
                    cell_at(map, pfirst, bx, by, p, ty + 1, tx + 1, i, j); // z sweep (every plane)
                    if (p < k0 || p > k1) continue;
                    fx_at(map, pfirst, bx, by, p, ty, tx + 1, i, j);     // x faces i, i+1
                    fx_at(map, pfirst, bx, by, p, ty, tx + 2, i + 1, j);
                    fy_at(map, pfirst, bx, by, p, ty + 1, tx + 1, i, j); // y faces j, j+1
                    fy_at(map, pfirst, bx, by, p, ty + 2, tx + 1, i, j + 1);
                }
        // ghost cells copied from the "Con" level (the block's share of the ghost shell)
        for (int p = pfirst; p <= k1 + 1; ++p) {
            const bool gp = p == 0 || p == g.C3 + 1;
            const int ia = i0 == 1 ? 0 : i0, ib = tx_last == g.C1 - i0 ? g.C1 + 1 : i0 + tx_last;
            const int ja = j0 == 1 ? 0 : j0, jb = ty_last == g.C2 - j0 ? g.C2 + 1 : j0 + ty_last;
            for (int jj = ja; jj <= jb; ++jj)
                for (int ii = ia; ii <= ib; ++ii)
                    if (gp || ii == 0 || ii == g.C1 + 1 || jj == 0 || jj == g.C2 + 1)
                        for (int q = 0; q < 4; ++q)
                            want(map, pfirst, bx, by, p, s2::off_cell(q, jj - (j0 - 1), ii - (i0 - 1)) * 4, 4,
                                 addr(B_CELL + q, g.cell(ii, jj, p), 4));
        }
        for (int p = k0; p <= k1; ++p) {
            for (int c = 0; c <= tx_last; ++c) {
                const int i = i0 + c, jt = j0 + ty_last + 1, ry = ty_last + 2;
                cell_at(map, pfirst, bx, by, p, 0, c + 1, i, j0 - 1); // below the tile
                fy_at(map, pfirst, bx, by, p, 0, c + 1, i, j0 - 1);
                fy_at(map, pfirst, bx, by, p, 1, c + 1, i, j0);
                cell_at(map, pfirst, bx, by, p, ry, c + 1, i, jt); // above the tile's last row
                fy_at(map, pfirst, bx, by, p, ry, c + 1, i, jt);
                fy_at(map, pfirst, bx, by, p, ry + 1, c + 1, i, jt + 1);
            }
            for (int rr = 0; rr <= ty_last; ++rr) {
                const int j = j0 + rr, it = i0 + tx_last + 1, xc = tx_last + 2;
                cell_at(map, pfirst, bx, by, p, rr + 1, 0, i0 - 1, j); // left of the row
                fx_at(map, pfirst, bx, by, p, rr, 0, i0 - 1, j);
                fx_at(map, pfirst, bx, by, p, rr, 1, i0, j);
                if (i0 == 1) want(map, pfirst, bx, by, p, s2::off_flag(rr + 1, 1), 1, addr(B_FL, g.cell(1, j, p), 1));
                cell_at(map, pfirst, bx, by, p, rr + 1, xc, it, j); // right of the row's last cell
                fx_at(map, pfirst, bx, by, p, rr, xc, it, j);
                fx_at(map, pfirst, bx, by, p, rr, xc + 1, it + 1, j);
            }
        }
    }
};

} // namespace

int step2_plan_check(int C1, int C2, int C3, int kch, char *msg, int cap) {
    const Geom g = device_geom(C1, C2, C3);
    if (kch <= 0) kch = s2::chunk(g);
    Plan2Check a(g), b(g, true);
    a.run(kch);
    b.run(kch);
    if (msg && cap > 0) std::snprintf(msg, (size_t)cap, "%s", (!a.err.empty() ? a.err : b.err).c_str());
    return a.bad + b.bad;
}

int staging_plan_check(int C1, int C2, int C3, int kch_in, char *msg, int cap) {
    const Geom g = device_geom(C1, C2, C3);
    const int kch = kch_in > 0 ? kch_in : stg::staged_chunk(g);
    PlanCheck<P1_STRESS | P1_FORCES | P1_RMAX> a(g);
    a.run(kch);
    PlanCheck<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX> b(g);
    b.run(kch);
    PlanCheck<P1_FORCES | P1_RSUM> c(g);
    c.run(kch);
    TmaCheck<P1_STRESS | P1_FORCES | P1_RMAX, 64, 4> ta(g);
    ta.run(kch);
    TmaCheck<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 64, 4> tb(g);
    tb.run(kch);
    TmaCheck<P1_FORCES | P1_RSUM, 64, 4> tc(g);
    tc.run(kch);
    TmaCheck<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 32, 8> td(g);
    td.run(kch);
    TmaCheck<P1_FORCES | P1_RSUM, 32, 8> te(g);
    te.run(kch);
    TmaCheck<P1_STRESS | P1_FORCES | P1_BULK | P1_RMAX, 128, 2> tf(g);
    tf.run(kch);
    TmaCheck<P1_FORCES | P1_RSUM, 128, 2> th(g);
    th.run(kch);
    char m2[256] = {0};
    const int d = step2_plan_check(C1, C2, C3, kch_in, m2, (int)sizeof m2);
    std::string e = std::string(m2);
    for (const std::string *x : {&th.err, &tf.err, &te.err, &td.err, &tc.err, &tb.err, &ta.err, &c.err, &b.err, &a.err})
        if (!x->empty()) e = *x;
    if (msg && cap > 0) std::snprintf(msg, (size_t)cap, "%s", e.c_str());
    return a.bad + b.bad + c.bad + ta.bad + tb.bad + tc.bad + td.bad + te.bad + tf.bad + th.bad + d;
}

} // namespace ark

extern "C" int ark_selftest_staging(int n1_cells, int n2_cells, int n3_cells, int planes_per_block, char *msg, int cap) {
    if (n1_cells < 1 || n2_cells < 1 || n3_cells < 1 || planes_per_block < 0) return -1;
    return ark::staging_plan_check(n1_cells, n2_cells, n3_cells, planes_per_block, msg, cap);
}
