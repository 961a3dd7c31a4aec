// Phase2 and the second Phase1 of a step in one kernel (FP32 contexts).
//
// After the first Phase1 the rest of the step is local: a face's new values depend on the two
// cells beside it (their half-step and old values) and on the old faces beyond them, and the
// second Phase1 of a cell depends on its six new faces, its half-step values and its forces.
// So a block owning a 64 x 4 tile of cell columns can march up a chunk of planes and, per
// plane, compute the three sweeps' extrapolations of its cells (plus the halo cells whose
// extrapolations the tile's faces need), update the faces below its cells (plus, without
// storing them, the faces above its last column and row, which belong to the next tiles), and
// finish the cells of the plane below with those faces: the new faces never travel through
// HBM before the second Phase1 reads them, and the cell levels are read once instead of three
// times.  The arithmetic is the sweeps' extrapolate / face_values and Phase1's half_step /
// UseForces code, with the same inputs, so the results are the separate kernels' bits.
//
// The new cell level cannot overwrite the old "Con" level in place (neighbouring tiles still
// read it), so it goes to a third level (the caller swaps it in afterwards).
//
// Data movement per plane: the two cell levels and the flags (rows j0-1 .. j0+4), the x faces
// (rows j0 .. j0+3) and the y faces (rows j0-1 .. j0+5), 68 values wide, are copied into a
// 3-stage shared-memory ring with 16-byte cp.async copies (the staged Phase1's scheme); the z
// faces and the forces, which only the cell's own thread reads, are loaded into registers one
// plane ahead.  The z sweep runs one plane behind the x and y sweeps' plane, and the second
// Phase1 one plane behind the z sweep.  Two barriers per plane.  With TMA = true the planes
// come as five tensor-map boxes instead (both levels, the flags, the x and y face sets: the
// staged Phase1's TMA scheme), issued by thread 0 and awaited on each stage's mbarrier.
// Included by ark_kernels.cuh inside namespace ark.
#pragma once

namespace s2 {

constexpr int SX = 64, SY = 4, NT = SX * SY;
constexpr int W = stg::W, WF = stg::WF;
constexpr int NS = 3;                  // stages in the ring
constexpr unsigned EDGE = 1, MID = 2;  // planes k0-1 and k1+1 (z sweep only), the block's planes
constexpr int CR = SY + 2;             // staged cell rows j0-1 .. j0+SY
constexpr int YR = SY + 3;             // staged y-face rows j0-1 .. j0+SY+1
constexpr int kMaxGroups = 20;

// Stage layout: float rows of W values (x = 64*bx .. 64*bx+67, i.e. cells i0-1 .. i0+66 and
// the faces with the same indices), then flag rows of WF bytes.  Cell arrays q: 0..3 the "Con"
// level's ro, u1, u2, u3; 4..7 the "nCon" (half-step) level's.  Face arrays a: p, u1, u2, u3.
constexpr int O_C = 0;
constexpr int O_FX = O_C + 8 * CR;
constexpr int O_FY = O_FX + 4 * SY;
constexpr int ROWS = O_FY + 4 * YR;
constexpr int FLAG_OFF = (ROWS * W * 4 + 127) / 128 * 128; // boxes start on 128-byte boundaries
constexpr int STAGE = (FLAG_OFF + CR * WF + 127) / 128 * 128;
constexpr int SMEM = NS * STAGE;
static_assert(STAGE % 128 == 0 && (O_C + 4 * CR) * W * 4 % 128 == 0 && O_FX * W * 4 % 128 == 0 && O_FY * W * 4 % 128 == 0,
              "stages and boxes on 128-byte boundaries");
static_assert(ROWS <= stg::kMaxRows && CR <= stg::kMaxFlagRows, "row tables");

// Offsets within a stage (floats; flags in bytes).  r: cell row j - (j0 - 1), x-face row
// j - j0, y-face row j - (j0 - 1); x: i - (i0 - 1).
__host__ __device__ inline int off_cell(int q, int r, int x) { return (O_C + q * CR + r) * W + x; }
__host__ __device__ inline int off_fx(int a, int r, int x) { return (O_FX + a * SY + r) * W + x; }
__host__ __device__ inline int off_fy(int a, int r, int x) { return (O_FY + a * YR + r) * W + x; }
__host__ __device__ inline int off_flag(int r, int x) { return FLAG_OFF + r * WF + x; }

// The arrays one launch stages.
struct Bases {
    const void *cell[8], *fl, *fx[4], *fy[4];
};

__host__ __device__ inline int build_groups(stg::Group *G, const Geom &g, const Bases &b, int bx, int by) {
    const int j0 = by * SY + 1;
    const int x0 = bx * SX;
    int n = 0;
    auto add = [&](const void *base, bool face, int elem, int bytes, int row0, int nrows, int dst, unsigned when) {
        stg::Group &q = G[n++];
        q.base = (const char *)base;
        q.plane = (face ? g.fs2 : g.cs2) * elem;
        q.pitch = (int)((face ? g.fs1 : g.cs1) * elem);
        q.xoff = x0 * elem;
        q.bytes = bytes;
        q.row0 = row0;
        q.nrows = nrows;
        q.maxrow = face ? g.C2 + 2 : g.C2 + 1;
        q.dst = (unsigned)dst;
        q.when = when;
    };
    for (int q = 0; q < 8; ++q) add(b.cell[q], false, 4, W * 4, j0 - 1, CR, off_cell(q, 0, 0) * 4, EDGE | MID);
    add(b.fl, false, 1, WF, j0 - 1, CR, FLAG_OFF, EDGE | MID);
    for (int a = 0; a < 4; ++a) add(b.fx[a], true, 4, W * 4, j0, SY, off_fx(a, 0, 0) * 4, MID);
    for (int a = 0; a < 4; ++a) add(b.fy[a], true, 4, W * 4, j0 - 1, YR, off_fy(a, 0, 0) * 4, MID);
    return n;
}

__host__ __device__ inline Bases bases_of(const DevState<float> &S, int con, int fcur) {
    Bases b;
    const Level<float> &Lc = S.lv[con], &Ln = S.lv[con ^ 1];
    b.cell[0] = Lc.ro;
    b.cell[1] = Lc.u1;
    b.cell[2] = Lc.u2;
    b.cell[3] = Lc.u3;
    b.cell[4] = Ln.ro;
    b.cell[5] = Ln.u1;
    b.cell[6] = Ln.u2;
    b.cell[7] = Ln.u3;
    b.fl = S.flags;
    for (int d = 0; d < 2; ++d) {
        const FaceSet<float> &F = S.fc[fcur][d];
        const void **dst = d == 0 ? b.fx : b.fy;
        dst[0] = F.p;
        for (int a = 0; a < 3; ++a) dst[a + 1] = F.u[a];
    }
    return b;
}

// The TMA form's boxes: the "Con" and "nCon" levels (ro, u1, u2, u3; cell rows j0-1 ..
// j0+SY), the flags, the x faces (rows j0 .. j0+SY-1) and the y faces (rows j0-1 .. j0+SY+1),
// p, u1, u2, u3; 0 when the arrays of a block are not a fixed stride apart.
inline int tma_boxes(stg::TmaBox *B, const Geom &g, const Bases &b) {
    const long long nc = g.ncell(), nf = g.nface();
    const long long cs0 = stg::block_stride(b.cell, 4, nc * 4), cs1 = stg::block_stride(b.cell + 4, 4, nc * 4);
    const long long xs = stg::block_stride(b.fx, 4, nf * 4), ys = stg::block_stride(b.fy, 4, nf * 4);
    if (!cs0 || !cs1 || !xs || !ys || !stg::rows_fit(g)) return 0;
    int n = 0;
    B[n++] = stg::make_box(g, b.cell[0], 4, false, 4, cs0, W, CR, -1, off_cell(0, 0, 0) * 4, EDGE | MID);
    B[n++] = stg::make_box(g, b.cell[4], 4, false, 4, cs1, W, CR, -1, off_cell(4, 0, 0) * 4, EDGE | MID);
    B[n++] = stg::make_box(g, b.fl, 1, false, 1, nc, WF, CR, -1, FLAG_OFF, EDGE | MID);
    B[n++] = stg::make_box(g, b.fx[0], 4, true, 4, xs, W, SY, 0, off_fx(0, 0, 0) * 4, MID);
    B[n++] = stg::make_box(g, b.fy[0], 4, true, 4, ys, W, YR, -1, off_fy(0, 0, 0) * 4, MID);
    return n;
}

// Planes per block: about eight waves of two blocks per SM on 152 SMs, 2 to 64 planes (small
// grids: short chunks, so that enough blocks run; each block also sweeps the two planes at its
// ends in z).
inline int chunk(const Geom &g) {
    const long long cols = (long long)((g.C1 + SX - 1) / SX) * ((g.C2 + SY - 1) / SY);
    long long k = (long long)g.C3 * cols / (152 * 2 * 8);
    k = k < 2 ? 2 : (k > 64 ? 64 : k);
    return (int)k;
}
inline dim3 grid(const Geom &g, int kch) { return dim3((g.C1 + SX - 1) / SX, (g.C2 + SY - 1) / SY, (g.C3 + kch - 1) / kch); }

#ifdef __CUDACC__
// What a face update takes from the cell behind the face and from the cell ahead of it.
struct Behind {
    float rf, af, bf, un;
    int fl;
};
struct Ahead {
    float qb, ab, bb, un;
    int fl;
};

// The extrapolation of a staged cell along x (AX = 0) or y (AX = 1): cell at stage row r,
// column x; its faces lo and hi at face rows flo / fhi and columns xlo / xhi.
template <int AX>
__device__ __forceinline__ Ext<float> stage_ext(const float *st, int r, int x, int flo, int fhi, int xlo, int xhi,
                                                const SweepK<float> &q) {
    // normal, first and second tangential components (u1 u2 u3 for x; u2 u1 u3 for y)
    constexpr int mN = AX == 0 ? 0 : 1, mA = AX == 0 ? 1 : 0, mB = 2;
    auto face = [&](int a, int row, int col) { return AX == 0 ? st[off_fx(a, row, col)] : st[off_fy(a, row, col)]; };
    return extrapolate<float, AX != 1>(face(1 + mN, fhi, xhi), face(1 + mN, flo, xlo), st[off_cell(5 + mN, r, x)],
                                       st[off_cell(1 + mN, r, x)], face(1 + mA, fhi, xhi), face(1 + mA, flo, xlo),
                                       st[off_cell(5 + mA, r, x)], st[off_cell(1 + mA, r, x)], face(1 + mB, fhi, xhi),
                                       face(1 + mB, flo, xlo), st[off_cell(5 + mB, r, x)], st[off_cell(1 + mB, r, x)],
                                       st[off_cell(4, r, x)], st[off_cell(0, r, x)], face(0, fhi, xhi), face(0, flo, xlo), q);
}

__device__ __forceinline__ FaceVal<float> face_val(float p, float u1, float u2, float u3, const K<float> &kk) {
    FaceVal<float> v;
    v.p = p;
    v.ro = face_ro(v.p, kk);
    v.u[0] = u1;
    v.u[1] = u2;
    v.u[2] = u3;
    return v;
}

template <class T, bool TMA>
__global__ void __launch_bounds__(NT, 2)
    k_phase2_phase1(const __grid_constant__ DevState<T> S, int con, int fcur, const __grid_constant__ Level<T> out, int kch,
                    const __grid_constant__ stg::TmaArgs A) {
    static_assert(sizeof(T) == 4, "FP32 contexts only");
    constexpr unsigned long long kLimitNs = 500000000ull;
    extern __shared__ __align__(128) unsigned char sm_raw[];
    __shared__ __align__(8) unsigned long long bar[NS];
    // the stages from the first 128-byte boundary (tensor copies land on 128-byte boundaries)
    unsigned char *const sm = TMA ? stg::align128(sm_raw) : sm_raw;
    __shared__ stg::Row rows[stg::kMaxRows], frows[stg::kMaxFlagRows];
    __shared__ int nrow, nfrow;
    __shared__ Behind XB[SY][SX + 1]; // x: index x holds cell i0-1+x
    __shared__ Ahead XA[SY];          // x: the cell after the row's last cell
    __shared__ Behind YB[SY + 1][SX]; // y: index r holds row j0-1+r
    __shared__ Ahead YA[SX];          // y: the row after the tile's last row
    // a cell's new upper x / y face (p, u1, u2, u3): written after barrier (C) of plane p, read by
    // the second Phase1 of plane p before barrier (C) of plane p+1, so one buffer serves
    __shared__ float4 NX[SY][SX], NY[SY][SX];
    const Geom g = S.g;
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * SX + tx;
    const int bxi = blockIdx.x, byi = blockIdx.y;
    const int i0 = bxi * SX + 1, j0 = byi * SY + 1;
    const int i = i0 + tx, j = j0 + ty;
    const int k0 = blockIdx.z * kch + 1;
    const int k1 = k0 + kch - 1 < g.C3 ? k0 + kch - 1 : g.C3;
    const int pfirst = k0 - 1, plast = k1 + 1;
    const int tx_last = g.C1 - i0 < SX - 1 ? g.C1 - i0 : SX - 1;
    const int ty_last = g.C2 - j0 < SY - 1 ? g.C2 - j0 : SY - 1;
    const bool valid = tx <= tx_last && ty <= ty_last;
    const unsigned sbase = stg::smem_u32(sm);
    if (!TMA && t == 0) {
        stg::Group G[kMaxGroups];
        const int ng = build_groups(G, g, bases_of(S, con, fcur), bxi, byi);
        int a, b;
        stg::expand_rows(G, ng, rows, a, frows, b);
        nrow = a;
        nfrow = b;
    }
    __syncthreads();
    // copies issued from the row table each plane (resolving them into registers, as the staged
    // Phase1 does, costs this kernel 22 registers it does not have: spills, 11% slower)
    const int ch = t % stg::kChunks, r0 = t / stg::kChunks;
    constexpr int kRowsPerPass = NT / stg::kChunks;
    auto bar_of = [&](int p) { return stg::smem_u32(&bar[(p - pfirst) % NS]); };
    auto parity_of = [&](int p) { return (unsigned)(((p - pfirst) / NS) & 1); };
    auto issue = [&](int p) {
        const unsigned to = sbase + (unsigned)(((p - pfirst) % NS) * STAGE);
        const unsigned kind = (p < k0 || p > k1) ? EDGE : MID;
        if (TMA) { // thread 0
            const unsigned b = bar_of(p);
            stg::mbar_expect_tx(b, A.m.bytes[kind]);
            for (int q = 0; q < A.m.n; ++q)
                if (A.m.when[q] & kind) stg::tma_load_4d(to + A.m.dst[q], &A.map[q], bxi * SX, j0 + A.m.row0[q], p, 0, b);
            return;
        }
        if (r0 < kRowsPerPass)
            for (int R = r0; R < nrow; R += kRowsPerPass) {
                const stg::Row w = rows[R];
                if ((w.dw >> 24) & kind) stg::cp16(to + (w.dw & 0xFFFFFFu) + 16u * ch, w.src + (long long)p * w.plane + 16 * ch);
            }
        if (t < stg::kFlagChunks * nfrow) {
            const stg::Row w = frows[t / stg::kFlagChunks];
            const int c = t % stg::kFlagChunks;
            if ((w.dw >> 24) & kind) stg::cp16(to + (w.dw & 0xFFFFFFu) + 16u * c, w.src + (long long)p * w.plane + 16 * c);
        }
    };
    // planes pfirst .. pfirst+NS-2 up front; at plane p (once it has landed and every thread is
    // past plane p-1) the slot of plane p-1 takes plane p+NS-1.  One commit group per plane.
    int issued = pfirst - 1; // (TMA) thread 0: the last plane issued
    if (!TMA) {
        for (int p = pfirst; p < pfirst + NS - 1; ++p) {
            if (p <= plast) issue(p);
            stg::cp_commit();
        }
    } else if (t == 0) {
        for (int q = 0; q < NS; ++q) stg::mbar_init(stg::smem_u32(&bar[q]), 1);
        stg::fence_mbar_init();
        stg::fence_proxy_async();
        for (int p = pfirst; p < pfirst + NS - 1 && p <= plast; ++p) {
            issue(p);
            issued = p;
        }
    }
    if (TMA) __syncthreads();

    const K<T> &kk = kconst<T>(S.k);
    const T dt = sc_dt<T>(S.sc);
    const SweepK<T> qx = sweep_consts(S, 0), qy = sweep_consts(S, 1), qz = sweep_consts(S, 2);
    const Level<T> Ln = S.lv[con ^ 1];
    const int nc_ = (int)g.ncell();
    const NCell<T> NCX = {Ln.u1, Ln.u2, Ln.u3, Ln.ro, nc_}, NCY = {Ln.u2, Ln.u1, Ln.u3, Ln.ro, nc_},
                   NCZ = {Ln.u3, Ln.u1, Ln.u2, Ln.ro, nc_};
    const FaceOut<T> WX = sweep_out(S, fcur, 0), WY = sweep_out(S, fcur, 1), WZ = sweep_out(S, fcur, 2);
    const FaceSet<T> FZ = S.fc[fcur][2];
    const bool bounded_x = !S.k.periodic_x;
    // the bounded x axis's edge invariants (main.cpp:1731-1745), as the x1 sweep applies them
    auto x_edges = [&](Ext<T> &e, int ic, const uint8_t *flg, int r) {
        if (!bounded_x) return;
        if (ic == 0) {
            e.rf = (flg[off_flag(r, 1)] & FL_LT) ? (T)1 : (T)0;
            e.af = (T)0;
            e.bf = (T)0;
        } else if (ic == g.C1 + 1) {
            e.qb = (T)(5. / 6.);
            e.ab = (T)0;
            e.bb = (T)0;
        }
    };

    // z faces of the column: p, u1, u2, u3 of faces p (lo), p+1 (hi), p+2 (next)
    T zlo[4] = {0, 0, 0, 0}, zhi[4] = {0, 0, 0, 0}, znx[4] = {0, 0, 0, 0};
    auto zload = [&](int kf, T v[4]) {
        const int f = g.fi(i, j, kf);
        v[0] = FZ.p[f];
        v[1] = FZ.u[0][f];
        v[2] = FZ.u[1][f];
        v[3] = FZ.u[2][f];
    };
    // (the next face is loaded one plane ahead and moved into place at the start of the next
    // plane, so each load has a plane's work to land)
    if (valid) {
        zload(pfirst, zlo);
        zload(pfirst + 1, zhi);
        zload(pfirst + 2, znx);
    }
    Behind zb = {0, 0, 0, 0, 0};           // the z extrapolation of plane p-1, behind face p
    T zn_lo[4] = {0, 0, 0, 0};             // the new z face p-1 (below plane p-1): p, u1, u2, u3
    T nfx[4] = {0, 0, 0, 0}, nfy[4] = {0, 0, 0, 0}; // the new x / y face below the cell of plane p-1
    T hro = 0, hu[3] = {0, 0, 0}, ff[3] = {0, 0, 0}; // half-step values and forces of plane p-1
    uint8_t hfl = 0;
    long long rsum = 0;
    const int r = ty + 1, x = tx + 1; // the thread's cell in the stage

    bool failed = false;
    for (int p = pfirst; p <= plast; ++p) {
        if (!TMA) {
            stg::cp_wait<NS - 2>();
            __syncthreads(); // (A)
            const int pn = p + NS - 1;
            if (pn <= plast) issue(pn);
            stg::cp_commit();
        } else {
            const bool ok = stg::mbar_wait(bar_of(p), parity_of(p), kLimitNs);
            if (__syncthreads_or(!ok)) { // (A)
                failed = true;
                break;
            }
            const int pn = p + NS - 1;
            if (t == 0 && pn <= plast) {
                stg::fence_proxy_async();
                issue(pn);
                issued = pn;
            }
        }
        const T *st = (const T *)(sm + ((p - pfirst) % NS) * STAGE);
        const uint8_t *flg = (const uint8_t *)st;

        // ---- z sweep of plane p, the z face p, the second Phase1 of plane p-1 ----
        if (valid) {
            if (p > pfirst) {
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    zlo[a] = zhi[a];
                    zhi[a] = znx[a];
                }
                if (p + 2 <= plast + 1) zload(p + 2, znx);
            }
            const Ext<T> ez = extrapolate<T, true>(zhi[3], zlo[3], st[off_cell(7, r, x)], st[off_cell(3, r, x)], zhi[1],
                                                   zlo[1], st[off_cell(5, r, x)], st[off_cell(1, r, x)], zhi[2], zlo[2],
                                                   st[off_cell(6, r, x)], st[off_cell(2, r, x)], st[off_cell(4, r, x)],
                                                   st[off_cell(0, r, x)], zhi[0], zlo[0], qz);
            const uint8_t fl = flg[off_flag(r, x)];
            const T un = st[off_cell(7, r, x)];
            T zn[4] = {0, 0, 0, 0};
            if (p >= k0) {
                Ext<T> eb = {}, ea = {};
                eb.rf = zb.rf;
                eb.af = zb.af;
                eb.bf = zb.bf;
                ea.qb = ez.qb;
                ea.ab = ez.ab;
                ea.bb = ez.bb;
                const FaceNew<T> v = face_values<T, false>(NCZ, g.ci(i, j, p - 1), g.ci(i, j, p), (uint8_t)zb.fl, fl, zb.un,
                                                           un, eb, ea, zlo[1], zlo[2], qz);
                if (p <= k1 || p == g.C3 + 1) face_store(WZ, g.fi(i, j, p), v);
                zn[0] = v.p;
                zn[1] = v.a;
                zn[2] = v.b;
                zn[3] = v.n;
            }
            if (p >= k0 + 1) {
                // the second Phase1 (with UseForces and the bulk-flow partial) of cell (i, j, p-1)
                T ro_cn, ucn[3], rden = (T)0;
                if (hfl & FL_LT) {
                    const float4 hx = NX[ty][tx], hy = NY[ty][tx];
                    FaceVal<T> lo[3], hi[3];
                    lo[0] = face_val(nfx[0], nfx[1], nfx[2], nfx[3], kk);
                    hi[0] = face_val(hx.x, hx.y, hx.z, hx.w, kk);
                    lo[1] = face_val(nfy[0], nfy[1], nfy[2], nfy[3], kk);
                    hi[1] = face_val(hy.x, hy.y, hy.z, hy.w, kk);
                    lo[2] = face_val(zn_lo[0], zn_lo[1], zn_lo[2], zn_lo[3], kk);
                    hi[2] = face_val(zn[0], zn[1], zn[2], zn[3], kk);
                    half_step(lo, hi, hro, hu, dt, kk, ro_cn, ucn, rden);
                } else {
                    ucn[0] = ucn[1] = ucn[2] = (T)0;
                    ro_cn = (T)0;
                }
                if (hfl & FL_EQ0) use_forces_f32(ucn, ff, dt, kk, rden); // UseForces (main.cpp:1035-1041)
                const int c = g.ci(i, j, p - 1);
                out.ro[c] = ro_cn;
                out.u1[c] = ucn[0];
                out.u2[c] = ucn[1];
                out.u3[c] = ucn[2];
                if (hfl & FL_EQ0) rsum += fixed_sum_term(ucn[0]);
            }
            zb.rf = ez.rf;
            zb.af = ez.af;
            zb.bf = ez.bf;
            zb.un = un;
            zb.fl = fl;
#pragma unroll
            for (int a = 0; a < 4; ++a) zn_lo[a] = zn[a];
        }
        // ghost cells of the new level: the "Con" level's, as the separate kernels leave them
        // (they write interior cells only).  Each ghost cell belongs to the one block whose tile,
        // extended by the ghost layer at the domain's edges, holds it (block-uniform test).
        {
            const bool gx0 = i0 == 1, gx1 = tx_last == g.C1 - i0, gy0 = j0 == 1, gy1 = ty_last == g.C2 - j0;
            const bool gp = p == 0 || p == g.C3 + 1;
            if (gx0 || gx1 || gy0 || gy1 || gp) {
                const int ia = gx0 ? 0 : i0, ib = gx1 ? g.C1 + 1 : i0 + tx_last;
                const int ja = gy0 ? 0 : j0, jb = gy1 ? g.C2 + 1 : j0 + ty_last;
                auto copy = [&](int ii, int jj) {
                    const int rr = jj - (j0 - 1), xx = ii - (i0 - 1), c = g.ci(ii, jj, p);
                    out.ro[c] = st[off_cell(0, rr, xx)];
                    out.u1[c] = st[off_cell(1, rr, xx)];
                    out.u2[c] = st[off_cell(2, rr, xx)];
                    out.u3[c] = st[off_cell(3, rr, xx)];
                };
                if (gp) { // a ghost plane: the whole extended tile
                    const int wi = ib - ia + 1, nc = wi * (jb - ja + 1);
                    for (int q = t; q < nc; q += NT) copy(ia + q % wi, ja + q / wi);
                } else if (t < 2 * (SX + 2)) { // the ghost rows below / above (with the corners)
                    const int ii = ia + (t % (SX + 2)), jj = t < SX + 2 ? 0 : g.C2 + 1;
                    if (ii <= ib && (t < SX + 2 ? gy0 : gy1)) copy(ii, jj);
                } else if (t < 2 * (SX + 2) + 2 * SY) { // the ghost columns left / right
                    const int q = t - 2 * (SX + 2), jj = j0 + (q % SY);
                    if (jj <= j0 + ty_last && (q < SY ? gx0 : gx1)) copy(q < SY ? 0 : g.C1 + 1, jj);
                }
            }
        }
        if (p < k0 || p > k1) continue; // the edge planes: z sweep only (block-uniform)

        // ---- x and y sweeps of plane p: extrapolations ----
        Ext<T> ex = {}, ey = {};
        uint8_t fl = 0;
        T unx = 0, uny = 0;
        if (valid) {
            fl = flg[off_flag(r, x)];
            ex = stage_ext<0>(st, r, x, ty, ty, x, x + 1, qx);
            ey = stage_ext<1>(st, r, x, r, r + 1, x, x, qy);
            unx = st[off_cell(5, r, x)];
            uny = st[off_cell(6, r, x)];
            XB[ty][tx + 1] = Behind{ex.rf, ex.af, ex.bf, unx, fl};
            YB[ty + 1][tx] = Behind{ey.rf, ey.af, ey.bf, uny, fl};
            // what the second Phase1 of this cell needs next plane
            hro = st[off_cell(4, r, x)];
            hu[0] = unx;
            hu[1] = uny;
            hu[2] = st[off_cell(7, r, x)];
            hfl = fl;
            const int c = g.ci(i, j, p);
            ff[0] = S.f[0][c];
            ff[1] = S.f[1][c];
            ff[2] = S.f[2][c];
        }
        // halo cells: the row below and above the tile (y), the cell left and right of each row (x)
        if (t < SX) {
            if (t <= tx_last) { // cell (i0+t, j0-1), behind face j0
                const Ext<T> e = stage_ext<1>(st, 0, t + 1, 0, 1, t + 1, t + 1, qy);
                YB[0][t] = Behind{e.rf, e.af, e.bf, st[off_cell(6, 0, t + 1)], (int)flg[off_flag(0, t + 1)]};
            }
        } else if (t < 2 * SX) {
            const int c = t - SX, ry = ty_last + 2; // cell (i0+c, j0+ty_last+1), ahead of the last row's top face
            if (c <= tx_last) {
                const Ext<T> e = stage_ext<1>(st, ry, c + 1, ry, ry + 1, c + 1, c + 1, qy);
                YA[c] = Ahead{e.qb, e.ab, e.bb, st[off_cell(6, ry, c + 1)], (int)flg[off_flag(ry, c + 1)]};
            }
        } else if (t < 2 * SX + SY) {
            const int rr = t - 2 * SX; // cell (i0-1, j0+rr), behind face i0
            if (rr <= ty_last) {
                Ext<T> e = stage_ext<0>(st, rr + 1, 0, rr, rr, 0, 1, qx);
                x_edges(e, i0 - 1, flg, rr + 1);
                XB[rr][0] = Behind{e.rf, e.af, e.bf, st[off_cell(5, rr + 1, 0)], (int)flg[off_flag(rr + 1, 0)]};
            }
        } else if (t < 2 * SX + 2 * SY) {
            const int rr = t - 2 * SX - SY, xc = tx_last + 2; // cell (i0+tx_last+1, j0+rr), ahead of the row's last face
            if (rr <= ty_last) {
                Ext<T> e = stage_ext<0>(st, rr + 1, xc, rr, rr, xc, xc + 1, qx);
                x_edges(e, i0 + tx_last + 1, flg, rr + 1);
                XA[rr] = Ahead{e.qb, e.ab, e.bb, st[off_cell(5, rr + 1, xc)], (int)flg[off_flag(rr + 1, xc)]};
            }
        }
        __syncthreads(); // (C)

        // ---- x and y face updates of plane p ----
        if (valid) {
            {   // x face i, and the face above the row's last cell
                const Behind b = XB[ty][tx];
                Ext<T> eb = {}, ea = {};
                eb.rf = b.rf;
                eb.af = b.af;
                eb.bf = b.bf;
                ea.qb = ex.qb;
                ea.ab = ex.ab;
                ea.bb = ex.bb;
                const FaceNew<T> v = face_values<T, false>(NCX, g.ci(i - 1, j, p), g.ci(i, j, p), (uint8_t)b.fl, fl, b.un,
                                                           unx, eb, ea, st[off_fx(2, ty, x)], st[off_fx(3, ty, x)], qx);
                face_store(WX, g.fi(i, j, p), v);
                nfx[0] = v.p;
                nfx[1] = v.n;
                nfx[2] = v.a;
                nfx[3] = v.b;
                if (tx >= 1) NX[ty][tx - 1] = make_float4(v.p, v.n, v.a, v.b);
                if (tx == tx_last) {
                    const Ahead a = XA[ty];
                    Ext<T> eb2 = {}, ea2 = {};
                    eb2.rf = ex.rf;
                    eb2.af = ex.af;
                    eb2.bf = ex.bf;
                    ea2.qb = a.qb;
                    ea2.ab = a.ab;
                    ea2.bb = a.bb;
                    const FaceNew<T> w = face_values<T, false>(NCX, g.ci(i, j, p), g.ci(i + 1, j, p), fl, (uint8_t)a.fl,
                                                               unx, a.un, eb2, ea2, st[off_fx(2, ty, x + 1)],
                                                               st[off_fx(3, ty, x + 1)], qx);
                    if (i == g.C1) face_store(WX, g.fi(i + 1, j, p), w);
                    NX[ty][tx] = make_float4(w.p, w.n, w.a, w.b);
                }
            }
            {   // y face j, and the face above the tile's last row
                const Behind b = YB[ty][tx];
                Ext<T> eb = {}, ea = {};
                eb.rf = b.rf;
                eb.af = b.af;
                eb.bf = b.bf;
                ea.qb = ey.qb;
                ea.ab = ey.ab;
                ea.bb = ey.bb;
                const FaceNew<T> v = face_values<T, true>(NCY, g.ci(i, j - 1, p), g.ci(i, j, p), (uint8_t)b.fl, fl, b.un,
                                                          uny, eb, ea, st[off_fy(1, r, x)], st[off_fy(3, r, x)], qy);
                face_store(WY, g.fi(i, j, p), v);
                nfy[0] = v.p;
                nfy[1] = v.a;
                nfy[2] = v.n;
                nfy[3] = v.b;
                if (ty >= 1) NY[ty - 1][tx] = make_float4(v.p, v.a, v.n, v.b);
                if (ty == ty_last) {
                    const Ahead a = YA[tx];
                    Ext<T> eb2 = {}, ea2 = {};
                    eb2.rf = ey.rf;
                    eb2.af = ey.af;
                    eb2.bf = ey.bf;
                    ea2.qb = a.qb;
                    ea2.ab = a.ab;
                    ea2.bb = a.bb;
                    const FaceNew<T> w = face_values<T, true>(NCY, g.ci(i, j, p), g.ci(i, j + 1, p), fl, (uint8_t)a.fl,
                                                              uny, a.un, eb2, ea2, st[off_fy(1, r + 1, x)],
                                                              st[off_fy(3, r + 1, x)], qy);
                    if (j == g.C2) face_store(WY, g.fi(i, j + 1, p), w);
                    NY[ty][tx] = make_float4(w.p, w.a, w.n, w.b);
                }
            }
        }
    }
    if (!TMA) stg::cp_wait<0>();
    if (TMA) {
        if (failed && t == 0) {
            atomicOr(&S.sc->status, STATUS_STAGING);
            for (int p = issued - NS + 1 > pfirst ? issued - NS + 1 : pfirst; p <= issued; ++p)
                stg::mbar_wait(bar_of(p), parity_of(p), kLimitNs);
        }
        __syncthreads();
        if (t == 0)
            for (int q = 0; q < NS; ++q) stg::mbar_inval(stg::smem_u32(&bar[q]));
    }
    const BIx bx = {bxi, byi, (int)blockIdx.z, (int)gridDim.x, (int)gridDim.y};
    tile_store<T, NT>(S, bx, false, true, 0, 0, 0, rsum);
}

// tma: the TMA form (falls back to the cp.async form when the arrays do not allow it)
template <class T> inline void launch(const DevState<T> &S, int con, int fcur, const Level<T> &out, cudaStream_t st, bool tma) {
    const int kch = chunk(S.g);
    stg::TmaArgs A;
    std::memset(&A, 0, sizeof A);
    if (tma) {
        stg::TmaBox B[stg::kMaxBoxes];
        tma = stg::encode_boxes(A, B, tma_boxes(B, S.g, bases_of(S, con, fcur)));
    }
    if (tma)
        k_phase2_phase1<T, true><<<grid(S.g, kch), dim3(SX, SY), SMEM + 128, st>>>(S, con, fcur, out, kch, A);
    else
        k_phase2_phase1<T, false><<<grid(S.g, kch), dim3(SX, SY), SMEM, st>>>(S, con, fcur, out, kch, A);
}
template <class T> inline void prepare() {
    cudaFuncSetAttribute(k_phase2_phase1<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    cudaFuncSetAttribute(k_phase2_phase1<T, false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_phase2_phase1<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM + 128);
    cudaFuncSetAttribute(k_phase2_phase1<T, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}
#endif

} // namespace s2
