// Phase1 with its planes staged in shared memory (FP32 contexts).
//
// A block owns a 64 x 4 tile of cell columns and marches through a chunk of planes of it.
// Everything a plane contributes (the level's velocities and flags with one halo row on each
// side for the stress, the densities, the faces of the three directions, the forces of the
// second Phase1) is copied into a ring of shared-memory stages with asynchronous 16-byte copies
// (cp.async: row segments of 68 floats or 80 flag bytes, 16-byte aligned because device rows
// are padded to a 128-byte pitch) issued by all threads, several planes ahead of the plane being
// computed, so the block keeps many more bytes in flight than kernels that load their operands
// into registers themselves.  The arithmetic is the same half_step / stress_force / UseForces
// code, in the same order, as k_phase1 and k_phase1_cell, so all three give the same bits.
// Included by ark_kernels.cuh inside namespace ark.
#pragma once

namespace stg {

constexpr int SX = 64, SY = 4, NT = SX * SY;
constexpr int W = 68;   // floats per staged row: x = 64*bx .. 64*bx+67 (cells i0-1 .. i0+66)
constexpr int WF = 80;  // bytes per staged flag row
constexpr int NS = 5;   // stages in the ring
constexpr unsigned DOWN = 1, MID = 2, TOP = 4; // the plane below, inside, above a block's range
constexpr int kMaxGroups = 20;

// Stage layout (float rows of W, then flag rows of WF bytes).  With the stress (first Phase1
// of a step) the cell rows run j0-1 .. j0+SY; without it j0 .. j0+SY-1 and the forces are read.
template <int MODE> struct Layout {
    static constexpr bool STRESS = (MODE & P1_STRESS) != 0;
    static constexpr bool FIN = !STRESS && (MODE & P1_FORCES) != 0;
    static constexpr int CROWS = STRESS ? SY + 2 : SY;
    static constexpr int CROW0 = STRESS ? -1 : 0;
    static constexpr int O_CU = 0;                 // u1, u2, u3: CROWS rows each
    static constexpr int O_CR = O_CU + 3 * CROWS;  // density (deviation): SY rows
    static constexpr int O_F1 = O_CR + SY;         // x1 faces p, u1, u2, u3: SY rows each
    static constexpr int O_F2 = O_F1 + 4 * SY;     // x2 faces: SY + 1 rows each
    static constexpr int O_F3 = O_F2 + 4 * (SY + 1); // x3 faces of the plane: SY rows each
    static constexpr int O_FF = O_F3 + 4 * SY;     // f1, f2, f3: SY rows each (second Phase1)
    static constexpr int ROWS = O_FF + (FIN ? 3 * SY : 0);
    static constexpr int FLAG_OFF = ROWS * W * 4;
    static constexpr int STAGE = FLAG_OFF + CROWS * WF;
    static constexpr int SMEM = NS * STAGE;
};

// Offsets (floats / bytes within a stage) of what the thread of tile column (tx, ty) reads.
// cr = ty - CROW0 is the thread's cell row among the staged cell rows, cx = tx + 1 its column.
template <int MODE> __host__ __device__ inline int off_cu(int m, int cr, int cx) {
    return (Layout<MODE>::O_CU + m * Layout<MODE>::CROWS + cr) * W + cx;
}
template <int MODE> __host__ __device__ inline int off_cr(int ty, int cx) { return (Layout<MODE>::O_CR + ty) * W + cx; }
template <int MODE> __host__ __device__ inline int off_flag(int cr, int cx) { return Layout<MODE>::FLAG_OFF + cr * WF + cx; }
// face set d (0, 1, 2), array a (0 = p, 1..3 = u1..u3), staged row r, column x
template <int MODE> __host__ __device__ inline int off_face(int d, int a, int r, int x) {
    using L = Layout<MODE>;
    return d == 0 ? (L::O_F1 + a * SY + r) * W + x
                  : d == 1 ? (L::O_F2 + a * (SY + 1) + r) * W + x : (L::O_F3 + a * SY + r) * W + x;
}
template <int MODE> __host__ __device__ inline int off_ff(int m, int ty, int cx) {
    return (Layout<MODE>::O_FF + m * SY + ty) * W + cx;
}

// A group of row segments of one array: row j (row0 <= j < row0 + nrows, j <= maxrow) of plane
// p is copied from base + p*plane + j*pitch + xoff to stage + dst + (j - row0)*bytes.
struct Group {
    const char *base;
    long long plane;
    int pitch, xoff, bytes;
    int row0, nrows, maxrow;
    unsigned dst, when;
};

// The arrays a Phase1 launch stages.
struct Bases {
    const void *cu[3], *cr, *fl, *fc[3][4], *ff[3];
};

template <int MODE> __host__ __device__ inline int build_groups(Group *G, const Geom &g, const Bases &b, int bx, int by) {
    using L = Layout<MODE>;
    const int j0 = by * SY + 1;
    const int x0 = bx * SX;
    int n = 0;
    auto add = [&](const void *base, bool face, int elem, int bytes, int row0, int nrows, int dst, unsigned when) {
        Group &q = G[n++];
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
    const unsigned cells_when = L::STRESS ? (DOWN | MID | TOP) : MID;
    for (int m = 0; m < 3; ++m) add(b.cu[m], false, 4, W * 4, j0 + L::CROW0, L::CROWS, (L::O_CU + m * L::CROWS) * W * 4, cells_when);
    add(b.cr, false, 4, W * 4, j0, SY, L::O_CR * W * 4, MID);
    add(b.fl, false, 1, WF, j0 + L::CROW0, L::CROWS, L::FLAG_OFF, cells_when);
    for (int a = 0; a < 4; ++a) add(b.fc[0][a], true, 4, W * 4, j0, SY, off_face<MODE>(0, a, 0, 0) * 4, MID);
    for (int a = 0; a < 4; ++a) add(b.fc[1][a], true, 4, W * 4, j0, SY + 1, off_face<MODE>(1, a, 0, 0) * 4, MID);
    for (int a = 0; a < 4; ++a) add(b.fc[2][a], true, 4, W * 4, j0, SY, off_face<MODE>(2, a, 0, 0) * 4, MID | TOP);
    if (L::FIN)
        for (int m = 0; m < 3; ++m) add(b.ff[m], false, 4, W * 4, j0, SY, off_ff<MODE>(m, 0, 0) * 4, MID);
    return n;
}

__host__ __device__ inline int group_rows(const Group &q) {
    const int r = q.maxrow - q.row0 + 1;
    return r < q.nrows ? r : q.nrows;
}

__host__ __device__ inline unsigned plan_bytes(const Group *G, int n, unsigned kind) {
    unsigned t = 0;
    for (int q = 0; q < n; ++q)
        if (G[q].when & kind) t += (unsigned)(group_rows(G[q]) * G[q].bytes);
    return t;
}

template <int MODE> __host__ __device__ inline Bases bases_of(const DevState<float> &S, int src, int fcur) {
    Bases b;
    b.cu[0] = S.lv[src].u1;
    b.cu[1] = S.lv[src].u2;
    b.cu[2] = S.lv[src].u3;
    b.cr = S.lv[src].ro;
    b.fl = S.flags;
    for (int d = 0; d < 3; ++d) {
        b.fc[d][0] = S.fc[fcur][d].p;
        for (int a = 0; a < 3; ++a) b.fc[d][a + 1] = S.fc[fcur][d].u[a];
    }
    for (int m = 0; m < 3; ++m) b.ff[m] = S.f[m];
    return b;
}

// The rows of a block's plan, expanded: the global address of the row in plane 0, the plane
// stride, the row's offset in a stage, and the stage kinds that load it.
struct Row {
    const char *src;
    int plane;   // bytes per plane (every device array is below 2^31 bytes per plane)
    unsigned dw; // offset in the stage (low 24 bits) | stage kinds << 24
};
constexpr int kMaxRows = 96;    // float rows (74 with the stress, 80 without)
constexpr int kMaxFlagRows = 8; // flag rows (6 or 4)
constexpr int kChunks = W * 4 / 16, kFlagChunks = WF / 16; // 16-byte copies per row

__host__ __device__ inline void expand_rows(const Group *G, int ng, Row *fr, int &nfr, Row *gr, int &ngr) {
    nfr = ngr = 0;
    for (int q = 0; q < ng; ++q) {
        const Group &gq = G[q];
        for (int r = 0; r < group_rows(gq); ++r) {
            Row &w = gq.bytes == WF ? gr[ngr++] : fr[nfr++];
            w.src = gq.base + (long long)(gq.row0 + r) * gq.pitch + gq.xoff;
            w.plane = (int)gq.plane;
            w.dw = (gq.dst + (unsigned)(r * gq.bytes)) | (gq.when << 24);
        }
    }
}

// Planes per block: enough blocks for about eight waves of two blocks per SM on 152 SMs,
// between 8 and 64 planes.
inline int staged_chunk(const Geom &g) {
    const long long cols = (long long)tiles_x(g) * ((g.C2 + SY - 1) / SY);
    long long k = (long long)g.C3 * cols / (152 * 2 * 8);
    k = k < 8 ? 8 : (k > 64 ? 64 : k);
    return (int)k;
}
inline dim3 staged_grid(const Geom &g, int kch) { return dim3(tiles_x(g), (g.C2 + SY - 1) / SY, (g.C3 + kch - 1) / kch); }

#ifdef __CUDACC__
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp16(unsigned dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// One thread's share of a block's copy plan, resolved once before the plane loop: float rows
// r0, r0 + NT/kChunks, ... at 16-byte chunk ch of each row, and (for the first kFlagChunks *
// nfrow threads) one chunk of a flag row.  Per plane a copy is then one address computation.
template <int MAXR> struct MyCopies {
    const char *src[MAXR + 1]; // the copy's source in plane 0
    int plane[MAXR + 1];       // bytes per plane of its array
    unsigned dw[MAXR + 1];     // destination in the stage | stage kinds << 24 (0: no copy)
    template <int NT>
    __device__ __forceinline__ void resolve(const Row *rows, int nrow, const Row *frows, int nfrow, int t) {
        constexpr int kRowsPerPass = NT / kChunks;
        const int ch = t % kChunks, r0 = t / kChunks;
#pragma unroll
        for (int q = 0; q < MAXR; ++q) {
            const int R = r0 + q * kRowsPerPass;
            if (r0 < kRowsPerPass && R < nrow) {
                const Row w = rows[R];
                src[q] = w.src + 16 * ch;
                plane[q] = w.plane;
                dw[q] = w.dw + 16u * ch;
            } else {
                src[q] = nullptr;
                plane[q] = 0;
                dw[q] = 0;
            }
        }
        if (t < kFlagChunks * nfrow) {
            const Row w = frows[t / kFlagChunks];
            const int c = t % kFlagChunks;
            src[MAXR] = w.src + 16 * c;
            plane[MAXR] = w.plane;
            dw[MAXR] = w.dw + 16u * c;
        } else {
            src[MAXR] = nullptr;
            plane[MAXR] = 0;
            dw[MAXR] = 0;
        }
    }
    // the copies of plane p whose kinds include `kind`, into the stage at shared address `to`
    __device__ __forceinline__ void issue(unsigned to, int p, unsigned kind) const {
#pragma unroll
        for (int q = 0; q <= MAXR; ++q)
            if ((dw[q] >> 24) & kind) cp16(to + (dw[q] & 0xFFFFFFu), src[q] + (long long)p * plane[q]);
    }
};

// A block's copy plan expanded into rows (shared memory; filled by thread 0).
struct RowTable {
    Row rows[kMaxRows], frows[kMaxFlagRows];
    int nrow, nfrow;
};

// One block's work: tile (bx.x, bx.y) of 64 x 4 columns, planes of chunk bx.z (kch planes); sm
// holds the stages (Layout<MODE>::SMEM bytes).  Every thread of the block calls it; it ends with
// no copy in flight, so a persistent kernel may run it again for another tile.
template <int MODE>
__device__ __forceinline__ void phase1_staged_body(const DevState<float> &S, int src, int dst, int fcur, int kch,
                                                   const BIx &bx, unsigned char *sm, RowTable &rt) {
    using L = Layout<MODE>;
    using T = float;
    constexpr bool STRESS = L::STRESS;
    Row *rows = rt.rows, *frows = rt.frows;
    const Geom g = S.g;
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * SX + tx;
    const int bxi = bx.x, byi = bx.y;
    const int i = bxi * SX + tx + 1, j = byi * SY + ty + 1;
    const int k0 = bx.z * kch + 1;
    const int k1 = k0 + kch - 1 < g.C3 ? k0 + kch - 1 : g.C3;
    const int pfirst = STRESS ? k0 - 1 : k0, plast = k1 + 1;
    const unsigned sbase = smem_u32(sm);
    if (t == 0) {
        Group G[kMaxGroups];
        const int ng = build_groups<MODE>(G, g, bases_of<MODE>(S, src, fcur), bxi, byi);
        int a, b;
        expand_rows(G, ng, rows, a, frows, b);
        rt.nrow = a;
        rt.nfrow = b;
    }
    __syncthreads();
    // float rows: thread t copies chunk t % 17 of rows t / 17, t / 17 + 15, ...; flag rows: the
    // first 5 * (flag rows) threads one chunk each
    constexpr int kMine = (L::ROWS + NT / kChunks - 1) / (NT / kChunks);
    MyCopies<kMine> mine;
    mine.template resolve<NT>(rows, rt.nrow, frows, rt.nfrow, t);
    auto issue = [&](int p) {
        const unsigned to = sbase + (unsigned)(((p - pfirst) % NS) * L::STAGE);
        const unsigned kind = p < k0 ? DOWN : (p > k1 ? TOP : MID);
        mine.issue(to, p, kind);
    };
    // Pipeline: planes pfirst .. pfirst+NS-2 are issued up front; at plane k, once plane k+1
    // has landed and every thread is past plane k-1, the slot of the plane no longer needed
    // (k-2 with the stress, which reads planes k-1..k+1; else k-1) takes plane k+NS-2 (k+NS-1).
    // Every thread commits one group per issue (possibly empty), so the group counts agree.
    for (int p = pfirst; p < pfirst + NS - 1; ++p) {
        if (p <= plast) issue(p);
        cp_commit();
    }

    const K<T> &kk = kconst<T>(S.k);
    const T dt = sc_dt<T>(S.sc);
    const T G1 = (MODE & P1_BULK) ? sc_G<T>(S.sc) : (T)0;
    const bool valid = i <= g.C1 && j <= g.C2;
    const int cr = ty - L::CROW0, cx = tx + 1;
    unsigned long long m0 = 0, m1 = 0, m2 = 0;
    long long rsum = 0;
    for (int k = k0; k <= k1; ++k) {
        // issued so far: up to plane k + NS - 3 with the stress (NS - 4 more than plane k + 1),
        // k + NS - 2 without it (NS - 3 more)
        if (STRESS) cp_wait<NS - 4>();
        else cp_wait<NS - 3>();
        __syncthreads();
        {
            const int pn = k + NS - (STRESS ? 2 : 1);
            if (pn <= plast) issue(pn);
            cp_commit();
        }
        if (valid) {
            const T *fm = (const T *)(sm + ((k - pfirst) % NS) * L::STAGE);
            const T *fu = (const T *)(sm + ((k + 1 - pfirst) % NS) * L::STAGE);
            const uint8_t *flm = (const uint8_t *)fm;
            const int c = g.ci(i, j, k);
            const uint8_t fl = flm[off_flag<MODE>(cr, cx)];
            const T ro_c = fm[off_cr<MODE>(ty, cx)];
            const T uc[3] = {fm[off_cu<MODE>(0, cr, cx)], fm[off_cu<MODE>(1, cr, cx)], fm[off_cu<MODE>(2, cr, cx)]};
            T ro_cn, ucn[3], rden = (T)0;
            if (fl & FL_LT) {
                FaceVal<T> lo[3], hi[3];
                auto fv = [&](const T *f, int d, int r, int x) {
                    FaceVal<T> v;
                    v.p = f[off_face<MODE>(d, 0, r, x)];
                    v.ro = face_ro(v.p, kk);
                    v.u[0] = f[off_face<MODE>(d, 1, r, x)];
                    v.u[1] = f[off_face<MODE>(d, 2, r, x)];
                    v.u[2] = f[off_face<MODE>(d, 3, r, x)];
                    return v;
                };
                lo[0] = fv(fm, 0, ty, cx);
                hi[0] = fv(fm, 0, ty, cx + 1);
                lo[1] = fv(fm, 1, ty, cx);
                hi[1] = fv(fm, 1, ty + 1, cx);
                lo[2] = fv(fm, 2, ty, cx);
                hi[2] = fv(fu, 2, ty, cx);
                half_step(lo, hi, ro_c, uc, dt, kk, ro_cn, ucn, rden);
            } else {
                ucn[0] = ucn[1] = ucn[2] = (T)0;
                ro_cn = (T)0;
            }
            T f[3] = {(T)0, (T)0, (T)0};
            if (STRESS) {
                if (fl & FL_EQ0) {
                    const T *fd = (const T *)(sm + ((k - 1 - pfirst) % NS) * L::STAGE);
                    const uint8_t *fld = (const uint8_t *)fd, *flu = (const uint8_t *)fu;
                    uint8_t fln[6];
                    T un[6][3];
                    fln[0] = flm[off_flag<MODE>(cr, cx - 1)];
                    fln[1] = flm[off_flag<MODE>(cr, cx + 1)];
                    fln[2] = flm[off_flag<MODE>(cr - 1, cx)];
                    fln[3] = flm[off_flag<MODE>(cr + 1, cx)];
                    fln[4] = fld[off_flag<MODE>(cr, cx)];
                    fln[5] = flu[off_flag<MODE>(cr, cx)];
#pragma unroll
                    for (int m = 0; m < 3; ++m) {
                        un[0][m] = fm[off_cu<MODE>(m, cr, cx - 1)];
                        un[1][m] = fm[off_cu<MODE>(m, cr, cx + 1)];
                        un[2][m] = fm[off_cu<MODE>(m, cr - 1, cx)];
                        un[3][m] = fm[off_cu<MODE>(m, cr + 1, cx)];
                        un[4][m] = fd[off_cu<MODE>(m, cr, cx)];
                        un[5][m] = fu[off_cu<MODE>(m, cr, cx)];
                    }
                    const T ro_cf = kk.ro0 + ro_c;
                    stress_force(fln, un, fl, uc, ro_cf, kk, f);
                    if (MODE & P1_BULK) f[0] = bulk_force(f[0], ro_cf, kk, G1);
                }
                S.f[0][c] = f[0];
                S.f[1][c] = f[1];
                S.f[2][c] = f[2];
            } else if (MODE & P1_FORCES) {
                f[0] = fm[off_ff<MODE>(0, ty, cx)];
                f[1] = fm[off_ff<MODE>(1, ty, cx)];
                f[2] = fm[off_ff<MODE>(2, ty, cx)];
            }
            if ((MODE & P1_FORCES) && (fl & FL_EQ0)) use_forces_f32(ucn, f, dt, kk, rden); // UseForces
            S.lv[dst].ro[c] = ro_cn;
            S.lv[dst].u1[c] = ucn[0];
            S.lv[dst].u2[c] = ucn[1];
            S.lv[dst].u3[c] = ucn[2];
            if (MODE & P1_RMAX) {
                const unsigned long long b0 = abs_key(ucn[0]), b1 = abs_key(ucn[1]), b2 = abs_key(ucn[2]);
                m0 = b0 > m0 ? b0 : m0;
                m1 = b1 > m1 ? b1 : m1;
                m2 = b2 > m2 ? b2 : m2;
            }
            if ((MODE & P1_RSUM) && (fl & FL_EQ0)) rsum += fixed_sum_term(ucn[0]);
        }
    }
    cp_wait<0>();
    if (MODE & (P1_RMAX | P1_RSUM)) tile_store<T, NT>(S, bx, (MODE & P1_RMAX) != 0, (MODE & P1_RSUM) != 0, m0, m1, m2, rsum);
}

template <int MODE>
__global__ void __launch_bounds__(NT, 2)
    k_phase1_staged(const __grid_constant__ DevState<float> S, int src, int dst, int fcur, int kch) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ RowTable rt;
    phase1_staged_body<MODE>(S, src, dst, fcur, kch, bix_here(), sm, rt);
}

template <int MODE> inline void launch_staged(const DevState<float> &S, int src, int dst, int fcur, cudaStream_t st) {
    const int kch = staged_chunk(S.g);
    k_phase1_staged<MODE><<<staged_grid(S.g, kch), dim3(SX, SY), Layout<MODE>::SMEM, st>>>(S, src, dst, fcur, kch);
}
template <int MODE> inline void prepare_staged() {
    cudaFuncSetAttribute(k_phase1_staged<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, Layout<MODE>::SMEM);
    cudaFuncSetAttribute(k_phase1_staged<MODE>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}
#endif

} // namespace stg
