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
//
// The TMA form (k_phase1_tma) stages the same planes with tensor-map copies instead: one
// thread issues, per plane, one 4-D box per block of arrays (a level's ro, u1, u2, u3; a face
// set's p, u1, u2, u3; the forces; the flags), and the threads wait on the stage's mbarrier.
// It needs each block of arrays in one allocation, a fixed stride apart (the contexts allocate
// them that way), and lays the stage out with 128-byte aligned boxes.
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
    // offsets (floats; flags in bytes) of what the thread of tile column (tx, ty) reads:
    // cr = ty - CROW0 is its cell row among the staged cell rows, cx = tx + 1 its column
    __host__ __device__ static int cu(int m, int cr, int cx) { return (O_CU + m * CROWS + cr) * W + cx; }
    __host__ __device__ static int ro(int ty, int cx) { return (O_CR + ty) * W + cx; }
    __host__ __device__ static int flag(int cr, int cx) { return FLAG_OFF + cr * WF + cx; }
    // face set d (0, 1, 2), array a (0 = p, 1..3 = u1..u3), staged row r, column x
    __host__ __device__ static int face(int d, int a, int r, int x) {
        return d == 0 ? (O_F1 + a * SY + r) * W + x : d == 1 ? (O_F2 + a * (SY + 1) + r) * W + x : (O_F3 + a * SY + r) * W + x;
    }
    __host__ __device__ static int ff(int m, int ty, int cx) { return (O_FF + m * SY + ty) * W + cx; }
};

// The TMA form's stage for a TSX x TSY tile: one box per block of arrays, each at a 128-byte
// boundary.  The level's four arrays (ro first) all take the cell rows (the stress's halo rows
// of ro are copied too).  Rows of W = TSX + 4 values (cells i0-1 .. i0+TSX+2) and WF flag bytes
// (TSX + 2 rounded up to 16).  Five stages when two blocks per SM hold them, else four.
constexpr int pad32(int f) { return (f + 31) / 32 * 32; } // floats to a 128-byte boundary
template <int MODE, int TSX = 64, int TSY = 4> struct TLayout {
    static constexpr bool STRESS = (MODE & P1_STRESS) != 0;
    static constexpr bool FIN = !STRESS && (MODE & P1_FORCES) != 0;
    static constexpr int SX = TSX, SY = TSY, NT = TSX * TSY;
    static constexpr int W = TSX + 4, WF = (TSX + 2 + 15) / 16 * 16;
    static constexpr int CROWS = STRESS ? SY + 2 : SY;
    static constexpr int CROW0 = STRESS ? -1 : 0;
    static constexpr int O_LV = 0;                                  // ro, u1, u2, u3: CROWS rows each
    static constexpr int O_F1 = pad32(O_LV + 4 * CROWS * W);        // x1 faces p, u1, u2, u3: SY rows each
    static constexpr int O_F2 = pad32(O_F1 + 4 * SY * W);           // x2 faces: SY + 1 rows each
    static constexpr int O_F3 = pad32(O_F2 + 4 * (SY + 1) * W);     // x3 faces: SY rows each
    static constexpr int O_FF = pad32(O_F3 + 4 * SY * W);           // f1, f2, f3: SY rows each
    static constexpr int END = pad32(O_FF + (FIN ? 3 * SY * W : 0));
    static constexpr int FLAG_OFF = END * 4;
    static constexpr int STAGE = (FLAG_OFF + CROWS * WF + 127) / 128 * 128;
    // two blocks per SM (228 KB of shared memory, 1 KB of it reserved per block; 128 bytes for
    // the alignment of the stages, 512 of static shared memory)
    static constexpr int NS = 2 * (5 * STAGE + 128 + 512 + 1024) <= 228 * 1024 ? 5 : 4;
    static constexpr int SMEM = NS * STAGE;
    static_assert(2 * (SMEM + 128 + 512 + 1024) <= 228 * 1024, "TMA stages: two blocks per SM");
    static_assert(W * 4 % 16 == 0 && TSX % 16 == 0, "rows of whole 16-byte units from 16-byte aligned x");
    __host__ __device__ static int cu(int m, int cr, int cx) { return O_LV + ((m + 1) * CROWS + cr) * W + cx; }
    __host__ __device__ static int ro(int ty, int cx) { return O_LV + (ty - CROW0) * W + cx; }
    __host__ __device__ static int flag(int cr, int cx) { return FLAG_OFF + cr * WF + cx; }
    __host__ __device__ static int face(int d, int a, int r, int x) {
        return d == 0 ? O_F1 + (a * SY + r) * W + x : d == 1 ? O_F2 + (a * (SY + 1) + r) * W + x : O_F3 + (a * SY + r) * W + x;
    }
    __host__ __device__ static int ff(int m, int ty, int cx) { return O_FF + (m * SY + ty) * W + cx; }
};

// The cp.async form's offsets as free functions (the host plan check uses them).
template <int MODE> __host__ __device__ inline int off_cu(int m, int cr, int cx) { return Layout<MODE>::cu(m, cr, cx); }
template <int MODE> __host__ __device__ inline int off_cr(int ty, int cx) { return Layout<MODE>::ro(ty, cx); }
template <int MODE> __host__ __device__ inline int off_flag(int cr, int cx) { return Layout<MODE>::flag(cr, cx); }
template <int MODE> __host__ __device__ inline int off_face(int d, int a, int r, int x) { return Layout<MODE>::face(d, a, r, x); }
template <int MODE> __host__ __device__ inline int off_ff(int m, int ty, int cx) { return Layout<MODE>::ff(m, ty, cx); }

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
// The same for a TSX x TSY tile of the TMA form.
template <int TSX, int TSY> inline int tile_chunk(const Geom &g) {
    const long long cols = (long long)((g.C1 + TSX - 1) / TSX) * ((g.C2 + TSY - 1) / TSY);
    long long k = (long long)g.C3 * cols / (152 * 2 * 8);
    k = k < 8 ? 8 : (k > 64 ? 64 : k);
    return (int)k;
}
template <int TSX, int TSY> inline dim3 tile_grid(const Geom &g, int kch) {
    return dim3((g.C1 + TSX - 1) / TSX, (g.C2 + TSY - 1) / TSY, (g.C3 + kch - 1) / kch);
}


// ---- TMA form: the boxes of a plane ----
// One block of n arrays (a level's ro, u1, u2, u3; a face set's p, u1, u2, u3; f1, f2, f3; or
// the flags alone), each planes x rows x pitch elements, the arrays `stride[2]` bytes apart.
// Per plane p a block copies elements x0 .. x0 + box[0] - 1 of rows j0 + row0 .. j0 + row0 +
// box[1] - 1 of each array into the stage at dst, array a row r at dst + (a * box[1] + r) *
// box[0] * elem.  Rows past the last come back as zeros (no valid cell reads them).
struct TmaBox {
    const void *base;
    int elem;            // bytes per element: 4 or 1
    long long dim[4];    // elements per row (the pitch), rows, planes, arrays
    long long stride[3]; // bytes between rows, planes, arrays
    int box[4];          // elements, rows, planes (1), arrays
    int row0;            // first row, relative to the tile's first row j0
    unsigned dst;        // byte offset in the stage
    unsigned when;       // the stage kinds (DOWN, MID, TOP) that load it
};
constexpr int kMaxBoxes = 6;

// The box of n arrays from base, `astride` bytes apart, cell (face = false) or face rows of g:
// bw elements by br rows from row j0 + row0, into the stage at dst, loaded by planes of `when`.
inline TmaBox make_box(const Geom &g, const void *base, int elem, bool face, int narr, long long astride, int bw, int br,
                       int row0, int dst, unsigned when) {
    TmaBox q;
    q.base = base;
    q.elem = elem;
    q.dim[0] = face ? g.fs1 : g.cs1;
    q.dim[1] = face ? g.C2 + 3 : g.C2 + 2;
    q.dim[2] = face ? g.C3 + 3 : g.C3 + 2;
    q.dim[3] = narr;
    q.stride[0] = (face ? g.fs1 : g.cs1) * elem;
    q.stride[1] = (face ? g.fs2 : g.cs2) * elem;
    q.stride[2] = astride;
    q.box[0] = bw;
    q.box[1] = br;
    q.box[2] = 1;
    q.box[3] = narr;
    q.row0 = row0;
    q.dst = (unsigned)dst;
    q.when = when;
    return q;
}
// The stride of n arrays that must lie a fixed stride apart, each of at least min_bytes (0 if
// they do not, or the stride is no multiple of 16 or not below 2^40, as tensor maps need).
inline long long block_stride(const void *const *arr, int n, long long min_bytes) {
    const long long s = (long long)((const char *)arr[1] - (const char *)arr[0]);
    if (s < min_bytes || s % 16 || s >= (1ll << 40)) return 0;
    for (int q = 2; q < n; ++q)
        if ((long long)((const char *)arr[q] - (const char *)arr[0]) != q * s) return 0;
    return s;
}
// The row and plane strides of g in bytes are multiples of 16 (tensor maps need it).
inline bool rows_fit(const Geom &g) { return (g.cs1 % 16) == 0 && (g.fs1 % 16) == 0 && (g.cs2 % 16) == 0 && (g.fs2 % 16) == 0; }

// The boxes of a launch of the TMA form, from the staged arrays (Bases); 0 when the arrays
// of a block are not a fixed stride apart (then the cp.async form runs) or a stride is out of
// the tensor maps' range.
template <int MODE, int TSX = 64, int TSY = 4> inline int tma_boxes(TmaBox *B, const Geom &g, const Bases &b) {
    using L = TLayout<MODE, TSX, TSY>;
    const long long nc = g.ncell(), nf = g.nface();
    const void *lv[4] = {b.cr, b.cu[0], b.cu[1], b.cu[2]};
    const long long lvs = block_stride(lv, 4, nc * 4);
    long long fcs[3];
    for (int d = 0; d < 3; ++d) fcs[d] = block_stride(b.fc[d], 4, nf * 4);
    const long long ffs = L::FIN ? block_stride(b.ff, 3, nc * 4) : 1;
    if (!lvs || !fcs[0] || !fcs[1] || !fcs[2] || !ffs || !rows_fit(g)) return 0;
    const unsigned cells_when = L::STRESS ? (DOWN | MID | TOP) : MID;
    int n = 0;
    B[n++] = make_box(g, b.cr, 4, false, 4, lvs, L::W, L::CROWS, L::CROW0, L::O_LV * 4, cells_when);
    B[n++] = make_box(g, b.fl, 1, false, 1, nc, L::WF, L::CROWS, L::CROW0, L::FLAG_OFF, cells_when);
    B[n++] = make_box(g, b.fc[0][0], 4, true, 4, fcs[0], L::W, L::SY, 0, L::O_F1 * 4, MID);
    B[n++] = make_box(g, b.fc[1][0], 4, true, 4, fcs[1], L::W, L::SY + 1, 0, L::O_F2 * 4, MID);
    B[n++] = make_box(g, b.fc[2][0], 4, true, 4, fcs[2], L::W, L::SY, 0, L::O_F3 * 4, MID | TOP);
    if (L::FIN) B[n++] = make_box(g, b.ff[0], 4, false, 3, ffs, L::W, L::SY, 0, L::O_FF * 4, MID);
    return n;
}
inline unsigned box_bytes(const TmaBox &q) { return (unsigned)(q.box[0] * q.box[1] * q.box[2] * q.box[3] * q.elem); }

#ifdef __CUDACC__
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp16(unsigned dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// A cell's values after Phase1: the half-step level written (ro_n, un), the level read (ro_c,
// uc) and the flags (what the folded x1 sweep extrapolates from).
struct XCell {
    float ro_n, un[3], ro_c, uc[3];
    uint8_t fl;
};

// One cell (i, j, k) of a staged Phase1 from the stages of planes k - 1 (sd, read with the
// stress), k (sk) and k + 1 (su), offsets by the stage layout L; the thread's tile column (tx, ty).
// The arithmetic of k_phase1_cell, in the same order.  xo (when given): the cell's values.
template <int MODE, class L>
__device__ __forceinline__ void staged_cell(const DevState<float> &S, int dst, const unsigned char *sd,
                                            const unsigned char *sk, const unsigned char *su, int i, int j, int k,
                                            int tx, int ty, const K<float> &kk, float dt, float G1, unsigned long long &m0,
                                            unsigned long long &m1, unsigned long long &m2, long long &rsum,
                                            XCell *xo = nullptr) {
    using T = float;
    constexpr bool STRESS = L::STRESS;
    const Geom &g = S.g;
    const int cr = ty - L::CROW0, cx = tx + 1;
    const T *fm = (const T *)sk, *fu = (const T *)su;
    const uint8_t *flm = sk;
    const int c = g.ci(i, j, k);
    const uint8_t fl = flm[L::flag(cr, cx)];
    const T ro_c = fm[L::ro(ty, cx)];
    const T uc[3] = {fm[L::cu(0, cr, cx)], fm[L::cu(1, cr, cx)], fm[L::cu(2, cr, cx)]};
    T ro_cn, ucn[3], rden = (T)0;
    if (fl & FL_LT) {
        FaceVal<T> lo[3], hi[3];
        auto fv = [&](const T *f, int d, int r, int x) {
            FaceVal<T> v;
            v.p = f[L::face(d, 0, r, x)];
            v.ro = face_ro(v.p, kk);
            v.u[0] = f[L::face(d, 1, r, x)];
            v.u[1] = f[L::face(d, 2, r, x)];
            v.u[2] = f[L::face(d, 3, r, x)];
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
            const T *fd = (const T *)sd;
            const uint8_t *fld = sd, *flu = su;
            uint8_t fln[6];
            T un[6][3];
            fln[0] = flm[L::flag(cr, cx - 1)];
            fln[1] = flm[L::flag(cr, cx + 1)];
            fln[2] = flm[L::flag(cr - 1, cx)];
            fln[3] = flm[L::flag(cr + 1, cx)];
            fln[4] = fld[L::flag(cr, cx)];
            fln[5] = flu[L::flag(cr, cx)];
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                un[0][m] = fm[L::cu(m, cr, cx - 1)];
                un[1][m] = fm[L::cu(m, cr, cx + 1)];
                un[2][m] = fm[L::cu(m, cr - 1, cx)];
                un[3][m] = fm[L::cu(m, cr + 1, cx)];
                un[4][m] = fd[L::cu(m, cr, cx)];
                un[5][m] = fu[L::cu(m, cr, cx)];
            }
            const T ro_cf = kk.ro0 + ro_c;
            stress_force(fln, un, fl, uc, ro_cf, kk, f);
            if (MODE & P1_BULK) f[0] = bulk_force(f[0], ro_cf, kk, G1);
        }
        S.f[0][c] = f[0];
        S.f[1][c] = f[1];
        S.f[2][c] = f[2];
    } else if (MODE & P1_FORCES) {
        f[0] = fm[L::ff(0, ty, cx)];
        f[1] = fm[L::ff(1, ty, cx)];
        f[2] = fm[L::ff(2, ty, cx)];
    }
    if ((MODE & P1_FORCES) && (fl & FL_EQ0)) use_forces_f32(ucn, f, dt, kk, rden); // UseForces
    S.lv[dst].ro[c] = ro_cn;
    S.lv[dst].u1[c] = ucn[0];
    S.lv[dst].u2[c] = ucn[1];
    S.lv[dst].u3[c] = ucn[2];
    if (xo) {
        xo->ro_n = ro_cn;
        xo->ro_c = ro_c;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            xo->un[m] = ucn[m];
            xo->uc[m] = uc[m];
        }
        xo->fl = fl;
    }
    if (MODE & P1_RMAX) {
        const unsigned long long b0 = abs_key(ucn[0]), b1 = abs_key(ucn[1]), b2 = abs_key(ucn[2]);
        m0 = b0 > m0 ? b0 : m0;
        m1 = b1 > m1 ? b1 : m1;
        m2 = b2 > m2 ? b2 : m2;
    }
    if ((MODE & P1_RSUM) && (fl & FL_EQ0)) rsum += fixed_sum_term(ucn[0]);
}

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
            const unsigned char *sk = sm + ((k - pfirst) % NS) * L::STAGE;
            const unsigned char *su = sm + ((k + 1 - pfirst) % NS) * L::STAGE;
            const unsigned char *sd = STRESS ? sm + ((k - 1 - pfirst) % NS) * L::STAGE : sk;
            staged_cell<MODE, L>(S, dst, sd, sk, su, i, j, k, tx, ty, kk, dt, G1, m0, m1, m2, rsum);
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

// kch: planes per block (0: staged_chunk's choice)
template <int MODE> inline void launch_staged(const DevState<float> &S, int src, int dst, int fcur, cudaStream_t st, int kch_in = 0) {
    const int kch = kch_in > 0 ? (kch_in < S.g.C3 ? kch_in : S.g.C3) : staged_chunk(S.g);
    k_phase1_staged<MODE><<<staged_grid(S.g, kch), dim3(SX, SY), Layout<MODE>::SMEM, st>>>(S, src, dst, fcur, kch);
}
template <int MODE> inline void prepare_staged() {
    cudaFuncSetAttribute(k_phase1_staged<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, Layout<MODE>::SMEM);
    cudaFuncSetAttribute(k_phase1_staged<MODE>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

// ---- TMA form: the kernel ----
// What each box of a launch loads (the same for every grid of one kernel form).
struct BoxMeta {
    int row0[kMaxBoxes];
    unsigned dst[kMaxBoxes], when[kMaxBoxes];
    unsigned bytes[5]; // the bytes a plane of kind DOWN (1), MID (2) or TOP (4) brings
    int n;
};
// The tensor maps of a launch (kernel parameters) and their boxes.
struct TmaArgs {
    CUtensorMap map[kMaxBoxes];
    BoxMeta m;
};

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(unsigned bar) { asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(bar) : "memory"); }
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity) {
    unsigned done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return done != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Waits for the phase of the given parity to complete; false after about limit_ns.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, unsigned long long limit_ns) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try(bar, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// A tensor map in global memory (written before the launch) made visible to the copy engine.
__device__ __forceinline__ void fence_tensormap(const CUtensorMap *m) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(m) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// One 4-D box (x, row, plane, array) into shared memory, completing on bar.
__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap *map, int x, int y, int z, int w, unsigned bar) {
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
                 ::"r"(dst), "l"(map), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
                 : "memory");
}

// One side of a seam face in X (q: X.b or X.a): the three extrapolated values, the cell's
// half-step values and (fl) its flags.
__device__ __forceinline__ void seam_put(float *const *q, int s, float e0, float e1, float e2, const XCell &c, bool fl) {
    q[0][s] = e0;
    q[1][s] = e1;
    q[2][s] = e2;
    q[3][s] = c.un[0];
    q[4][s] = c.un[1];
    q[5][s] = c.un[2];
    q[6][s] = c.ro_n;
    if (fl) q[7][s] = __int_as_float((int)c.fl);
}
// One block's work in the staged Phase1 with TMA copies: tile (bx.x, bx.y) of TSX x TSY columns,
// planes of chunk bx.z (kch planes), by TSX * TSY consumer threads (one cell column each) and
// one producer warp (threads TSX * TSY ..; its lane 0 works).  The producer issues a plane's
// boxes into its stage (NS stages) once every consumer warp has released the plane the slot
// held; every consumer waits for the planes it reads on the stage's "full" mbarrier and each
// consumer warp, done with a plane, arrives on the stage's "empty" mbarrier.  No block-wide
// barrier runs per plane.  A consumer at plane k reads k - 1 (with the stress), k and k + 1
// and then releases k - 1 (with the stress) or k.  bar: NS full, NS empty mbarriers and an
// abort flag.  map(q) is box q's tensor map (global maps are fenced for the tensor-map proxy
// first when fence_maps is set).  A wait that does not end within half a second sets
// STATUS_STAGING and the abort flag; every thread then leaves its loop (at most one more
// bounded wait each), and the block lets its copies in flight land (again with a limit) and
// leaves.  Every thread calls it; it ends with no copy in flight and the mbarriers
// invalidated, so a persistent kernel may run it again.
//
// XS & 1 (Phase1 + stress only): the x1 sweep folded in.  The x extrapolation of a cell needs its
// half-step values (just computed), its old values and its two old x faces (staged), so per
// plane every cell also extrapolates along x (main.cpp:1756-1873) and updates the x face below
// it from the cell behind (main.cpp:1920-2008): the lane before, or for the first lane of a
// tile row's second warp the last lane of the first, handed over through shared memory (xh: a
// slot per plane of a ring of NS, completed on its own mbarrier with a bounded wait; the first
// warp can run at most NS - 2 planes ahead of the second, since the stages it needs are only
// refilled once the second has released them, so a slot is never rewritten before it was
// read).  The faces at the tiles' seams (below a tile's first column, and face C1 + 1) are
// left to k_sweep_x_seams: the tile's first and last cells write all that their side of such a
// face needs into X (see XSeams).  Same arithmetic, same inputs, same bits as k_sweep_x.
//
// XS & 2: the x3 sweep folded in too.  A cell's z extrapolation needs its two old z faces, both
// staged (its plane's and the plane above's), and the z face below a cell needs the cell one
// plane down: this thread's previous plane, carried in registers.  So every plane but the
// chunk's first also updates the z face below its cells (main.cpp:2261-2494, the x3 sweep's
// extrapolate and face_values with the same inputs).  The face below a chunk's first plane and
// face C3 + 1 are left to k_sweep_z_seams: contiguous rows of faces, coalesced.
template <int TSX, int TSY, int NS> struct XHand {
    static constexpr int NH = TSX / 32 > 1 ? TSX / 32 - 1 : 1; // hand-overs per row
    unsigned long long bar[TSY][NH][NS];
    float v[TSY][NH][NS][8]; // rf, af, bf, u1, u2, u3, ro of the half-step level, flags
};
template <int MODE, int TSX, int TSY, int XS = 0, class Maps>
__device__ __forceinline__ void phase1_tma_body(const DevState<float> &S, const Maps &map, const BoxMeta &A, bool fence_maps,
                                                int src, int dst, int kch, const BIx &bx, unsigned char *sm,
                                                unsigned long long *bar, int fcur = 0, const XSeams *X = nullptr,
                                                XHand<TSX, TSY, TLayout<MODE, TSX, TSY>::NS> *xh = nullptr) {
    using L = TLayout<MODE, TSX, TSY>;
    using T = float;
    constexpr bool STRESS = L::STRESS;
    constexpr int NS = L::NS, SX = TSX, SY = TSY, NT = TSX * TSY;
    constexpr int NW = TSX / 32; // warps per tile row
    static_assert(!XS || (STRESS && TSX % 32 == 0), "the x1 sweep folds into Phase1 + stress, whole warps per row");
    constexpr unsigned long long kLimitNs = 500000000ull;
    const Geom g = S.g;
    const int t = threadIdx.y * blockDim.x + threadIdx.x, tx = t % SX, ty = t / SX;
    const bool consumer = t < NT;
    const int i = bx.x * SX + tx + 1, j = bx.y * SY + ty + 1;
    const int x0 = bx.x * SX, j0 = bx.y * SY + 1;
    const int k0 = bx.z * kch + 1;
    const int k1 = k0 + kch - 1 < g.C3 ? k0 + kch - 1 : g.C3;
    const int pfirst = STRESS ? k0 - 1 : k0, plast = k1 + 1;
    const unsigned sbase = smem_u32(sm);
    auto bar_of = [&](int p) { return smem_u32(&bar[(p - pfirst) % NS]); };       // full
    auto empty_of = [&](int p) { return smem_u32(&bar[NS + (p - pfirst) % NS]); }; // empty
    auto parity_of = [&](int p) { return (unsigned)(((p - pfirst) / NS) & 1); };
    volatile unsigned long long *const abort_flag = bar + 2 * NS;
    if (t == NT) {
        if (fence_maps)
            for (int q = 0; q < A.n; ++q) fence_tensormap(map(q));
        for (int q = 0; q < NS; ++q) {
            mbar_init(smem_u32(&bar[q]), 1);
            mbar_init(smem_u32(&bar[NS + q]), NT / 32);
        }
        if ((XS & 1) && NW > 1)
            for (int r = 0; r < SY; ++r)
                for (int h = 0; h < NW - 1; ++h)
                    for (int q = 0; q < NS; ++q) mbar_init(smem_u32(&xh->bar[r][h][q]), 1);
        *abort_flag = 0;
        fence_mbar_init();
        fence_proxy_async();
    }
    __syncthreads();

    bool failed = false;
    int issued = pfirst - 1; // the producer: the last plane issued
    unsigned long long m0 = 0, m1 = 0, m2 = 0;
    long long rsum = 0;
    if (t == NT) { // the producer
        for (int p = pfirst; p <= plast; ++p) {
            // the slot's previous plane, p - NS, released by every consumer warp
            if (p - NS >= pfirst && !mbar_wait(empty_of(p - NS), parity_of(p - NS), kLimitNs)) {
                *abort_flag = 1;
                failed = true;
                break;
            }
            if (*abort_flag) break;
            const unsigned kind = p < k0 ? DOWN : (p > k1 ? TOP : MID);
            const unsigned to = sbase + (unsigned)(((p - pfirst) % NS) * L::STAGE), b = bar_of(p);
            fence_proxy_async();
            mbar_expect_tx(b, A.bytes[kind]);
            for (int q = 0; q < A.n; ++q)
                if (A.when[q] & kind) tma_load_4d(to + A.dst[q], map(q), x0, j0 + A.row0[q], p, 0, b);
            issued = p;
        }
    } else if (consumer) {
        const K<T> &kk = kconst<T>(S.k);
        const T dt = sc_dt<T>(S.sc);
        const T G1 = (MODE & P1_BULK) ? sc_G<T>(S.sc) : (T)0;
        const bool valid = i <= g.C1 && j <= g.C2;
        // the folded x1 sweep: its constants and output faces; the warp's place in the tile row
        // and whether its first lane's face takes a hand-over (warp-uniform)
        const SweepK<T> qx = (XS & 1) ? sweep_consts(S, 0) : SweepK<T>{};
        const FaceOut<T> WX = (XS & 1) ? sweep_out(S, fcur, 0) : FaceOut<T>{};
        const int lane = t & 31, w = tx >> 5;
        const bool takes = (XS & 1) && NW > 1 && w > 0 && x0 + 32 * w + 1 <= g.C1 && j <= g.C2;
        // the folded x3 sweep: its constants and output faces; the cell one plane down (its
        // forward extrapolation, half-step u3, u1, u2, density, flags)
        const SweepK<T> qz = (XS & 2) ? sweep_consts(S, 2) : SweepK<T>{};
        const FaceOut<T> WZ = (XS & 2) ? sweep_out(S, fcur, 2) : FaceOut<T>{};
        Ext<T> zprev = {};
        T zun = (T)0, zua = (T)0, zub = (T)0, zro = (T)0;
        uint8_t zfl = 0;
        for (int k = k0; k <= k1; ++k) {
            bool ok = true;
            if (k == k0) {
                if (STRESS) ok = mbar_wait(bar_of(k - 1), parity_of(k - 1), kLimitNs);
                ok = ok && mbar_wait(bar_of(k), parity_of(k), kLimitNs);
            }
            ok = ok && mbar_wait(bar_of(k + 1), parity_of(k + 1), kLimitNs);
            if (!ok) *abort_flag = 1;
            // warp-uniform (the warp's lanes meet at __syncwarp below)
            if (__any_sync(0xffffffffu, !ok || *abort_flag != 0)) {
                failed = true;
                break;
            }
            const unsigned char *sk = sm + ((k - pfirst) % NS) * L::STAGE;
            const unsigned char *su = sm + ((k + 1 - pfirst) % NS) * L::STAGE;
            XCell xc = {};
            if (valid) {
                const unsigned char *sd = STRESS ? sm + ((k - 1 - pfirst) % NS) * L::STAGE : sk;
                staged_cell<MODE, L>(S, dst, sd, sk, su, i, j, k, tx, ty, kk, dt, G1, m0, m1, m2, rsum, XS ? &xc : nullptr);
            }
            if constexpr ((XS & 2) != 0) {
                // the cell's z extrapolation (the x3 sweep's: normal u3, tangential u1 and u2)
                const T *fm = (const T *)sk, *fu = (const T *)su;
                const int cx = tx + 1;
                auto Z = [&](const T *f, int a) { return f[L::face(2, a, ty, cx)]; };
                if (valid) {
                    const Ext<T> ez =
                        extrapolate<T, true>(Z(fu, 3), Z(fm, 3), xc.un[2], xc.uc[2], Z(fu, 1), Z(fm, 1), xc.un[0], xc.uc[0],
                                             Z(fu, 2), Z(fm, 2), xc.un[1], xc.uc[1], xc.ro_n, xc.ro_c, Z(fu, 0), Z(fm, 0), qz);
                    if (k > k0) { // the face below the cell (main.cpp:1920-2008 as the x3 sweep applies it)
                        NVals<T> nv;
                        nv.a[0] = zua;
                        nv.b[0] = zub;
                        nv.r[0] = zro;
                        nv.a[1] = xc.un[0];
                        nv.b[1] = xc.un[1];
                        nv.r[1] = xc.ro_n;
                        face_store(WZ, ARK_CK(g.fi(i, j, k), WZ.nf),
                                   face_values_v<T, false>(nv, zfl, xc.fl, zun, xc.un[2], zprev, ez, Z(fm, 1), Z(fm, 2), qz));
                    }
                    zprev = ez;
                    zun = xc.un[2];
                    zua = xc.un[0];
                    zub = xc.un[1];
                    zro = xc.ro_n;
                    zfl = xc.fl;
                }
            }
            if constexpr ((XS & 1) != 0) {
                // the cell's x extrapolation (the x1 sweep's extrapolate, from the same values)
                const T *fm = (const T *)sk;
                const int cx = tx + 1;
                auto F = [&](int a, int x) { return fm[L::face(0, a, ty, x)]; };
                Ext<T> e = {};
                T uAo = (T)0, uBo = (T)0;
                if (valid) {
                    e = extrapolate<T, true>(F(1, cx + 1), F(1, cx), xc.un[0], xc.uc[0], F(2, cx + 1), F(2, cx), xc.un[1],
                                             xc.uc[1], F(3, cx + 1), F(3, cx), xc.un[2], xc.uc[2], xc.ro_n, xc.ro_c,
                                             F(0, cx + 1), F(0, cx), qx);
                    uAo = F(2, cx);
                    uBo = F(3, cx);
                }
                // the cell behind the face below: the lane before
                Ext<T> pv = {};
                NVals<T> nv;
                pv.rf = __shfl_up_sync(0xffffffffu, e.rf, 1);
                pv.af = __shfl_up_sync(0xffffffffu, e.af, 1);
                pv.bf = __shfl_up_sync(0xffffffffu, e.bf, 1);
                T ucb = __shfl_up_sync(0xffffffffu, xc.un[0], 1);
                nv.a[0] = __shfl_up_sync(0xffffffffu, xc.un[1], 1);
                nv.b[0] = __shfl_up_sync(0xffffffffu, xc.un[2], 1);
                nv.r[0] = __shfl_up_sync(0xffffffffu, xc.ro_n, 1);
                int flb = __shfl_up_sync(0xffffffffu, (int)xc.fl, 1);
                nv.a[1] = xc.un[1];
                nv.b[1] = xc.un[2];
                nv.r[1] = xc.ro_n;
                if constexpr (NW > 1) {
                    // hand-over within the tile row: warp w's last lane to warp w + 1's first
                    const int u = k - k0, slot = u % NS;
                    const unsigned par = (unsigned)((u / NS) & 1);
                    if (w < NW - 1 && lane == 31) {
                        float *hv = xh->v[ty][w][slot];
                        hv[0] = e.rf;
                        hv[1] = e.af;
                        hv[2] = e.bf;
                        hv[3] = xc.un[0];
                        hv[4] = xc.un[1];
                        hv[5] = xc.un[2];
                        hv[6] = xc.ro_n;
                        hv[7] = __int_as_float((int)xc.fl);
                        mbar_arrive(smem_u32(&xh->bar[ty][w][slot])); // releases the writes above
                    }
                    bool got = true;
                    if (takes) got = mbar_wait(smem_u32(&xh->bar[ty][w - 1][slot]), par, kLimitNs);
                    if (!got) *abort_flag = 1;
                    if (__any_sync(0xffffffffu, !got)) {
                        failed = true;
                        break;
                    }
                    if (takes && lane == 0) {
                        const float *hv = xh->v[ty][w - 1][slot];
                        pv.rf = hv[0];
                        pv.af = hv[1];
                        pv.bf = hv[2];
                        ucb = hv[3];
                        nv.a[0] = hv[4];
                        nv.b[0] = hv[5];
                        nv.r[0] = hv[6];
                        flb = __float_as_int(hv[7]);
                    }
                }
                if (valid && tx != 0) // the face below the cell (main.cpp:1920-2008)
                    face_store(WX, ARK_CK(g.fi(i, j, k), WX.nf),
                               face_values_v<T, false>(nv, (uint8_t)flb, xc.fl, ucb, xc.un[0], pv, e, uAo, uBo, qx));
                const bool px = S.k.periodic_x;
                const uint8_t *flm = sk;
                if (valid && tx == 0) { // the tile's seam b = bx.x: the cell ahead of its face
                    const int s = ARK_CK(seam_slot(g, SX, bx.x, j, k), X->n);
                    seam_put(X->a, s, e.qb, e.ab, e.bb, xc, true);
                    X->a[8][s] = uAo;
                    X->a[9][s] = uBo;
                    if (i == 1) { // face 1: the ghost position 0 behind it (its own flags), the face's u1, p
                        X->b[7][s] = __int_as_float((int)flm[L::flag(ty - L::CROW0, cx - 1)]);
                        X->a[10][s] = F(1, cx);
                        X->a[11][s] = F(0, cx);
                        if (!px) // bounded: the inflow invariant, the values of cell 1 (xcell)
                            seam_put(X->b, s, (xc.fl & FL_LT) ? (T)1 : (T)0, (T)0, (T)0, xc, false);
                    }
                }
                if (valid && (tx == SX - 1 || i == g.C1)) { // seam bx.x + 1: the cell behind its face
                    const int s = ARK_CK(seam_slot(g, SX, bx.x + 1, j, k), X->n);
                    seam_put(X->b, s, e.rf, e.af, e.bf, xc, true);
                    if (i == g.C1) { // face C1 + 1: the ghost position C1 + 1 ahead of it, the old face
                        X->a[7][s] = __int_as_float((int)flm[L::flag(ty - L::CROW0, cx + 1)]);
                        X->a[8][s] = F(2, cx + 1);
                        X->a[9][s] = F(3, cx + 1);
                        X->a[10][s] = F(1, cx + 1);
                        X->a[11][s] = F(0, cx + 1);
                        if (!px) // bounded: the outflow invariant, the values of cell C1 (xcell)
                            seam_put(X->a, s, (T)(5. / 6.), (T)0, (T)0, xc, false);
                    }
                }
            }
            // the warp is done with plane k - 1 (with the stress) or k
            __syncwarp();
            if ((t & 31) == 0) mbar_arrive(empty_of(STRESS ? k - 1 : k));
        }
    }
    if (failed) atomicOr(&S.sc->status, STATUS_STAGING);
    __syncthreads();
    if (t == NT && *abort_flag) // the last NS planes issued hold each stage's newest phase
        for (int p = issued - NS + 1 > pfirst ? issued - NS + 1 : pfirst; p <= issued; ++p)
            mbar_wait(bar_of(p), parity_of(p), kLimitNs);
    __syncthreads();
    if (t == NT) {
        for (int q = 0; q < 2 * NS; ++q) mbar_inval(smem_u32(&bar[q]));
        if ((XS & 1) && NW > 1)
            for (int r = 0; r < SY; ++r)
                for (int h = 0; h < NW - 1; ++h)
                    for (int q = 0; q < NS; ++q) mbar_inval(smem_u32(&xh->bar[r][h][q]));
    }
    if (MODE & (P1_RMAX | P1_RSUM))
        tile_store<T, NT + 32>(S, bx, (MODE & P1_RMAX) != 0, (MODE & P1_RSUM) != 0, m0, m1, m2, rsum);
}

// The stages from the first 128-byte boundary of the dynamic shared memory (tensor copies
// land on 128-byte boundaries; launches ask for 128 bytes more).
__device__ __forceinline__ unsigned char *align128(unsigned char *p) { return p + ((128u - (smem_u32(p) & 127u)) & 127u); }

// The single-grid kernel: maps and boxes as parameters.  XS: the sweeps folded in (1: x1, 3: x1
// and x3; fcur: the face generation read; X: the seam arrays).
template <int MODE, int TSX, int TSY, int XS = 0>
__global__ void __launch_bounds__(TSX *TSY + 32, 2)
    k_phase1_tma(const __grid_constant__ DevState<float> S, const __grid_constant__ TmaArgs A, int src, int dst, int kch,
                 int fcur, const __grid_constant__ XSeams X) {
    using L = TLayout<MODE, TSX, TSY>;
    using H = XHand<TSX, TSY, L::NS>;
    // two blocks per SM with the hand-over slots too
    static_assert(!XS || 2 * (L::SMEM + 128 + 512 + (int)sizeof(H) + 1024) <= 228 * 1024, "shared memory: two blocks per SM");
    extern __shared__ __align__(128) unsigned char sm_raw[];
    __shared__ __align__(8) unsigned long long bar[2 * L::NS + 1];
    __shared__ __align__(8) unsigned char xh_raw[XS ? sizeof(H) : 8];
    auto map = [&](int q) { return &A.map[q]; };
    phase1_tma_body<MODE, TSX, TSY, XS>(S, map, A.m, false, src, dst, kch, bix_here(), align128(sm_raw), bar, fcur, &X,
                                        reinterpret_cast<H *>(xh_raw));
}

// cuTensorMapEncodeTiled through the runtime's entry-point lookup (no link to libcuda)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
inline EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return (EncodeTiledFn)p;
    }();
    return fn;
}

// What n boxes load.
inline void box_meta(BoxMeta &m, const TmaBox *B, int n) {
    std::memset(&m, 0, sizeof m);
    for (int q = 0; q < n; ++q) {
        m.row0[q] = B[q].row0;
        m.dst[q] = B[q].dst;
        m.when[q] = B[q].when;
        for (unsigned kind = DOWN; kind <= TOP; kind <<= 1)
            if (B[q].when & kind) m.bytes[kind] += box_bytes(B[q]);
    }
    m.n = n;
}
// The tensor map of one box.
inline bool encode_box(CUtensorMap *map, const TmaBox &b) {
    const EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t dim[4] = {(cuuint64_t)b.dim[0], (cuuint64_t)b.dim[1], (cuuint64_t)b.dim[2], (cuuint64_t)b.dim[3]};
    const cuuint64_t stride[3] = {(cuuint64_t)b.stride[0], (cuuint64_t)b.stride[1], (cuuint64_t)b.stride[2]};
    const cuuint32_t box[4] = {(cuuint32_t)b.box[0], (cuuint32_t)b.box[1], (cuuint32_t)b.box[2], (cuuint32_t)b.box[3]};
    const cuuint32_t unit[4] = {1, 1, 1, 1};
    return enc(map, b.elem == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 4, const_cast<void *>(b.base),
               dim, stride, box, unit, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
// The tensor maps of n boxes; false when there are none or the encoder refuses one.
inline bool encode_boxes(TmaArgs &A, const TmaBox *B, int n) {
    if (n <= 0 || !encode_tiled()) return false;
    std::memset(&A, 0, sizeof A);
    for (int q = 0; q < n; ++q)
        if (!encode_box(&A.map[q], B[q])) return false;
    box_meta(A.m, B, n);
    return true;
}
// The tensor maps of a launch; false when the arrays do not allow the TMA form.
template <int MODE, int TSX, int TSY> inline bool tma_args(TmaArgs &A, const DevState<float> &S, int src, int fcur) {
    TmaBox B[kMaxBoxes];
    const int n = tma_boxes<MODE, TSX, TSY>(B, S.g, bases_of<MODE>(S, src, fcur));
    return encode_boxes(A, B, n);
}

// TSX x TSY tiles (64 x 4 or 32 x 8); kch: planes per block (0: tile_chunk's choice)
template <int MODE, int TSX = 64, int TSY = 4>
inline void launch_staged_tma(const DevState<float> &S, int src, int dst, int fcur, cudaStream_t st, int kch_in = 0) {
    TmaArgs A;
    if (!tma_args<MODE, TSX, TSY>(A, S, src, fcur)) {
        launch_staged<MODE>(S, src, dst, fcur, st, kch_in);
        return;
    }
    const int kch = kch_in > 0 ? (kch_in < S.g.C3 ? kch_in : S.g.C3) : tile_chunk<TSX, TSY>(S.g);
    k_phase1_tma<MODE, TSX, TSY><<<tile_grid<TSX, TSY>(S.g, kch), dim3(TSX * TSY + 32), TLayout<MODE, TSX, TSY>::SMEM + 128, st>>>(
        S, A, src, dst, kch, fcur, XSeams{});
}
// Phase1 + stress with the x1 sweep (XS = 1) or the x1 and x3 sweeps (XS = 3) folded in (X.tw
// and X.kch set to the tile width and the planes per block); false, launching nothing, when the
// arrays do not allow the TMA form
template <int MODE, int TSX, int TSY, int XS>
inline bool launch_staged_tma_xs(const DevState<float> &S, int src, int dst, int fcur, XSeams &X, cudaStream_t st, int kch_in) {
    TmaArgs A;
    if (!tma_args<MODE, TSX, TSY>(A, S, src, fcur)) return false;
    const int kch = kch_in > 0 ? (kch_in < S.g.C3 ? kch_in : S.g.C3) : tile_chunk<TSX, TSY>(S.g);
    X.tw = TSX;
    X.kch = kch;
    k_phase1_tma<MODE, TSX, TSY, XS>
        <<<tile_grid<TSX, TSY>(S.g, kch), dim3(TSX * TSY + 32), TLayout<MODE, TSX, TSY>::SMEM + 128, st>>>(S, A, src, dst, kch,
                                                                                                      fcur, X);
    return true;
}
// The bounded-wait check: the same launch with every plane expecting `extra` bytes more than its
// boxes bring, so no stage's mbarrier completes and every block gives up (STATUS_STAGING) after
// its bounded waits; no copy is left in flight.  False when the TMA form is not available.
template <int MODE>
inline bool launch_staged_tma_unmet(const DevState<float> &S, int src, int dst, int fcur, unsigned extra, cudaStream_t st) {
    TmaArgs A;
    if (!tma_args<MODE, 64, 4>(A, S, src, fcur)) return false;
    for (unsigned kind = DOWN; kind <= TOP; kind <<= 1) A.m.bytes[kind] += extra;
    const int kch = tile_chunk<64, 4>(S.g);
    k_phase1_tma<MODE, 64, 4><<<tile_grid<64, 4>(S.g, kch), dim3(64 * 4 + 32), TLayout<MODE, 64, 4>::SMEM + 128, st>>>(S, A, src,
                                                                                                           dst, kch, fcur,
                                                                                                           XSeams{});
    return true;
}
template <int MODE, int TSX = 64, int TSY = 4, int XS = 0> inline void prepare_staged_tma() {
    encode_tiled(); // looked up here, outside any stream capture
    constexpr int smem = TLayout<MODE, TSX, TSY>::SMEM + 128;
    cudaFuncSetAttribute(k_phase1_tma<MODE, TSX, TSY, XS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_phase1_tma<MODE, TSX, TSY, XS>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}
#endif

} // namespace stg
