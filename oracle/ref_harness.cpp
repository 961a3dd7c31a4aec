/*
 * Oracle harness around the UNMODIFIED reference solver -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference's source/main.cpp, Arr3d.cpp, Arr2d.cpp and BoundaryConditions.cpp are
 * compiled in place (oracle/Makefile, -Dmain=ark_reference_main) against the single-rank
 * MPI shim in oracle/mpi_shim/mpi.h.  This file replaces only what the reference's own
 * main() does around the solver (main.cpp:53-116, Input() main.cpp:118-278 and
 * InitializeData() main.cpp:280-372): it allocates the reference's global arrays with the
 * reference's dimensions, zero-fills them (the reference leaves them uninitialised,
 * source/Arr3d.cpp:12), loads a caller-supplied initial state, wires the neighbour
 * ranks for a periodic-x/z, wall-y channel, and then calls the reference's own
 * TimeStepSize/Phase1/StressTensor/UseForces/Phase2 in the order of main.cpp:80-91.
 *
 * Periodic x and z: the neighbour globals left/right/bottom/top point at rank 0 itself,
 * so every MPI_Sendrecv along those axes becomes a self-copy (a periodic ghost fill), and
 * coordX = coordZ = -1 so the Neumann edge copies (main.cpp:803-845, 1633-1698) and the
 * inflow/outflow invariants (main.cpp:1731-1745) do not fire.  Walls in y: down/up are
 * MPI_PROC_NULL and condition(i,0,k) = condition(i,n2,k) = 1, as main.cpp:366-371 does.
 *
 * Bulk forcing (not part of the reference; defined identically in the GPU library and in
 * the C restatement): at the start of each step U_b is the mean of u1 over interior cells
 * with condition == 0, summed exactly in 2^-32 fixed point; after TimeStepSize,
 * G = (U_target - U_b) / dt, and after StressTensor every fluid cell gets
 * f1 = f1 + (ro_c * dvc) * G, so each UseForces adds about dt/2 * G to u1.
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <mpi.h>

#include "Arr3d.h"
#include "BoundaryConditions.h"

/* ---- the reference's globals (defined in main.cpp through its headers) ---- */
extern int l, n1, n2, n3, nStop, nPrint, nStep, n1_g, n2_g, n3_g;
extern double x1_e, x1_w, x2_n, x2_s, x3_t, x3_b;
extern double dx1, dx2, dx3;
extern double *x1, *x2, *x3;
extern Arr3d *roCon, *u1Con, *u2Con, *u3Con, *tCon;
extern Arr3d *ronCon, *u1nCon, *u2nCon, *u3nCon, *tnCon;
extern Arr3d *p1, *ro1, *u11, *u21, *u31, *t1;
extern Arr3d *p2, *ro2, *u12, *u22, *u32, *t2;
extern Arr3d *p3, *ro3, *u13, *u23, *u33, *t3;
extern double *rBuf, *qBuf, *tfBuf, *tbBuf, *u2fBuf, *u2bBuf, *u3fBuf, *u3bBuf;
extern Arr3d *condition;
extern Arr3d *averageU1, *averageU2, *averageU3;
extern Arr3d *f1, *f2, *f3;
extern Arr3d *sigm11, *sigm21, *sigm31, *sigm12, *sigm22, *sigm32, *sigm13, *sigm23, *sigm33;
extern double sound, ro0_g, dt, VIS, u10, u20, u30, t0, TIME, CFL;
extern bool x1Period, x2Period, x3Period, needSwap, useTecplot;
extern int left, right, up, down, top, bottom, nproc, rank, px, py, pz, coordX, coordY, coordZ;
extern int coords[3], dims[3];
extern MPI_Comm newComm;
extern const char *dirPath;
/* the reference's output and statistics functions (main.cpp:2577-2891) */
void WriteDataParaView();
void WriteAverageValues(double time);
void WriteEnergy();
void AverageValues();


/* ---- the reference's solver functions (main.cpp:12-21) ---- */
void Input();
void InitializeData();
void TimeStepSize();
void Phase1();
void Phase2();
void StressTensor();
void UseForces();

namespace {

Arr3d *make_zero(int a, int b, int c) {
    Arr3d *arr = new Arr3d(a, b, c);
    std::memset(arr->ref(), 0, sizeof(double) * (size_t)a * b * c);
    return arr;
}

double *make_zero_vec(int n) {
    double *v = new double[n];
    std::memset(v, 0, sizeof(double) * (size_t)n);
    return v;
}

bool g_ready = false;
double g_utarget = 1.0;
int g_forcing = 1;
double g_last_ub = 0.0, g_last_g = 0.0;

/* Named access to every array the harness exposes; cell arrays are
 * (n1+1)(n2+1)(n3+1), face and stress arrays (n1+2)(n2+2)(n3+2). */
struct Named { const char *name; Arr3d **arr; int face; };
const Named kArrays[] = {
    {"roCon", &roCon, 0},   {"u1Con", &u1Con, 0},   {"u2Con", &u2Con, 0},
    {"u3Con", &u3Con, 0},   {"tCon", &tCon, 0},     {"ronCon", &ronCon, 0},
    {"u1nCon", &u1nCon, 0}, {"u2nCon", &u2nCon, 0}, {"u3nCon", &u3nCon, 0},
    {"tnCon", &tnCon, 0},   {"f1", &f1, 0},         {"f2", &f2, 0},
    {"f3", &f3, 0},         {"condition", &condition, 0},
    {"p1", &p1, 1},   {"ro1", &ro1, 1}, {"u11", &u11, 1}, {"u21", &u21, 1}, {"u31", &u31, 1}, {"t1", &t1, 1},
    {"p2", &p2, 1},   {"ro2", &ro2, 1}, {"u12", &u12, 1}, {"u22", &u22, 1}, {"u32", &u32, 1}, {"t2", &t2, 1},
    {"p3", &p3, 1},   {"ro3", &ro3, 1}, {"u13", &u13, 1}, {"u23", &u23, 1}, {"u33", &u33, 1}, {"t3", &t3, 1},
    {"sigm11", &sigm11, 1}, {"sigm21", &sigm21, 1}, {"sigm31", &sigm31, 1},
    {"sigm12", &sigm12, 1}, {"sigm22", &sigm22, 1}, {"sigm32", &sigm32, 1},
    {"sigm13", &sigm13, 1}, {"sigm23", &sigm23, 1}, {"sigm33", &sigm33, 1},
};

const Named *find(const char *name) {
    for (const Named &a : kArrays)
        if (std::strcmp(a.name, name) == 0) return &a;
    return nullptr;
}

size_t count_of(const Named *a) {
    return a->face ? (size_t)(n1 + 2) * (n2 + 2) * (n3 + 2) : (size_t)(n1 + 1) * (n2 + 1) * (n3 + 1);
}

/* Mean of u1nCon over interior cells with condition == 0, exact in 2^-32 fixed point. */
double bulk_velocity() {
    long long s = 0, nf = 0;
    for (int k = 1; k < n3; ++k)
        for (int j = 1; j < n2; ++j)
            for (int i = 1; i < n1; ++i) {
                if (condition->elem(i, j, k) != 0) continue;
                double u = u1nCon->elem(i, j, k);
                if (u != u) u = 0.0;
                if (u > 1073741824.0) u = 1073741824.0;
                if (u < -1073741824.0) u = -1073741824.0;
                s += llrint(u * 4294967296.0);
                ++nf;
            }
    if (nf == 0) return 0.0;
    return ((double)s * (1.0 / 4294967296.0)) / (double)nf;
}

void add_bulk_force(double G) {
    const double dvc = dx1 * dx2 * dx3;
    for (int i = 1; i < n1; ++i)
        for (int j = 1; j < n2; ++j)
            for (int k = 1; k < n3; ++k)
                if (condition->elem(i, j, k) == 0)
                    f1->elem(i, j, k) = f1->elem(i, j, k) + (roCon->elem(i, j, k) * dvc) * G;
}

}  // namespace

extern "C" {

/* Allocate the reference's arrays for a C1 x C2 x C3-cell box (node counts n = C + 1,
 * main.cpp:147-151) and set the scalar parameters.  periodic_x/z select self-neighbours
 * on those axes; y is always bounded by walls. */
int ref_setup(int C1, int C2, int C3, double Lx, double Ly, double Lz, double nu, double c,
              double rho0, double cfl, double temp0, int periodic_x, int periodic_z) {
    if (g_ready) return 1;
    n1_g = C1 + 1; n2_g = C2 + 1; n3_g = C3 + 1;
    dims[0] = dims[1] = dims[2] = 1;
    px = py = pz = 1;
    coords[0] = coords[1] = coords[2] = 0;
    coordX = -1; coordY = 0; coordZ = -1;
    nproc = 1; rank = 0; newComm = 0;
    left = right = periodic_x ? 0 : MPI_PROC_NULL;
    down = up = MPI_PROC_NULL;
    bottom = top = periodic_z ? 0 : MPI_PROC_NULL;
    if (!periodic_x) coordX = 0; /* non-periodic x: the reference's own edge handling */
    if (!periodic_z) coordZ = 0;
    x1Period = periodic_x != 0; x2Period = false; x3Period = periodic_z != 0;
    needSwap = true; useTecplot = false; l = 1;

    n1 = n1_g; n2 = n2_g; n3 = n3_g;
    x1_w = 0.; x1_e = Lx; x2_s = -0.5 * Ly; x2_n = 0.5 * Ly; x3_b = 0.; x3_t = Lz;
    CFL = cfl; VIS = nu; t0 = temp0; sound = c; ro0_g = rho0;
    u10 = u20 = u30 = 0.;
    nStep = 0; TIME = 0.; dt = 0.;
    dx1 = (x1_e - x1_w) / (n1_g - 1);
    dx2 = (x2_n - x2_s) / (n2_g - 1);
    dx3 = (x3_t - x3_b) / (n3_g - 1);

    x1 = make_zero_vec(n1 + 2); x2 = make_zero_vec(n2 + 2); x3 = make_zero_vec(n3 + 2);
    const int a = n1 + 1, b = n2 + 1, cc = n3 + 1;
    roCon = make_zero(a, b, cc); tCon = make_zero(a, b, cc);
    u1Con = make_zero(a, b, cc); u2Con = make_zero(a, b, cc); u3Con = make_zero(a, b, cc);
    ronCon = make_zero(a, b, cc); tnCon = make_zero(a, b, cc);
    u1nCon = make_zero(a, b, cc); u2nCon = make_zero(a, b, cc); u3nCon = make_zero(a, b, cc);
    f1 = make_zero(a, b, cc); f2 = make_zero(a, b, cc); f3 = make_zero(a, b, cc);
    condition = make_zero(a, b, cc);
    averageU1 = make_zero(a, b + 1, cc); averageU2 = make_zero(a, b + 1, cc);
    averageU3 = make_zero(a, b + 1, cc);
    const int fa = n1 + 2, fb = n2 + 2, fc = n3 + 2;
    Arr3d **faces[] = {&ro1, &t1, &u11, &u21, &u31, &p1, &ro2, &t2, &u12, &u22, &u32, &p2,
                       &ro3, &t3, &u13, &u23, &u33, &p3, &sigm11, &sigm21, &sigm31,
                       &sigm12, &sigm22, &sigm32, &sigm13, &sigm23, &sigm33};
    for (Arr3d **f : faces) *f = make_zero(fa, fb, fc);
    int nmax = n1 > n2 ? n1 : n2;
    nmax = nmax > n3 ? nmax : n3;
    rBuf = make_zero_vec(nmax + 2); qBuf = make_zero_vec(nmax + 1);
    tfBuf = make_zero_vec(nmax + 2); tbBuf = make_zero_vec(nmax + 2);
    u2fBuf = make_zero_vec(nmax + 2); u2bBuf = make_zero_vec(nmax + 2);
    u3fBuf = make_zero_vec(nmax + 2); u3bBuf = make_zero_vec(nmax + 2);

    /* walls: solid ghost rows in y (main.cpp:366-371) */
    for (int i = 0; i < n1 + 1; ++i)
        for (int k = 0; k < n3 + 1; ++k) {
            condition->elem(i, 0, k) = 1;
            condition->elem(i, n2, k) = 1;
        }
    g_ready = true;
    return 0;
}

/* Free everything ref_setup allocated so the next ref_setup can pick a new size. */
int ref_teardown() {
    if (!g_ready) return 0;
    for (const Named &a : kArrays) { delete *a.arr; *a.arr = nullptr; }
    delete averageU1; delete averageU2; delete averageU3;
    delete[] x1; delete[] x2; delete[] x3;
    delete[] rBuf; delete[] qBuf; delete[] tfBuf; delete[] tbBuf;
    delete[] u2fBuf; delete[] u2bBuf; delete[] u3fBuf; delete[] u3bBuf;
    g_ready = false;
    return 0;
}

/* The reference's own stock case: Input() (main.cpp:118-278: 200x60x1 cells, backward-facing
 * step, VIS 1e-3, c 10, CFL 0.2) and InitializeData() (main.cpp:280-372), on one rank with
 * every neighbour MPI_PROC_NULL and coords 0 (bounded x, y and z).  The arrays Input()
 * allocates are zero-filled before InitializeData() (the reference leaves them
 * uninitialised), and the "Con" level starts equal to "nCon" (TimeStepSize reads it before
 * any Phase1 has written it). */
int ref_stock_setup() {
    if (g_ready) return 1;
    dims[0] = dims[1] = dims[2] = 1;
    coords[0] = coords[1] = coords[2] = 0;
    nproc = 1; rank = 0; newComm = 0;
    left = right = down = up = bottom = top = MPI_PROC_NULL;
    Input();
    g_ready = true;
    for (const Named &a : kArrays) std::memset((*a.arr)->ref(), 0, sizeof(double) * count_of(&a));
    InitializeData();
    const size_t nc = (size_t)(n1 + 1) * (n2 + 1) * (n3 + 1);
    std::memcpy(roCon->ref(), ronCon->ref(), sizeof(double) * nc);
    std::memcpy(u1Con->ref(), u1nCon->ref(), sizeof(double) * nc);
    std::memcpy(u2Con->ref(), u2nCon->ref(), sizeof(double) * nc);
    std::memcpy(u3Con->ref(), u3nCon->ref(), sizeof(double) * nc);
    std::memcpy(tCon->ref(), tnCon->ref(), sizeof(double) * nc);
    g_forcing = 0;
    return 0;
}

/* Grid and parameters after ref_stock_setup: cells C1..C3, then dx1..dx3, VIS, sound, ro0_g, CFL. */
int ref_stock_params(int *cells, double *vals) {
    if (!g_ready) return 1;
    cells[0] = n1 - 1; cells[1] = n2 - 1; cells[2] = n3 - 1;
    vals[0] = dx1; vals[1] = dx2; vals[2] = dx3; vals[3] = VIS; vals[4] = sound; vals[5] = ro0_g; vals[6] = CFL;
    vals[7] = x1_e - x1_w; vals[8] = x2_n - x2_s; vals[9] = x3_t - x3_b;
    return 0;
}

int ref_set_forcing(int on, double u_target) {
    g_forcing = on;
    g_utarget = u_target;
    return 0;
}

size_t ref_array_len(const char *name) {
    const Named *a = find(name);
    return a && g_ready ? count_of(a) : 0;
}

int ref_put(const char *name, const double *src) {
    const Named *a = find(name);
    if (!a || !g_ready) return 1;
    std::memcpy((*a->arr)->ref(), src, sizeof(double) * count_of(a));
    return 0;
}

int ref_get(const char *name, double *dst) {
    const Named *a = find(name);
    if (!a || !g_ready) return 1;
    std::memcpy(dst, (*a->arr)->ref(), sizeof(double) * count_of(a));
    return 0;
}

/* Single calls of the reference's own functions (per-phase parity). */
void ref_time_step_size() { TimeStepSize(); }
void ref_phase1() { Phase1(); }
void ref_stress_tensor() { StressTensor(); }
void ref_use_forces() { UseForces(); }
void ref_phase2() { Phase2(); }
void ref_set_dt(double v) { dt = v; }
double ref_get_dt() { return dt; }
double ref_get_time() { return TIME; }
int ref_get_nstep() { return nStep; }
double ref_last_ub() { return g_last_ub; }
double ref_last_g() { return g_last_g; }

/* The reference's BoundaryConditions class (source/BoundaryConditions.cpp:7-83), constructed
 * on the "nCon" level (u1nCon, u2nCon, u3nCon, ronCon, tnCon) with the node counts n1, n2, n3
 * and the given periodicity and t0, then alongX1/2/3 for axis 1/2/3. */
int ref_boundary_conditions(int axis, int x1_period, int x2_period, int x3_period, double t0_bc) {
    if (!g_ready || axis < 1 || axis > 3) return 1;
    BoundaryConditions bc(u1nCon, u2nCon, u3nCon, ronCon, tnCon, x1_period != 0, x2_period != 0, x3_period != 0,
                          n1, n2, n3, t0_bc);
    if (axis == 1) bc.alongX1();
    else if (axis == 2) bc.alongX2();
    else bc.alongX3();
    return 0;
}

/* nsteps full time steps in the order of main.cpp:80-91, plus the bulk forcing. */
int ref_run(int nsteps) {
    if (!g_ready) return 1;
    for (int s = 0; s < nsteps; ++s) {
        double ub = g_forcing ? bulk_velocity() : 0.0;
        TimeStepSize();
        nStep++;
        TIME += 0.5 * dt;
        Phase1();
        StressTensor();
        if (g_forcing) {
            double G = (g_utarget - ub) / dt;
            add_bulk_force(G);
            g_last_ub = ub;
            g_last_g = G;
        }
        UseForces();
        Phase2();
        Phase1();
        UseForces();
        TIME += 0.5 * dt;
    }
    return 0;
}

/* ---- output and statistics (the golden files of the writers) ----
 * The reference writes as rank 0 of its decomposition, with coordX = coordZ = 0 in the row
 * offsets of main.cpp:2670-2671; the harness keeps them at -1 on periodic axes only to keep
 * the bounded-edge code of the step from firing, so they are 0 while a writer runs. */
static std::string g_dir;

struct WriterCoords {
    int cx, cz;
    WriterCoords() : cx(coordX), cz(coordZ) { coordX = 0; coordZ = 0; }
    ~WriterCoords() { coordX = cx; coordZ = cz; }
};

/* WriteDataParaView (main.cpp:2577-2745): dir/out_<nStep>.vtk; dir ends in '/'. */
int ref_write_paraview(const char *dir) {
    if (!g_ready || !dir) return 1;
    g_dir = dir;
    dirPath = g_dir.c_str();
    WriterCoords wc;
    WriteDataParaView();
    return 0;
}

/* AverageValues (main.cpp:2878-2891): averageU += u?nCon * dt. */
int ref_average_values() {
    if (!g_ready) return 1;
    AverageValues();
    return 0;
}

/* WriteAverageValues(start_time) (main.cpp:2747-2849): dir/average.vtk. */
int ref_write_average(const char *dir, double start_time) {
    if (!g_ready || !dir) return 1;
    g_dir = dir;
    dirPath = g_dir.c_str();
    WriterCoords wc;
    WriteAverageValues(start_time);
    return 0;
}

/* WriteEnergy (main.cpp:2851-2876): appends "(TIME; energy) " to dir/energy.txt. */
int ref_write_energy(const char *dir) {
    if (!g_ready || !dir) return 1;
    g_dir = dir;
    dirPath = g_dir.c_str();
    WriteEnergy();
    return 0;
}

/* averageU1..3 (layout (n1+1) x (n2+2) x (n3+1), main.cpp:225-227). */
size_t ref_average_len() { return g_ready ? (size_t)(n1 + 1) * (n2 + 2) * (n3 + 1) : 0; }
int ref_get_average(int m, double *out) {
    if (!g_ready || m < 1 || m > 3 || !out) return 1;
    Arr3d *a = m == 1 ? averageU1 : m == 2 ? averageU2 : averageU3;
    std::memcpy(out, a->ref(), sizeof(double) * ref_average_len());
    return 0;
}

}  // extern "C"
