/*
 * CPU restatement of the reference CABARET time step -- TEST INFRASTRUCTURE ONLY.
 * See ark_oracle.h.  Build: oracle/Makefile (`make -C oracle port`), always with
 * -ffp-contract=off so every a*b+c rounds twice, exactly as the reference does on x86.
 *
 * Every arithmetic expression keeps the reference's operand order (C evaluates
 * left to right), because the parity bar for the FP64 path is bit-for-bit.  The three
 * Phase2 sweeps (main.cpp:1726-2011, 2023-2255, 2261-2494) are written once, for a
 * generic axis, with the per-axis differences of the reference kept as parameters:
 *   - the Q-limiter source term of the x1 and x3 sweeps uses (r_cn - r_c)
 *     (main.cpp:1804, 2321); the x2 sweep uses (q_cn - q_c) (main.cpp:2083);
 *   - in the x2 sweep's wall branches that take the cell value, the tangential u1 is
 *     read from u2nCon (main.cpp:2219, 2238); x1 and x3 read the matching component.
 *
 * OpenMP parallelises over independent lines and cells only; the two reductions are
 * order independent (a MIN, and an integer sum), so results do not depend on the
 * thread count.
 */
#include "ark_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct ark_oracle {
    int C[3];     /* cells per axis */
    int n[3];     /* reference node counts n = C + 1 (main.cpp:147-151) */
    double dx[3];
    double nu, sound, rho0, cfl;
    int periodic_x, periodic_z;
    double dt, time;
    int nstep;
    int forcing;
    double u_target, last_ub, last_g;
    size_t ncell, nface;
    size_t cs[3], fs[3]; /* strides of cell and face arrays */
    /* cells: time level "Con" and "nCon" */
    double *ro, *u[3], *ron, *un[3];
    double *f[3], *cond;
    /* faces normal to axis d: pressure, density, velocity components */
    double *p[3], *rof[3], *uf[3][3];
    /* viscous stress sigma_{m d}: component m on faces normal to d */
    double *sig[3][3];
};

static double min3d(double x1, double x2, double x3) {
    /* ternary form of main.cpp:2963-2967 (a NaN argument is skipped, not propagated) */
    x1 = x1 > x2 ? x2 : x1;
    x1 = x1 > x3 ? x3 : x1;
    return x1;
}

static double max3d(double x1, double x2, double x3) {
    /* main.cpp:2969-2973 */
    x1 = x1 < x2 ? x2 : x1;
    x1 = x1 < x3 ? x3 : x1;
    return x1;
}

static inline size_t cidx(const ark_oracle *o, int i, int j, int k) {
    return ((size_t)k * (size_t)(o->n[1] + 1) + (size_t)j) * (size_t)(o->n[0] + 1) + (size_t)i;
}

static inline size_t fidx(const ark_oracle *o, int i, int j, int k) {
    return ((size_t)k * (size_t)(o->n[1] + 2) + (size_t)j) * (size_t)(o->n[0] + 2) + (size_t)i;
}

static double *zalloc(size_t n) { return (double *)calloc(n, sizeof(double)); }

void aor_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

ark_oracle *aor_create(int C1, int C2, int C3, double Lx, double Ly, double Lz, double nu,
                       double sound, double rho0, double cfl, int periodic_x, int periodic_z) {
    if (C1 < 1 || C2 < 1 || C3 < 1) return NULL;
    ark_oracle *o = (ark_oracle *)calloc(1, sizeof(ark_oracle));
    o->C[0] = C1; o->C[1] = C2; o->C[2] = C3;
    for (int d = 0; d < 3; ++d) o->n[d] = o->C[d] + 1;
    /* grid steps as InitializeData computes them (main.cpp:284-290):
     * (east - west) / (n_g - 1) with the domain [0,Lx] x [-Ly/2,Ly/2] x [0,Lz] */
    o->dx[0] = (Lx - 0.) / (double)(o->n[0] - 1);
    o->dx[1] = (0.5 * Ly - -0.5 * Ly) / (double)(o->n[1] - 1);
    o->dx[2] = (Lz - 0.) / (double)(o->n[2] - 1);
    o->nu = nu; o->sound = sound; o->rho0 = rho0; o->cfl = cfl;
    o->periodic_x = periodic_x; o->periodic_z = periodic_z;
    o->forcing = 1; o->u_target = 1.0;
    o->ncell = (size_t)(o->n[0] + 1) * (o->n[1] + 1) * (o->n[2] + 1);
    o->nface = (size_t)(o->n[0] + 2) * (o->n[1] + 2) * (o->n[2] + 2);
    o->cs[0] = 1; o->cs[1] = (size_t)(o->n[0] + 1); o->cs[2] = o->cs[1] * (size_t)(o->n[1] + 1);
    o->fs[0] = 1; o->fs[1] = (size_t)(o->n[0] + 2); o->fs[2] = o->fs[1] * (size_t)(o->n[1] + 2);
    o->ro = zalloc(o->ncell); o->ron = zalloc(o->ncell); o->cond = zalloc(o->ncell);
    for (int m = 0; m < 3; ++m) {
        o->u[m] = zalloc(o->ncell); o->un[m] = zalloc(o->ncell); o->f[m] = zalloc(o->ncell);
    }
    for (int d = 0; d < 3; ++d) {
        o->p[d] = zalloc(o->nface); o->rof[d] = zalloc(o->nface);
        for (int m = 0; m < 3; ++m) { o->uf[d][m] = zalloc(o->nface); o->sig[d][m] = zalloc(o->nface); }
    }
    /* solid ghost rows in y, as main.cpp:366-371 marks them */
    for (int k = 0; k <= o->n[2]; ++k)
        for (int i = 0; i <= o->n[0]; ++i) {
            o->cond[cidx(o, i, 0, k)] = 1.0;
            o->cond[cidx(o, i, o->n[1], k)] = 1.0;
        }
    return o;
}

void aor_destroy(ark_oracle *o) {
    if (!o) return;
    free(o->ro); free(o->ron); free(o->cond);
    for (int m = 0; m < 3; ++m) { free(o->u[m]); free(o->un[m]); free(o->f[m]); }
    for (int d = 0; d < 3; ++d) {
        free(o->p[d]); free(o->rof[d]);
        for (int m = 0; m < 3; ++m) { free(o->uf[d][m]); free(o->sig[d][m]); }
    }
    free(o);
}

/* ---- named access ------------------------------------------------------------ */

static double *lookup(const ark_oracle *o, const char *name, size_t *len) {
    static const char *const cellnames[] = {"roCon", "u1Con", "u2Con", "u3Con", "ronCon", "u1nCon",
                                            "u2nCon", "u3nCon", "f1", "f2", "f3", "condition"};
    double *const cellptr[] = {o->ro, o->u[0], o->u[1], o->u[2], o->ron, o->un[0],
                               o->un[1], o->un[2], o->f[0], o->f[1], o->f[2], o->cond};
    for (int a = 0; a < 12; ++a)
        if (strcmp(name, cellnames[a]) == 0) { *len = o->ncell; return cellptr[a]; }
    /* faces: p{d}, ro{d}, u{m}{d}, sigm{m}{d} with d, m in 1..3 */
    *len = o->nface;
    size_t L = strlen(name);
    if (L == 2 && name[0] == 'p' && name[1] >= '1' && name[1] <= '3') return o->p[name[1] - '1'];
    if (L == 3 && name[0] == 'r' && name[1] == 'o' && name[2] >= '1' && name[2] <= '3')
        return o->rof[name[2] - '1'];
    if (L == 3 && name[0] == 'u' && name[1] >= '1' && name[1] <= '3' && name[2] >= '1' && name[2] <= '3')
        return o->uf[name[2] - '1'][name[1] - '1'];
    if (L == 6 && strncmp(name, "sigm", 4) == 0 && name[4] >= '1' && name[4] <= '3' &&
        name[5] >= '1' && name[5] <= '3')
        return o->sig[name[5] - '1'][name[4] - '1'];
    *len = 0;
    return NULL;
}

size_t aor_len(const ark_oracle *o, const char *name) {
    size_t len = 0;
    return lookup(o, name, &len) ? len : 0;
}

int aor_put(ark_oracle *o, const char *name, const double *src) {
    size_t len = 0;
    double *a = lookup(o, name, &len);
    if (!a) return 1;
    memcpy(a, src, len * sizeof(double));
    return 0;
}

int aor_get(const ark_oracle *o, const char *name, double *dst) {
    size_t len = 0;
    double *a = lookup(o, name, &len);
    if (!a) return 1;
    memcpy(dst, a, len * sizeof(double));
    return 0;
}

void aor_set_forcing(ark_oracle *o, int on, double u_target) { o->forcing = on; o->u_target = u_target; }
void aor_set_dt(ark_oracle *o, double dt) { o->dt = dt; }
double aor_dt(const ark_oracle *o) { return o->dt; }
double aor_time(const ark_oracle *o) { return o->time; }
int aor_nstep(const ark_oracle *o) { return o->nstep; }
double aor_last_ub(const ark_oracle *o) { return o->last_ub; }
double aor_last_g(const ark_oracle *o) { return o->last_g; }

/* ---- ghost cells: the halo exchange of a single rank ---------------------------
 * With one rank, the reference's MPI_Sendrecv pairs (main.cpp:603-801, 1049-1631)
 * reduce to: on a periodic axis, ghost 0 <- cell C and ghost C+1 <- cell 1 (faces:
 * halo 0 <- face C, halo C+2 <- face 2), over the interior of the other two axes;
 * on a bounded axis nothing is received.  Bounded x and z then get the zero-gradient
 * copies of main.cpp:803-845 (stress) and main.cpp:1633-1698 (Phase2). */

static void wrap_cells(const ark_oracle *o, double *a, int axis) {
    const int *n = o->n;
    if (axis == 0) {
        for (int k = 1; k < n[2]; ++k)
            for (int j = 1; j < n[1]; ++j) {
                a[cidx(o, 0, j, k)] = a[cidx(o, n[0] - 1, j, k)];
                a[cidx(o, n[0], j, k)] = a[cidx(o, 1, j, k)];
            }
    } else {
        for (int j = 1; j < n[1]; ++j)
            for (int i = 1; i < n[0]; ++i) {
                a[cidx(o, i, j, 0)] = a[cidx(o, i, j, n[2] - 1)];
                a[cidx(o, i, j, n[2])] = a[cidx(o, i, j, 1)];
            }
    }
}

static void wrap_faces(const ark_oracle *o, double *a, int axis) {
    const int *n = o->n;
    if (axis == 0) {
        for (int k = 1; k < n[2]; ++k)
            for (int j = 1; j < n[1]; ++j) {
                a[fidx(o, 0, j, k)] = a[fidx(o, n[0] - 1, j, k)];
                a[fidx(o, n[0] + 1, j, k)] = a[fidx(o, 2, j, k)];
            }
    } else {
        for (int j = 1; j < n[1]; ++j)
            for (int i = 1; i < n[0]; ++i) {
                a[fidx(o, i, j, 0)] = a[fidx(o, i, j, n[2] - 1)];
                a[fidx(o, i, j, n[2] + 1)] = a[fidx(o, i, j, 2)];
            }
    }
}

static void neumann_cells(const ark_oracle *o, double *a, int axis) {
    const int *n = o->n;
    if (axis == 0) {
        for (int k = 1; k < n[2]; ++k)
            for (int j = 1; j < n[1]; ++j) {
                a[cidx(o, n[0], j, k)] = a[cidx(o, n[0] - 1, j, k)];
                a[cidx(o, 0, j, k)] = a[cidx(o, 1, j, k)];
            }
    } else {
        for (int j = 1; j < n[1]; ++j)
            for (int i = 1; i < n[0]; ++i) {
                a[cidx(o, i, j, 0)] = a[cidx(o, i, j, 1)];
                a[cidx(o, i, j, n[2])] = a[cidx(o, i, j, n[2] - 1)];
            }
    }
}

static void neumann_faces_z(const ark_oracle *o, double *a) {
    const int *n = o->n;
    for (int j = 1; j < n[1]; ++j)
        for (int i = 1; i < n[0]; ++i) {
            a[fidx(o, i, j, 0)] = a[fidx(o, i, j, 1)];
            a[fidx(o, i, j, n[2] + 1)] = a[fidx(o, i, j, n[2])];
        }
}

/* ---- TimeStepSize (main.cpp:374-415) ------------------------------------------- */

void aor_time_step_size(ark_oracle *o) {
    const int *n = o->n;
    const double CFL = o->cfl, VIS = o->nu, sound = o->sound;
    const double dx1 = o->dx[0], dx2 = o->dx[1], dx3 = o->dx[2];
    double dt = 1e8; /* pow(10, 8) */
#pragma omp parallel
    {
        double mine = 1e8;
#pragma omp for collapse(2) schedule(static)
        for (int i = 1; i < n[0]; ++i)
            for (int j = 1; j < n[1]; ++j)
                for (int k = 1; k < n[2]; ++k) {
                    size_t c = cidx(o, i, j, k);
                    double dtu1 = CFL * dx1 / (sound + fabs(o->u[0][c]));
                    double dtu2 = CFL * dx2 / (sound + fabs(o->u[1][c]));
                    double dtu3 = CFL * dx3 / (sound + fabs(o->u[2][c]));
                    double dtu = min3d(dtu1, dtu2, dtu3);
                    double dtv;
                    if (VIS > 1e-16) {
                        double dtv1 = CFL * dx1 * dx1 / (2. * VIS);
                        double dtv2 = CFL * dx2 * dx2 / (2. * VIS);
                        double dtv3 = CFL * dx3 * dx3 / (2. * VIS);
                        dtv = min3d(dtv1, dtv2, dtv3);
                    } else {
                        dtv = 1e16;
                    }
                    mine = min3d(mine, dtu, dtv);
                }
#pragma omp critical
        dt = dt > mine ? mine : dt;
    }
    o->dt = dt;
}

/* ---- Phase1 (main.cpp:417-575), without the temperature line ------------------- */

void aor_phase1(ark_oracle *o) {
    const int *n = o->n;
    const size_t nc = o->ncell;
    (void)nc;
    /* Con <- nCon on interior cells (main.cpp:419-432) */
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k < n[2]; ++k)
        for (int j = 1; j < n[1]; ++j)
            for (int i = 1; i < n[0]; ++i) {
                size_t c = cidx(o, i, j, k);
                o->ro[c] = o->ron[c];
                for (int m = 0; m < 3; ++m) o->u[m][c] = o->un[m][c];
            }
    const double dx1 = o->dx[0], dx2 = o->dx[1], dx3 = o->dx[2];
    const double ds1 = dx2 * dx3, ds2 = dx1 * dx3, ds3 = dx1 * dx2;
    const double dvc = dx1 * dx2 * dx3;
    const double dt = o->dt, ro0 = o->rho0;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k < n[2]; ++k)
        for (int j = 1; j < n[1]; ++j)
            for (int i = 1; i < n[0]; ++i) {
                size_t c = cidx(o, i, j, k);
                double ro_cn, u_cn[3];
                if (o->cond[c] < 0.5) {
                    /* the six faces: west/east (d=0), south/north (d=1), bottom/top (d=2) */
                    size_t lo[3] = {fidx(o, i, j, k), fidx(o, i, j, k), fidx(o, i, j, k)};
                    size_t hi[3] = {fidx(o, i + 1, j, k), fidx(o, i, j + 1, k), fidx(o, i, j, k + 1)};
                    double rl[3], rh[3], pl[3], ph[3], ul[3][3], uh[3][3];
                    for (int d = 0; d < 3; ++d) {
                        rl[d] = o->rof[d][lo[d]]; rh[d] = o->rof[d][hi[d]];
                        pl[d] = o->p[d][lo[d]];   ph[d] = o->p[d][hi[d]];
                        for (int m = 0; m < 3; ++m) { ul[d][m] = o->uf[d][m][lo[d]]; uh[d][m] = o->uf[d][m][hi[d]]; }
                    }
                    const double ds[3] = {ds1, ds2, ds3};
                    const double ro_c = o->ro[c];
                    /* new density (main.cpp:530-533) */
                    ro_cn = (ro_c * dvc - 0.5 * dt * (
                                 (rh[0] * uh[0][0] - rl[0] * ul[0][0]) * ds[0] +
                                 (rh[1] * uh[1][1] - rl[1] * ul[1][1]) * ds[1] +
                                 (rh[2] * uh[2][2] - rl[2] * ul[2][2]) * ds[2])) / dvc;
                    /* momentum component m (main.cpp:536-551): flux through faces normal
                     * to d is (ro * u_m) * u_d, plus p when m == d */
                    for (int m = 0; m < 3; ++m) {
                        double fl[3];
                        for (int d = 0; d < 3; ++d) {
                            if (m == d)
                                fl[d] = (rh[d] * uh[d][m] * uh[d][d] + ph[d]) - (rl[d] * ul[d][m] * ul[d][d] + pl[d]);
                            else
                                fl[d] = rh[d] * uh[d][m] * uh[d][d] - rl[d] * ul[d][m] * ul[d][d];
                        }
                        u_cn[m] = (ro_c * o->u[m][c] * dvc - 0.5 * dt * (
                                       fl[0] * ds[0] + fl[1] * ds[1] + fl[2] * ds[2])) / (ro_cn * dvc);
                    }
                } else {
                    u_cn[0] = u_cn[1] = u_cn[2] = 0.;
                    ro_cn = ro0;
                }
                for (int m = 0; m < 3; ++m) o->un[m][c] = u_cn[m];
                o->ron[c] = ro_cn;
            }
}

/* ---- StressTensor (main.cpp:577-1024) ------------------------------------------ */

void aor_stress_tensor(ark_oracle *o) {
    const int *n = o->n;
    for (int d = 0; d < 3; ++d)
        for (int m = 0; m < 3; ++m) memset(o->sig[d][m], 0, o->nface * sizeof(double));
    /* halo of u1Con, u2Con, u3Con (main.cpp:603-801) and bounded-edge copies (main.cpp:803-845) */
    for (int m = 0; m < 3; ++m) {
        if (o->periodic_x) wrap_cells(o, o->u[m], 0); else neumann_cells(o, o->u[m], 0);
        if (o->periodic_z) wrap_cells(o, o->u[m], 2); else neumann_cells(o, o->u[m], 2);
    }
    const double VIS = o->nu;
    /* faces normal to axis d, face index 1..n[d] along d, interior across (main.cpp:856-982) */
    for (int d = 0; d < 3; ++d) {
        const double dxd = o->dx[d];
        const int hi0 = d == 0 ? n[0] : n[0] - 1;
        const int hi1 = d == 1 ? n[1] : n[1] - 1;
        const int hi2 = d == 2 ? n[2] : n[2] - 1;
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = 1; k <= hi2; ++k)
            for (int j = 1; j <= hi1; ++j)
                for (int i = 1; i <= hi0; ++i) {
                    size_t c = cidx(o, i, j, k);
                    size_t cw = c - o->cs[d];
                    double cond_c = o->cond[c], cond_cw = o->cond[cw];
                    double v[3];
                    for (int m = 0; m < 3; ++m) {
                        double u_c = o->u[m][c], u_cw = o->u[m][cw];
                        if (cond_cw < 0.5 && cond_c < 0.5) v[m] = VIS * (u_c - u_cw) / dxd;
                        else if (cond_cw < 0.5 && cond_c > 0.5) v[m] = 2 * VIS * (-u_cw) / dxd;
                        else if (cond_cw > 0.5 && cond_c < 0.5) v[m] = 2 * VIS * u_c / dxd;
                        else v[m] = 0.;
                    }
                    size_t fc = fidx(o, i, j, k);
                    for (int m = 0; m < 3; ++m) o->sig[d][m][fc] = v[m];
                }
    }
    /* friction force (main.cpp:995-1023) */
    const double ds1 = o->dx[1] * o->dx[2], ds2 = o->dx[0] * o->dx[2], ds3 = o->dx[0] * o->dx[1];
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k < n[2]; ++k)
        for (int j = 1; j < n[1]; ++j)
            for (int i = 1; i < n[0]; ++i) {
                size_t c = cidx(o, i, j, k);
                size_t f0 = fidx(o, i, j, k);
                if (o->cond[c] == 0) {
                    double ro_c = o->ro[c];
                    for (int m = 0; m < 3; ++m)
                        o->f[m][c] = ((o->sig[0][m][f0 + o->fs[0]] - o->sig[0][m][f0]) * ds1 +
                                      (o->sig[1][m][f0 + o->fs[1]] - o->sig[1][m][f0]) * ds2 +
                                      (o->sig[2][m][f0 + o->fs[2]] - o->sig[2][m][f0]) * ds3) * ro_c;
                } else {
                    o->f[0][c] = o->f[1][c] = o->f[2][c] = 0.;
                }
            }
}

/* ---- UseForces (main.cpp:1026-1045) -------------------------------------------- */

void aor_use_forces(ark_oracle *o) {
    const int *n = o->n;
    const double dvc = o->dx[0] * o->dx[1] * o->dx[2];
    const double dt = o->dt;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k < n[2]; ++k)
        for (int j = 1; j < n[1]; ++j)
            for (int i = 1; i < n[0]; ++i) {
                size_t c = cidx(o, i, j, k);
                if (o->cond[c] == 0) {
                    double ro_cn = o->ron[c];
                    for (int m = 0; m < 3; ++m)
                        o->un[m][c] = (ro_cn * dvc * o->un[m][c] + 0.5 * dt * o->f[m][c]) / (dvc * ro_cn);
                }
            }
}

/* ---- Phase2 (main.cpp:1047-2495) ------------------------------------------------ */

/* One sweep along axis d over one line of cells, written from the reference's x1
 * sweep (main.cpp:1726-2011) with the axis made a parameter.  a and b are the two
 * tangential components in the reference's buffer order (x1: u2,u3; x2: u1,u3;
 * x3: u1,u2).  c0 is the cell index of the line start (index 0 along d); the cell
 * at line index s is c0 + s*cst, face s is f0 + s*fst. */
static void sweep_line(ark_oracle *o, int d, size_t c0, size_t f0, double *buf) {
    const int nd = o->n[d];
    const size_t cst = o->cs[d], fst = o->fs[d];
    const int a = d == 0 ? 1 : 0;
    const int b = d == 2 ? 1 : 2;
    const double sound = o->sound, ro0_g = o->rho0, dt = o->dt, dxd = o->dx[d];
    const int q_uses_r = (d != 1);        /* main.cpp:1804 and 2321 vs 2083 */
    const int wall_a_from_normal = (d == 1); /* main.cpp:2219 and 2238 */
    double *rBuf = buf, *qBuf = buf + (nd + 2), *afBuf = buf + 2 * (nd + 2), *abBuf = buf + 3 * (nd + 2),
           *bfBuf = buf + 4 * (nd + 2), *bbBuf = buf + 5 * (nd + 2);
    const double *pF = o->p[d], *uN = o->uf[d][d], *uA = o->uf[d][a], *uB = o->uf[d][b];
    const double *nN = o->un[d], *nA = o->un[a], *nB = o->un[b];
    const double *cN = o->u[d], *cA = o->u[a], *cB = o->u[b];

    int lo = 0, hi = nd;
    if (d == 0 && !o->periodic_x) {
        /* inflow / outflow invariants of a bounded x axis (main.cpp:1731-1745) */
        lo = 1;
        hi = nd - 1;
        rBuf[1] = (o->cond[c0 + cst] < 0.5) ? 1. : 0.;
        afBuf[1] = 0.; bfBuf[1] = 0.;
        qBuf[nd] = 5. / 6.;
        abBuf[nd] = 0.; bbBuf[nd] = 0.;
    }

    for (int s = lo; s <= hi; ++s) {
        size_t c = c0 + (size_t)s * cst, fb = f0 + (size_t)s * fst, ff = fb + fst;
        double u1_f = uN[ff], u1_b = uN[fb], u1_cn = nN[c], u1_c = cN[c];
        double u2_f = uA[ff], u2_b = uA[fb], u2_cn = nA[c], u2_c = cA[c];
        double u3_f = uB[ff], u3_b = uB[fb], u3_cn = nB[c], u3_c = cB[c];
        double ro_cn = o->ron[c], ro_c = o->ro[c];
        double p_f = pF[ff], p_b = pF[fb];
        double p_cn = sound * sound * (ro_cn - ro0_g);
        double p_c = sound * sound * (ro_c - ro0_g);

        double r_f = u1_f + p_f / (ro0_g * sound);
        double r_b = u1_b + p_b / (ro0_g * sound);
        double r_cn = u1_cn + p_cn / (ro0_g * sound);
        double r_c = u1_c + p_c / (ro0_g * sound);
        double r_fn = 2 * r_cn - r_b;

        double q_f = u1_f - p_f / (ro0_g * sound);
        double q_b = u1_b - p_b / (ro0_g * sound);
        double q_cn = u1_cn - p_cn / (ro0_g * sound);
        double q_c = u1_c - p_c / (ro0_g * sound);
        double q_bn = 2 * q_cn - q_f;

        double u2_fn = 2 * u2_cn - u2_b;
        double u2_bn = 2 * u2_cn - u2_f;
        double u3_fn = 2 * u3_cn - u3_b;
        double u3_bn = 2 * u3_cn - u3_f;

        double gr = 2 * (r_cn - r_c) / dt + (u1_cn + sound) * (r_f - r_b) / dxd;
        double gq = q_uses_r ? 2 * (r_cn - r_c) / dt + (u1_cn - sound) * (q_f - q_b) / dxd
                             : 2 * (q_cn - q_c) / dt + (u1_cn - sound) * (q_f - q_b) / dxd;
        double gu2 = 2 * (u2_cn - u2_c) / dt + u1_cn * (u2_f - u2_b) / dxd;
        double gu3 = 2 * (u3_cn - u3_c) / dt + u1_cn * (u3_f - u3_b) / dxd;

        double rmax = max3d(r_f, r_c, r_b) + dt * gr;
        double rmin = min3d(r_f, r_c, r_b) + dt * gr;
        double qmax = max3d(q_f, q_c, q_b) + dt * gq;
        double qmin = min3d(q_f, q_c, q_b) + dt * gq;
        double u2_max = max3d(u2_f, u2_c, u2_b) + dt * gu2;
        double u2_min = min3d(u2_f, u2_c, u2_b) + dt * gu2;
        double u3_max = max3d(u3_f, u3_c, u3_b) + dt * gu3;
        double u3_min = min3d(u3_f, u3_c, u3_b) + dt * gu3;

        if (r_fn > rmax) r_fn = rmax;
        if (r_fn < rmin) r_fn = rmin;
        if (q_bn > qmax) q_bn = qmax;
        if (q_bn < qmin) q_bn = qmin;
        if (u2_fn > u2_max) u2_fn = u2_max;
        if (u2_fn < u2_min) u2_fn = u2_min;
        if (u2_bn > u2_max) u2_bn = u2_max;
        if (u2_bn < u2_min) u2_bn = u2_min;
        if (u3_fn > u3_max) u3_fn = u3_max;
        if (u3_fn < u3_min) u3_fn = u3_min;
        if (u3_bn > u3_max) u3_bn = u3_max;
        if (u3_bn < u3_min) u3_bn = u3_min;

        rBuf[s + 1] = r_fn;
        qBuf[s] = q_bn;
        afBuf[s + 1] = u2_fn;
        abBuf[s] = u2_bn;
        bfBuf[s + 1] = u3_fn;
        bbBuf[s] = u3_bn;
    }

    /* faces 1..nd of the line (main.cpp:1920-2010) */
    double *pW = o->p[d], *uNW = o->uf[d][d], *rW = o->rof[d], *uAW = o->uf[d][a], *uBW = o->uf[d][b];
    for (int s = 1; s <= nd; ++s) {
        size_t cf = c0 + (size_t)s * cst, cb = cf - cst, fc = f0 + (size_t)s * fst;
        double cond_b = o->cond[cb], cond_f = o->cond[cf];
        double un_, pn, ro_n, ua, ub;
        if (cond_b < 0.5 && cond_f < 0.5) {
            double rn = rBuf[s], qn = qBuf[s];
            un_ = (rn + qn) / 2;
            pn = (rn - qn) * sound * ro0_g / 2;
            ro_n = ro0_g + pn / (sound * sound);
            double ucf = nN[cf], ucb = nN[cb];
            if (ucf >= 0 && ucb >= 0) {
                ua = afBuf[s]; ub = bfBuf[s];
            } else if (ucf <= 0 && ucb <= 0) {
                ua = abBuf[s]; ub = bbBuf[s];
            } else if (ucb >= 0 && ucf <= 0) {
                if (ucb > -ucf) { ua = afBuf[s]; ub = bfBuf[s]; }
                else { ua = abBuf[s]; ub = bbBuf[s]; }
            } else {
                ua = nA[cf] + nA[cb] - uA[fc];
                ub = nB[cf] + nB[cb] - uB[fc];
            }
        } else {
            un_ = 0.;
            if (cond_b > 0.5 && cond_f < 0.5) {
                if (nN[cf] <= 0) {
                    double qn = qBuf[s];
                    pn = -qn * sound * ro0_g;
                    ro_n = ro0_g + pn / (sound * sound);
                    ua = abBuf[s]; ub = bbBuf[s];
                } else {
                    ro_n = o->ron[cf];
                    pn = (ro_n - ro0_g) * (sound * sound);
                    ua = wall_a_from_normal ? nN[cf] : nA[cf];
                    ub = nB[cf];
                }
            } else if (cond_b < 0.5 && cond_f > 0.5) {
                if (nN[cb] >= 0) {
                    double rn = rBuf[s];
                    pn = rn * sound * ro0_g;
                    ro_n = ro0_g + pn / (sound * sound);
                    ua = afBuf[s]; ub = bfBuf[s];
                } else {
                    ro_n = o->ron[cb];
                    pn = (ro_n - ro0_g) * (sound * sound);
                    ua = wall_a_from_normal ? nN[cb] : nA[cb];
                    ub = nB[cb];
                }
            } else {
                pn = 0.;
                ro_n = ro0_g;
                ua = 0.; ub = 0.;
            }
        }
        pW[fc] = pn;
        uNW[fc] = un_;
        rW[fc] = ro_n;
        uAW[fc] = ua;
        uBW[fc] = ub;
    }
}

void aor_phase2(ark_oracle *o) {
    const int *n = o->n;
    /* halo (main.cpp:1049-1631): cells u?nCon, roCon, ronCon and the faces of the
     * exchanged axis; then bounded-edge copies (main.cpp:1633-1698) */
    double *cellf[5] = {o->un[0], o->un[1], o->un[2], o->ro, o->ron};
    for (int a = 0; a < 5; ++a) {
        if (o->periodic_x) wrap_cells(o, cellf[a], 0);
        if (o->periodic_z) wrap_cells(o, cellf[a], 2);
    }
    double *fx[5] = {o->uf[0][0], o->uf[0][1], o->uf[0][2], o->rof[0], o->p[0]};
    double *fz[5] = {o->uf[2][0], o->uf[2][1], o->uf[2][2], o->rof[2], o->p[2]};
    for (int a = 0; a < 5; ++a) {
        if (o->periodic_x) wrap_faces(o, fx[a], 0);
        if (o->periodic_z) wrap_faces(o, fz[a], 2);
    }
    if (!o->periodic_x) {
        /* main.cpp:1633-1657: u?nCon and ronCon only (roCon is not copied in x) */
        double *nx[4] = {o->un[0], o->un[1], o->un[2], o->ron};
        for (int a = 0; a < 4; ++a) neumann_cells(o, nx[a], 0);
    }
    if (!o->periodic_z) {
        /* main.cpp:1660-1698: cells incl. roCon, and the x3-normal face halos */
        double *nz[5] = {o->un[0], o->un[1], o->un[2], o->ron, o->ro};
        for (int a = 0; a < 5; ++a) neumann_cells(o, nz[a], 2);
        for (int a = 0; a < 5; ++a) neumann_faces_z(o, fz[a]);
    }

    const int nmax = (n[0] > n[1] ? (n[0] > n[2] ? n[0] : n[2]) : (n[1] > n[2] ? n[1] : n[2]));
    /* x1 sweep: lines over (j,k) interior; x2: (i,k); x3: (i,j) */
    for (int d = 0; d < 3; ++d) {
        const int e1 = d == 0 ? 1 : 0; /* the two axes across the line */
        const int e2 = d == 2 ? 1 : 2;
#pragma omp parallel
        {
            double *buf = (double *)malloc(sizeof(double) * 6 * (size_t)(nmax + 2));
#pragma omp for collapse(2) schedule(static)
            for (int y = 1; y < n[e2]; ++y)
                for (int x = 1; x < n[e1]; ++x) {
                    int idx[3] = {0, 0, 0};
                    idx[e1] = x;
                    idx[e2] = y;
                    size_t c0 = cidx(o, idx[0], idx[1], idx[2]);
                    size_t f0 = fidx(o, idx[0], idx[1], idx[2]);
                    sweep_line(o, d, c0, f0, buf);
                }
            free(buf);
        }
    }
}

/* ---- bulk forcing (project definition, identical in the GPU library) ------------ */

double aor_bulk_velocity(const ark_oracle *o) {
    const int *n = o->n;
    long long s = 0, nf = 0;
#pragma omp parallel for collapse(2) reduction(+ : s, nf) schedule(static)
    for (int k = 1; k < n[2]; ++k)
        for (int j = 1; j < n[1]; ++j)
            for (int i = 1; i < n[0]; ++i) {
                size_t c = cidx(o, i, j, k);
                if (o->cond[c] != 0) continue;
                double u = o->un[0][c];
                if (u != u) u = 0.0;
                if (u > 1073741824.0) u = 1073741824.0;
                if (u < -1073741824.0) u = -1073741824.0;
                s += llrint(u * 4294967296.0);
                ++nf;
            }
    if (nf == 0) return 0.0;
    return ((double)s * (1.0 / 4294967296.0)) / (double)nf;
}

static void add_bulk_force(ark_oracle *o, double G) {
    const int *n = o->n;
    const double dvc = o->dx[0] * o->dx[1] * o->dx[2];
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k < n[2]; ++k)
        for (int j = 1; j < n[1]; ++j)
            for (int i = 1; i < n[0]; ++i) {
                size_t c = cidx(o, i, j, k);
                if (o->cond[c] == 0) o->f[0][c] = o->f[0][c] + (o->ro[c] * dvc) * G;
            }
}

/* nsteps steps in the order of main.cpp:80-91 */
int aor_run(ark_oracle *o, int nsteps) {
    for (int s = 0; s < nsteps; ++s) {
        double ub = o->forcing ? aor_bulk_velocity(o) : 0.0;
        aor_time_step_size(o);
        o->nstep++;
        o->time += 0.5 * o->dt;
        aor_phase1(o);
        aor_stress_tensor(o);
        if (o->forcing) {
            double G = (o->u_target - ub) / o->dt;
            add_bulk_force(o, G);
            o->last_ub = ub;
            o->last_g = G;
        }
        aor_use_forces(o);
        aor_phase2(o);
        aor_phase1(o);
        aor_use_forces(o);
        o->time += 0.5 * o->dt;
    }
    return 0;
}
