/*
 * CPU restatement of the reference CABARET time step -- TEST INFRASTRUCTURE ONLY.
 *
 * This is the oracle: the GPU library is checked against it, and bench.py times it as
 * the CPU baseline.  The product never links it.  It restates, in plain C, the
 * reference's TimeStepSize (source/main.cpp:374-415), Phase1 (main.cpp:417-575),
 * StressTensor (main.cpp:577-1024), UseForces (main.cpp:1026-1045) and Phase2
 * (main.cpp:1047-2495), on the reference's own array layout (Arr3d, i fastest,
 * source/Arr3d.cpp:19-21): cell arrays (C1+2)(C2+2)(C3+2), face arrays
 * (C1+3)(C2+3)(C3+3).  The passive temperature t is not carried (it never feeds back
 * into rho, u1, u2, u3).  Parity with the reference itself is pinned by compiling the
 * reference in place (oracle/_ref) and by the golden fixtures under tests/golden.
 *
 * Array names follow the reference globals: roCon u1Con u2Con u3Con (cells, time level
 * "Con"), ronCon u1nCon u2nCon u3nCon (cells, "nCon"), f1 f2 f3 (forces), condition,
 * p1 ro1 u11 u21 u31 (faces normal to x1), p2 ro2 u12 u22 u32, p3 ro3 u13 u23 u33,
 * sigm11 .. sigm33 (viscous stress on faces).
 */
#ifndef ARK_ORACLE_H
#define ARK_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ark_oracle ark_oracle;

ark_oracle *aor_create(int C1, int C2, int C3, double Lx, double Ly, double Lz, double nu,
                       double sound, double rho0, double cfl, int periodic_x, int periodic_z);
void aor_destroy(ark_oracle *o);
void aor_set_threads(int n);

size_t aor_len(const ark_oracle *o, const char *name);
int aor_put(ark_oracle *o, const char *name, const double *src);
int aor_get(const ark_oracle *o, const char *name, double *dst);

void aor_set_forcing(ark_oracle *o, int on, double u_target);
void aor_set_dt(ark_oracle *o, double dt);
double aor_dt(const ark_oracle *o);
double aor_time(const ark_oracle *o);
int aor_nstep(const ark_oracle *o);
double aor_last_ub(const ark_oracle *o);
double aor_last_g(const ark_oracle *o);

void aor_time_step_size(ark_oracle *o);
void aor_phase1(ark_oracle *o);
void aor_stress_tensor(ark_oracle *o);
void aor_use_forces(ark_oracle *o);
void aor_phase2(ark_oracle *o);
double aor_bulk_velocity(const ark_oracle *o);
int aor_run(ark_oracle *o, int nsteps);

#ifdef __cplusplus
}
#endif
#endif
