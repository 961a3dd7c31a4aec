/*
 * ark_gpu.h -- C ABI of the GB300 CABARET time step (libark_gb300.so).
 *
 * The reference (ark-cpp-mpi) has no plugin or FFI layer: its solver is a set of
 * `void f(void)` functions working on global Arr3d arrays (source/main.cpp:12-21,
 * headers/bulk.h:51-108, headers/stress.h:21-23, headers/forces.h:15) and driven by the
 * loop in main.cpp:80-104.  This header is the drop-in for that loop: the same step
 * pieces under the same names, operating on a context instead of globals, plus a fused
 * `ark_step` that runs main.cpp:82-91 on the device.
 *
 * Host arrays use the reference's Arr3d layout (source/Arr3d.cpp:19-21):
 * element (i,j,k) at [k*N1*N2 + j*N1 + i], i fastest.  With C1 x C2 x C3 cells
 * (reference node counts n = C + 1, main.cpp:147-151):
 *   cell arrays  : N = (C1+2, C2+2, C3+2)  -- Arr3d(n1+1, n2+1, n3+1), main.cpp:198-224
 *   face arrays  : N = (C1+3, C2+3, C3+3)  -- Arr3d(n1+2, n2+2, n3+2), main.cpp:226-251
 * Interior cells are 1..C; faces normal to axis d are 1..C_d+1 along d.
 *
 * Every call returns an int status (ARK_OK == 0).  Nothing exits the process or traps the
 * GPU.  One context belongs to one host thread and one CUDA stream; the library keeps no
 * global state.  Host arrays stay owned by the caller; the context owns all device memory.
 */
#ifndef ARK_GPU_H
#define ARK_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum ark_status {
    ARK_OK = 0,
    ARK_ERR_PARAM = 1,       /* bad argument or unsupported configuration                 */
    ARK_ERR_CUDA = 2,        /* a CUDA call failed; ark_last_error() has the text         */
    ARK_ERR_NONFINITE = 3,   /* a NaN or Inf reached the velocity field                    */
    ARK_ERR_STATE = 4,       /* call out of order (e.g. a step before ark_upload)          */
    ARK_ERR_NOMEM = 5,       /* device allocation failed                                   */
    ARK_ERR_UNSUPPORTED = 6, /* a valid request this build does not implement              */
    ARK_ERR_IO = 7           /* a file could not be opened or written                       */
};

enum ark_precision {
    ARK_FP64 = 0, /* parity path: FP64 storage and arithmetic, bit-for-bit with the reference */
    ARK_FP32 = 1  /* FP32 storage and arithmetic; dt, flow-rate and conservation sums in FP64 */
};

/* Scalar parameters.  Names follow headers/constants.h:20-22 and headers/bulk.h:18-35. */
typedef struct ark_params {
    int n1_cells, n2_cells, n3_cells; /* C1, C2, C3 (the reference's n?_g - 1)                 */
    double lx, ly, lz;                /* domain extents: dx_d = L_d / C_d (main.cpp:284-290)    */
    double vis;                       /* VIS, kinematic viscosity                               */
    double sound;                     /* sound speed                                            */
    double ro0;                       /* ro0_g, unperturbed density                             */
    double cfl;                       /* CFL number                                             */
    int periodic_x;                   /* 1: periodic x.  0: bounded, zero-gradient ghosts and the
                                         inflow R = 1 / outflow Q = 5/6 invariants (main.cpp:1731-1745) */
    int periodic_z;                   /* 1: periodic z.  0: bounded, zero-gradient ghosts        */
    int precision;                    /* enum ark_precision                                     */
    int forcing;                      /* 1: constant-flow-rate bulk forcing                     */
    double u_target;                  /* bulk velocity the forcing holds                        */
    int keep_stress;                  /* 1: ark_stress_tensor also fills the sigm?? arrays      */
    int device;                       /* CUDA device ordinal                                    */
} ark_params;

/* Host state in Arr3d layout.  Names are the reference globals.  In ark_download any
 * pointer may be NULL (that array is skipped); ark_upload needs all of them. */
typedef struct ark_host_state {
    double *roCon, *u1Con, *u2Con, *u3Con;     /* cells, level "Con"  (main.cpp:199-204)   */
    double *ronCon, *u1nCon, *u2nCon, *u3nCon; /* cells, level "nCon" (main.cpp:206-211)   */
    double *condition;                         /* cells, 1 solid / 0 fluid (main.cpp:219)  */
    double *p1, *ro1, *u11, *u21, *u31;        /* faces normal to x1 (main.cpp:227-232)    */
    double *p2, *ro2, *u12, *u22, *u32;        /* faces normal to x2 (main.cpp:235-240)    */
    double *p3, *ro3, *u13, *u23, *u33;        /* faces normal to x3 (main.cpp:243-248)    */
} ark_host_state;

/* Scalars of the time loop: dt and TIME (headers/constants.h:20), nStep (headers/bulk.h:18),
 * and the bulk-forcing state of the last step. */
typedef struct ark_scalars {
    double dt;
    double time;
    long long nstep;
    double bulk_velocity; /* mean u1 over fluid cells, taken at the start of the step */
    double bulk_force;    /* G = (u_target - bulk_velocity) / dt                       */
} ark_scalars;

/* Conservation sums over interior fluid cells of the "nCon" level.  Each term is summed in
 * exact 2^-32 fixed point, so the result does not depend on the launch configuration. */
typedef struct ark_sums {
    double mass;      /* sum of ro                            */
    double momentum1; /* sum of ro * u1                       */
    double momentum2; /* sum of ro * u2                       */
    double momentum3; /* sum of ro * u3                       */
    double kinetic;   /* sum of (u1^2 + u2^2 + u3^2) / 2 (the WriteEnergy sum, main.cpp:2851-2860) */
    long long cells;  /* fluid cells summed                   */
} ark_sums;

typedef struct ark_ctx ark_ctx;

/* ---- lifetime ------------------------------------------------------------------------ */

/* Allocates every device array (replaces Input()'s allocation block, main.cpp:198-277).
 * Returns NULL and sets *status on failure. */
ark_ctx *ark_create(const ark_params *params, int *status);

/* Frees the context (replaces FreeMemory(), main.cpp:2893-2961). */
int ark_destroy(ark_ctx *ctx);

/* Text of the last error on this thread. */
const char *ark_last_error(void);
const char *ark_status_string(int status);

/* Number of doubles in a host cell array / face array for these parameters. */
size_t ark_cell_count(const ark_params *params);
size_t ark_face_count(const ark_params *params);

/* ---- state transfer --------------------------------------------------------------------- */

/* Copies a complete host state to the device (synchronous).  After the first upload,
 * host->condition may be NULL: the previous condition, dt, TIME and nStep are kept, so a
 * caller that keeps the state on the host can round-trip it every step. */
int ark_upload(ark_ctx *ctx, const ark_host_state *host);

/* Copies the device state back into every non-NULL host array (synchronous). */
int ark_download(ark_ctx *ctx, ark_host_state *host);

/* Reads or writes one named array ("f1".."f3", "sigm11".."sigm33", or any ark_host_state
 * member name) in Arr3d layout.  Synchronous. */
int ark_get_array(ark_ctx *ctx, const char *name, double *host);
int ark_put_array(ark_ctx *ctx, const char *name, const double *host);

/* ---- the reference's step pieces (same names, same semantics) -------------------------- */

/* TimeStepSize (main.cpp:374-415): dt from the "Con" velocities.  When forcing is on it also
 * takes the bulk velocity of the "nCon" level and sets G for the next ark_stress_tensor. */
int ark_time_step_size(ark_ctx *ctx);

/* Phase1 (main.cpp:417-575): "Con" <- "nCon", then the conservative half step. */
int ark_phase1(ark_ctx *ctx);

/* StressTensor (main.cpp:577-1024): ghost fill of u?Con, viscous stress, force f1..f3
 * (plus the bulk force when forcing is on). */
int ark_stress_tensor(ark_ctx *ctx);

/* UseForces (main.cpp:1026-1045). */
int ark_use_forces(ark_ctx *ctx);

/* Phase2 (main.cpp:1047-2495): ghost fill, then the x1, x2 and x3 characteristic sweeps. */
int ark_phase2(ark_ctx *ctx);

/* BoundaryConditions::alongX1/2/3 (source/BoundaryConditions.cpp:22-83) applied to the "nCon"
 * cell level on the device with the context's own periodicity: axis 1 zero-gradient copy;
 * axis 2 no-slip (the channel's walls: u = 0, ro zero-gradient); axis 3 periodic copy when
 * periodic_z, else no-slip. */
int ark_boundary_fill(ark_ctx *ctx, int axis);

/* BoundaryConditions(u1nCon, u2nCon, u3nCon, ronCon, tnCon, x1Period, x2Period, x3Period, n1,
 * n2, n3, t0).alongX<axis>() (source/BoundaryConditions.cpp:7-83) with the periodicity given
 * explicitly: on the interior of the other two axes, axis 1 copies the zero-gradient ghosts
 * (x1_period is accepted and, as in the class, not read); axes 2 and 3 copy the periodic
 * images when x2_period / x3_period, else set u = 0 and copy ro zero-gradient.  The passive
 * temperature is not carried, so t0 and the class's periodic-x3 temperature line
 * (BoundaryConditions.cpp:73, which copies ro into t) have no counterpart.  FP32 contexts copy
 * their stored rho - ro0, which is the same copy. */
int ark_boundary_conditions(ark_ctx *ctx, int axis, int x1_period, int x2_period, int x3_period);

/* Sets / reads dt (used by the step pieces above). */
int ark_set_dt(ark_ctx *ctx, double dt);

/* ---- the fused time loop ----------------------------------------------------------------- */

/* nsteps iterations of main.cpp:82-91 (TimeStepSize, Phase1, StressTensor, UseForces, Phase2,
 * Phase1, UseForces, with nStep and TIME advanced as there), asynchronous on the context's
 * stream.  The step is captured once into a CUDA graph and replayed. */
int ark_step(ark_ctx *ctx, int nsteps);

/* Blocks until the context's stream is idle and reports a deferred device error
 * (ARK_ERR_NONFINITE when a NaN/Inf was seen in the velocity field). */
int ark_sync(ark_ctx *ctx);

/* Runs nsteps like ark_step and returns the device time between CUDA events recorded on
 * the context's stream around them (milliseconds). */
int ark_time_steps(ark_ctx *ctx, int nsteps, double *ms);

/* Runs nsteps un-graphed fused steps with a CUDA event after every launch and writes the
 * mean device time of each launch (ms) into ms[0..cap-1], in step order; *count receives the
 * number of launches per step.  ark_kernel_name(i) names launch i. */
int ark_kernel_times(ark_ctx *ctx, int nsteps, double *ms, int cap, int *count);
const char *ark_kernel_name(int index);
/* The name of launch `index` of ctx's step as currently configured (FP32 contexts that run Phase2
 * and the second Phase1 as one kernel have 5 launches, the last "phase2_phase1_forces"); NULL
 * past the end. */
const char *ark_step_kernel_name(ark_ctx *ctx, int index);

int ark_get_scalars(ark_ctx *ctx, ark_scalars *out);
int ark_set_scalars(ark_ctx *ctx, const ark_scalars *in);
int ark_conservation_sums(ark_ctx *ctx, ark_sums *out);

/* Mean u1 over the fluid cells of each y plane of the "nCon" level (mean_u1[j-1], j = 1..C2,
 * summed in exact fixed point) and, when wall_shear is not NULL, the wall shear stress at
 * y = -ly/2 and y = +ly/2 in StressTensor's one-sided wall form 2*VIS*u_c/dx2
 * (main.cpp:924-927).  Synchronous. */
int ark_mean_profile(ark_ctx *ctx, double *mean_u1, double *wall_shear);

/* ---- output and statistics ---------------------------------------------------------------
 * VTK files as WriteDataParaView (main.cpp:2577-2745) and WriteAverageValues
 * (main.cpp:2747-2849) write them: legacy binary rectilinear grid, node coordinates (i-1)*dx,
 * cell data as big-endian doubles.  The data are packed on the device in file order and
 * streamed to the file in k slabs.  The file is created or truncated.
 *   ARK_VTK_FULL: every k plane at its place (the layout the file's header declares).
 *   ARK_VTK_REFERENCE: byte for byte the reference's file.  Its row offsets carry no k term
 *     (main.cpp:2670-2671, 2693-2694, 2737-2738, 2843-2844), so each k plane overwrites the
 *     first plane's slot: the file holds the last plane (k = C3) at the start of each block,
 *     zero bytes for the rest of the block, and ends after the last block's first plane.
 *     Identical to ARK_VTK_FULL when n3_cells == 1 (the reference's own 2-D case). */
typedef enum { ARK_VTK_FULL = 0, ARK_VTK_REFERENCE = 1 } ark_vtk_layout;

/* WriteDataParaView: U = (u1, u2, u3) and "scalars PC" = density of the "nCon" level, and
 * the vorticity R of the current face values (main.cpp:2716-2733).  The reference names the
 * file <dirPath>out_<nStep>.vtk; here the caller passes the path.  Synchronous. */
int ark_write_vtk(ark_ctx *ctx, const char *path, int layout);

/* AverageValues (main.cpp:2878-2891): averageU_m += u_m(nCon) * dt over interior cells, dt
 * of the last step.  The averages are FP64 device arrays in the reference's averageU layout
 * ((n1_cells+2) x (n2_cells+3) x (n3_cells+2), one j row more than a cell array), zero until
 * first used; ark_get_array / ark_put_array reach them as "averageU1".."averageU3". */
int ark_average_values(ark_ctx *ctx);
/* on != 0: every step of ark_step ends with AverageValues (inside the step's CUDA graph). */
int ark_set_averaging(ark_ctx *ctx, int on);
/* WriteAverageValues(start_time): averageU / (TIME - start_time) as the U vectors. */
int ark_write_average_vtk(ark_ctx *ctx, const char *path, double start_time, int layout);

/* WriteEnergy's value (main.cpp:2851-2870): the sum over interior cells of
 * (u1^2 + u2^2 + u3^2)/2 of the "nCon" level, times the domain volume lz*ly*lx.  The sum
 * is FP64 in a fixed tree order (deterministic; the reference's sequential order differs
 * from it in the last bits).  Synchronous. */
int ark_kinetic_energy(ark_ctx *ctx, double *energy);
/* WriteEnergy: appends "(TIME; energy) " (printf "(%f; %f) ") to the file at path. */
int ark_write_energy(ark_ctx *ctx, const char *path);

/* Per y plane of the "nCon" level: the means over the interior cells of the plane of u1, u2,
 * u3, u1^2, u2^2, u3^2, u1u2, u1u3, u2u3 (out[9*(j-1) + q], 9 * n2_cells doubles): the mean
 * profiles and, with the means, the Reynolds stresses.  Fixed-order FP64 sums.  Synchronous. */
int ark_plane_stats(ark_ctx *ctx, double *out);

/* The vorticity R of WriteDataParaView for every interior cell: out[3*n + m], n = (i-1) +
 * n1_cells*((j-1) + n2_cells*(k-1)), host byte order.  Synchronous. */
int ark_vorticity(ark_ctx *ctx, double *out);

/* Self-check of the correctly rounded FP64 divisions the FP64 kernels use, against the GPU's
 * IEEE division, on n random operand pairs (numerators over the whole exponent range, zeros
 * and subnormals included) and on small exact cases: the integer-pipe quotient by a divisor
 * with a prepared significand reciprocal (run constants, dt), the same with the numerator
 * doubled, the per-cell divisor's reciprocal built by integer Newton steps and its quotients,
 * the exact halving, and the Markstein form q = a*RN(1/b) with two corrections that the rare
 * cases fall back to; also that the device prepares the same reciprocals as the host.
 * *mismatches receives the count (0 expected).
 * Runs on the current device. */
int ark_selftest_division(long long n, unsigned long long seed, long long *mismatches);

/* Check of the error path of the TMA-staged Phase1's bounded waits (FP32 contexts with a
 * state): launches one Phase1 + stress on ctx's state whose planes expect 16 bytes more than
 * their copies bring, so no stage's mbarrier completes; every block gives up after its bounded
 * waits (half a second each), lets its copies land and leaves, and the next ark_sync reports
 * ARK_ERR_CUDA.  No fault: the context stays usable, but its state is no longer a step's result
 * and its error bit stays set (re-create the context).  Returns ARK_OK once launched. */
int ark_selftest_staging_timeout(ark_ctx *ctx);

/* Bounds-checked builds (compiled with -DARK_CHECK, the library's lib_check/ variant): the
 * kernels compare the indices of their global-memory accesses (sweeps, ghost fills, halo
 * exchange, boundary conditions, the closure's inference) and the cell coordinates their blocks
 * decode (Phase1 kernels, the ensemble's work lists) with the extents they must stay inside; an
 * index outside is replaced by 0 (the access stays inside the array) and recorded, nothing
 * traps.  out[0..3] = {violations since the last reset, the first value, its bound, the source
 * line in csrc/}; reset != 0 clears the record.  Ordinary builds return ARK_ERR_UNSUPPORTED.
 * Call after ark_sync. */
int ark_bounds_check(int reset, long long *out);

/* Host-only check (no GPU needed) of the copy plan of the FP32 Phase1 kernel that stages its
 * planes in shared memory, for an n1 x n2 x n3-cell grid and planes_per_block planes per block
 * (0: the kernel's own choice): every 16-byte copy inside its array and its stage and aligned,
 * no two copies into one byte, and every shared-memory read of every thread mapped to the
 * element the one-cell kernel reads; and the same for the FP32 kernel that runs Phase2 and the
 * second Phase1 together (its reads mapped to the elements the sweep kernels read).  Returns the
 * number of problems (msg receives the first), or -1 for a bad size. */
int ark_selftest_staging(int n1_cells, int n2_cells, int n3_cells, int planes_per_block, char *msg, int cap);

/* ---- learned eddy-viscosity closure (a project extension; the reference has none) --------
 * A network nu_t / nu = softplus(w3 . GELU(W2 GELU(W1 x_n + b1) + b2) + b3) (10 -> 32 -> 32 ->
 * 1, BF16 weights, FP32 accumulation; GELU in its tanh form) of 10 features of the local velocity gradient (the seven
 * integrity-basis invariants of S and W as signed roots, the wall-frame shear -sgn(y) S_12 and
 * vorticity -sgn(y) W_12, and y+ = (ly/2 - |y|) u_tau / vis), normalised x_n = (x - mu) / sd.
 * Trained on 3 x 3 x 3 box-filtered fields of fine runs against the least-squares eddy
 * viscosity of the filtered-out stress, max(0, -tau^d : S^d / (2 S^d : S^d)), by the library's
 * own forward / backward kernels and Adam (FP32 master weights).  Parameters (1441, FP64 in
 * these calls) are ordered W1[32][10], b1[32], W2[32][32], b2[32], w3[32], b3. */
typedef struct ark_closure_data ark_closure_data; /* training samples on the device */
typedef struct ark_mlp ark_mlp;                   /* the network and its optimiser state */

const char *ark_closure_last_error(void);
ark_closure_data *ark_closure_data_create(long long capacity, int device, int *status);
int ark_closure_data_destroy(ark_closure_data *data);
long long ark_closure_data_size(const ark_closure_data *data);
int ark_closure_data_clear(ark_closure_data *data);
/* rows [first, first + count): features (10 floats per row) and targets (nu* / nu) */
int ark_closure_data_get(ark_closure_data *data, long long first, long long count, float *features, float *targets);
int ark_closure_data_append(ark_closure_data *data, long long count, const float *features, const float *targets);
/* Appends the samples of the context's "nCon" level: the interior velocities box-filtered
 * 3 x 3 x 3 (x, z periodic; the walls reflect velocities), then on the lattice i = ox + sx*a,
 * k = oz + sz*b (1-based i = 1 + ox + ..., every j) the features of the filtered field and the
 * target.  FP32 or FP64 context of a periodic channel without interior solids. */
int ark_closure_sample(ark_ctx *ctx, ark_closure_data *data, int sx, int sz, int ox, int oz, double u_tau);
/* Per y plane of the field filtered by the last ark_closure_sample: the means over x and z of
 * u1, u2, u3, u1^2, u2^2, u3^2, u1u2, u1u3, u2u3 (out[9*(j-1) + q], 9 * n2_cells doubles). */
int ark_closure_data_filtered_stats(ark_closure_data *data, double *out);

ark_mlp *ark_mlp_create(unsigned long long seed, int device, int *status);
int ark_mlp_destroy(ark_mlp *mlp);
int ark_mlp_set(ark_mlp *mlp, const double *params, const double *mu, const double *sd);
int ark_mlp_get(ark_mlp *mlp, double *params, double *mu, double *sd);
/* mu, sd of the dataset's features */
int ark_mlp_fit_normalization(ark_mlp *mlp, ark_closure_data *data);
/* gradient of the mean squared error over rows [first, first + count) (FP32 accumulation in a
 * fixed order) and the error itself */
int ark_mlp_gradient(ark_mlp *mlp, ark_closure_data *data, long long first, long long count, double *grad, double *loss);
int ark_mlp_train(ark_mlp *mlp, ark_closure_data *data, int epochs, long long batch, double lr, double *loss);
/* nu_t / nu of rows [first, first + count): FP32 throughout (as trained) ... */
int ark_mlp_predict(ark_mlp *mlp, ark_closure_data *data, long long first, long long count, float *out);
/* ... and through the step's inference: the two hidden layers as BF16 tensor-core multiplies
 * (FP32 accumulation, BF16 activations) and GELU with the hardware tanh approximation. */
int ark_mlp_predict_tc(ark_mlp *mlp, ark_closure_data *data, long long first, long long count, float *out);
/* mlp != NULL: every ark_step of this FP32 context evaluates nu_t from the "Con" velocities
 * before the stress and uses vis + (nu_t(c) + nu_t(neighbour))/2 on each face, with the
 * network as it is at this call (call again after further training).  mlp == NULL: the plain
 * step.  The step pieces called one by one stay plain.  The array is readable as "nut". */
int ark_set_closure(ark_ctx *ctx, const ark_mlp *mlp, double u_tau);

/* Times the kernel shapes of the step on the live state (it advances) and keeps the fastest,
 * one setting at a time: the shape of the Phase1 with stress (0 one cell per thread, 1
 * marching, 2 staged in shared memory with cp.async copies (FP32), 3 face quantities computed
 * once (FP64), 4 staged with TMA tensor copies (FP32) on 64 x 4 tiles, 6 the same on 128 x 2
 * tiles), of the second Phase1, the Phase2 form
 * (FP32: three sweep kernels, or one kernel for the three sweeps and the second Phase1 with
 * cp.async or TMA copies, or the x1 sweep folded into a TMA-staged Phase1 + stress with a seam
 * kernel in its place), the x2/x3 sweeps' segment length (8 to 64 faces), the x1
 * sweep's lines per warp (1 to 4) and the staged / face-centric Phase1's planes per block, each
 * candidate timed three times (best kept).  The results do not depend on the shapes.  choice
 * (5 ints, may be NULL): the chosen {shape 1, shape 2, segment, microseconds per step, Phase2
 * form: 0 sweep kernels, 1 one sweep kernel (only by ARK_PHASE2_FUSED=1), 2 sweeps and second
 * Phase1 in one kernel, 3 the same with TMA copies, 4 the x1 sweep folded into Phase1 + stress}. */
int ark_autotune(ark_ctx *ctx, int steps_per_candidate, int *choice);

/* ---- ensembles: many independent channels in one launch per phase ------------------------
 * The members (FP32 contexts, each with its own grid size and parameters, all on one device
 * and all with or all without bulk forcing) advance together: every phase of the step is one
 * persistent launch over a table of the members' blocks, and the step is one CUDA graph.
 * Each member's result is bit-identical to running it alone in an FP32 ark_ctx.  The
 * single-device analogue of the reference running independent problems side by side, one
 * per MPI job. */
typedef struct ark_ensemble ark_ensemble;

ark_ensemble *ark_ensemble_create(const ark_params *params, int n, int *status);
int ark_ensemble_destroy(ark_ensemble *ens);
const char *ark_ensemble_last_error(void);
int ark_ensemble_size(const ark_ensemble *ens);
int ark_ensemble_upload(ark_ensemble *ens, int member, const ark_host_state *host);
int ark_ensemble_download(ark_ensemble *ens, int member, ark_host_state *host);
int ark_ensemble_step(ark_ensemble *ens, int nsteps);
int ark_ensemble_sync(ark_ensemble *ens);
int ark_ensemble_time_steps(ark_ensemble *ens, int nsteps, double *ms);
/* Per-launch times of a step (ms, averaged over nsteps; names from ark_ensemble_kernel_name). */
int ark_ensemble_kernel_times(ark_ensemble *ens, int nsteps, double *ms, int cap, int *count);
/* The name of launch `index` of an ensemble step (NULL past the last). */
const char *ark_ensemble_kernel_name(int index);
/* The same for the ensemble's current shape: with the x3 sweep folded into Phase1 + stress
 * (shapes 6 and 7), "phase1_stress_sweep_x3" and "sweep_x3_seams" in launches 2 and 5; with the
 * x1 sweep too (8 and 9), "phase1_stress_sweep_x1_x3" and "sweep_x1_seams" in launches 2 and 3. */
const char *ark_ensemble_step_kernel_name(const ark_ensemble *ens, int index);
int ark_ensemble_get_scalars(ark_ensemble *ens, int member, ark_scalars *out);
int ark_ensemble_mean_profile(ark_ensemble *ens, int member, double *mean_u1, double *wall_shear);
/* Times each candidate kernel shape (for each Phase1: 0 one cell per thread, 1 marching, 2 planes
 * staged in shared memory with cp.async copies, 4 the same with TMA tensor copies, 5 TMA with
 * 32 x 8 tiles for the members whose width is an odd multiple of 32; for the Phase1 with stress
 * also 6 and 7, shapes 4 and 5 with the x3 sweep folded in, and 8 and 9, with the x1 and x3
 * sweeps folded in; the x2/x3 sweep segment
 * length) for steps_per_candidate steps on the
 * live state -- the results do not depend on the shape -- and keeps the fastest.  choice (4
 * ints, or NULL): {Phase1+stress shape, second Phase1 shape, segment target, microseconds per
 * step}. */
int ark_ensemble_autotune(ark_ensemble *ens, int steps_per_candidate, int *choice);
/* Sets the kernel shape directly (march_a: 0, 1, 2 or 4 to 9, march_b: 0, 1, 2, 4 or 5 as
 * above).  Until this or ark_ensemble_autotune is called, an ensemble uses 7, 5 and 32-face
 * segments. */
int ark_ensemble_set_shape(ark_ensemble *ens, int march_a, int march_b, int segment);

/* ---- slab groups: one channel split along z -------------------------------------------------
 * The reference's domain decomposition (main.cpp:53-67: MPI_Dims_create / MPI_Cart_create,
 * one-plane halos) applied along z on one device: the grid's C3 planes are split into nslabs
 * slabs (C3 / nslabs planes each, one more for the first C3 % nslabs), each an ark_ctx of its
 * own that keeps its x wrap and y walls, and the z ghosts are exchanged plane by plane at the
 * reference's two exchange points of a step: the "Con" velocities and density before the stress
 * (main.cpp:601-801) and, before Phase2, the half-step level, the old density and the faces
 * normal to z (main.cpp:1049-1631).  dt (main.cpp:412, MPI_Allreduce MIN) and the bulk-flow sum
 * are reduced exactly over all slabs (max |u| as integer bit patterns, fixed-point sums), so the
 * group's result is the single context's bit for bit.  Periodic z wraps around the group; a
 * bounded z copies zero-gradient at its ends.  A step is one CUDA graph on the group's stream.
 * Upload and download take whole-domain host states (Arr3d layout); the step is the fused
 * main.cpp:82-91 with the three separate Phase2 sweep kernels. */
typedef struct ark_slabs ark_slabs;

ark_slabs *ark_slabs_create(const ark_params *params, int nslabs, int *status);
int ark_slabs_destroy(ark_slabs *group);
int ark_slabs_count(const ark_slabs *group);
int ark_slabs_upload(ark_slabs *group, const ark_host_state *host);
int ark_slabs_download(ark_slabs *group, ark_host_state *host);
int ark_slabs_step(ark_slabs *group, int nsteps);
int ark_slabs_sync(ark_slabs *group);
int ark_slabs_time_steps(ark_slabs *group, int nsteps, double *ms);
int ark_slabs_get_scalars(ark_slabs *group, ark_scalars *out);
int ark_slabs_conservation_sums(ark_slabs *group, ark_sums *out);

/* The decomposition plan (host only, no GPU needed): the global interior planes
 * [*k_first, *k_last] (1-based) of slab `slab` of nslabs over n3_cells planes, and its
 * neighbour slabs below and above (-1 at a bounded end; periodic z wraps). */
int ark_slab_plan(int n3_cells, int nslabs, int slab, int periodic_z, int *k_first, int *k_last, int *below,
                  int *above);
/* The halo schedule (host only): for a cell array (face = 0) or a face array (face = 1) of a
 * slab of c3 planes, the ghost plane written on side 0 (below) or 1 (above) and the plane of
 * the source slab (c3_src planes) it is copied from: cells ghost 0 <- plane c3_src of the slab
 * below, ghost c3+1 <- plane 1 of the slab above; faces halo 0 <- face c3_src, halo c3+2 <-
 * face 2; bounded != 0 (no neighbour): the slab's own zero-gradient planes 1, c3 (faces 1,
 * c3+1). */
int ark_slab_halo_planes(int face, int side, int c3, int c3_src, int bounded, int *dst_plane, int *src_plane);

/* ---- host-side helpers (no GPU needed) ----------------------------------------------------- */

/* Seeded channel-flow initial state (a project definition, not part of the reference):
 * interior cell (i,j,k), visited k-major / i fastest, draws three splitmix64 uniforms
 * r1,r2,r3 in [0,1) and sets u1 = 1.5*u_target*(1 - y*y) + amp*(2*r1 - 1),
 * u2 = amp*(2*r2 - 1), u3 = amp*(2*r3 - 1), ro = ro0, with y = -ly/2 + (j - 0.5)*dy.
 * Ghost cells are periodic copies in x and z; y ghost rows are solid (condition = 1).
 * Faces hold the mean of their two cells (0 on the y walls), p = 0, face ro = ro0.
 * "Con" starts equal to "nCon".  Fills every array of *out (caller-allocated). */
int ark_channel_init(const ark_params *params, uint64_t seed, double amp, ark_host_state *out);

/* Conservation sums (the same fixed-point sums as ark_conservation_sums) of FP64 DEVICE
 * arrays that the caller owns, in Arr3d cell layout: ro, u1, u2, u3 and condition, each
 * (C1+2)(C2+2)(C3+2) doubles, cells with condition == 0 summed.  No counterpart in the
 * reference.  It allocates nothing, for callers that cannot allocate device memory at this
 * point (their memory is held by a full grid or by another framework's pool, and a
 * cudaMalloc/cudaFree would synchronize the device or fail); it needs no ark_ctx.
 * Limit: at most 67,108,864 interior cells (larger grids return ARK_ERR_PARAM).  Scratch is
 * one static 65,600-byte device array per GPU, kept until exit and shared by all calls:
 * calls that overlap on the GPU race.  Runs on the current device's legacy default stream
 * and waits for the result.  The first call on a device looks up the scratch address and
 * keeps it, so make that call before any stream capture; a cudaDeviceReset of the device
 * after it is not supported.  Errors set ark_last_error(). */
int ark_conservation_sums_noalloc(const ark_params *params, const double *ro, const double *u1,
                                  const double *u2, const double *u3, const double *condition,
                                  ark_sums *out);

/* Allocates every array of a host state in page-locked memory (zero-filled), sized for
 * params; ark_free_host_state releases them.  Either works without ark_create. */
int ark_alloc_host_state(const ark_params *params, ark_host_state *out);
int ark_free_host_state(ark_host_state *host);

#ifdef __cplusplus
}
#endif
#endif
