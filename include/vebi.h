/*
 * vebi.h -- C-ABI of the GB300 time-step library for the vebisph ISPH solver.
 *
 * The library replaces one call of the Fortran driver:
 *     call div_free(x_mint,y_mint,x_maxt,y_maxt)        source/base/sph2D_incom.F90:97
 * whose body is source/base/div_free.F90:22-124.  In the reference every routine of
 * the step communicates through module globals (source/para/common_2d.F90:20-80); here
 * the same state lives on the device inside an opaque context, and the host copies the
 * particle fields in and out through plain pointers.
 *
 * Conventions
 *  - All entry points are extern "C", take plain pointers/sizes and return an int status
 *    (VEBI_OK == 0).  Warnings are reported in vebi_step_stats.warnings and do not fail.
 *  - Particle fields use the reference's Fortran layout: a field of shape (npar, m) is m
 *    contiguous planes of leading dimension `ld` (the reference's npar,
 *    source/para/common_parameter.F90:5).  tau_p(npar,2,2) is 4 planes ordered
 *    (1,1),(2,1),(1,2),(2,2).  Particle numbering is the reference's: wall ("boundary")
 *    particles first (1..nbS), fluid after (nbS+1..npfb); the library never reorders them.
 *  - Floating point is IEEE binary64 (rkind = c_double, source/para/kind_parameters.F90:11)
 *    and integers are int32 (ikind = c_int, :12).  The logical(c_bool) `inbin` array is
 *    one byte per particle.
 *  - A context owns one CUDA stream and all device memory; it is not thread-safe.
 *    One host thread drives one context, as the reference's serial main loop does.
 */
#ifndef VEBI_H
#define VEBI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VEBI_MAX_PATCHES 16
#define VEBI_MAX_CIRCLES 8
#define VEBI_NSTAGES 16

/* ---- status codes (each maps to a `stop` site of the reference) ------------------- */
enum {
  VEBI_OK = 0,
  VEBI_ERR_ARG = 1,            /* bad argument / inconsistent sizes                          */
  VEBI_ERR_CUDA = 2,           /* CUDA runtime or launch error                                */
  VEBI_ERR_OUT_OF_DOMAIN = 3,  /* neighbour_finding_mod.F90:82-88  (cell index out of range)  */
  VEBI_ERR_CELL_CAPACITY = 4,  /* neighbour_finding_mod.F90:93-103 (cell population > nplink) */
  VEBI_ERR_NEIGH_CAPACITY = 5, /* new: the reference overruns ij_link(npfb,nplink) silently   */
  VEBI_ERR_ALL_IN_BIN = 6,     /* put_in_bin.F90:51-54                                        */
  VEBI_ERR_MIRROR_CAPACITY = 7,/* new: the reference overruns irelation(npfb+1:npfb+esti)     */
  VEBI_ERR_TIMEOUT = 8,        /* a bounded device-side wait gave up                          */
  VEBI_ERR_NO_DEVICE = 9,      /* no usable CUDA device                                       */
  VEBI_ERR_BOUNDARY = 10,      /* check_boundaries failed (input.F90:190-244)                 */
  VEBI_ERR_DIVERGED = 11       /* new, opt-in (vebi_set_velocity_limit): a particle velocity
                                  became non-finite or exceeded the limit                      */
};

/* warning bits in vebi_step_stats.warnings (the reference prints and continues) */
enum {
  VEBI_WARN_BICGSTAB_BREAKDOWN = 1, /* rho == 0, "BICGSTAB Fails" (linear_solver.F90:332-335)  */
  VEBI_WARN_MAXITER = 2,            /* itermax reached without meeting tol                      */
  VEBI_WARN_ESCAPEES = 4            /* replace_escapees relocated particles (mirror_..:336-407) */
};

/* precision modes of the step */
enum {
  VEBI_PREC_FP64 = 0,   /* plain FP64 step: the reference's arithmetic                       */
  VEBI_PREC_MIXED = 1   /* FP32 pair sums/SpMV, FP64 PPE refinement and eigen-step           */
};

/* PPE preconditioner.  NONE is the reference (closed domains unpreconditioned,
 * linear_solver.F90:318; open domains Jacobi, :82-227).  MULTIGRID (opt-in) applies one
 * aggregation-multigrid V-cycle on the cell grid per preconditioning step: the solver stops on
 * the same residual test and reaches the same solution within its tolerance, in far fewer
 * iterations; results differ from the reference's by that tolerance. */
enum {
  VEBI_PRECOND_NONE = 0,
  VEBI_PRECOND_MULTIGRID = 1
};

/*
 * Run parameters.  Field meanings follow INDAT (source/base/input.F90:18-38) and
 * IBOUND (input.F90:51-81).  Patch and circle arrays are 0-based copies of the
 * reference's 1-based arrays; patch indices stored in them (b_periodic_parent) keep
 * the reference's 1-based values.
 */
typedef struct vebi_params {
  /* INDAT */
  double h, dx, dv;                    /* smoothing length, spacing, particle volume        */
  double Ra, Pr, El, beta;             /* Rayleigh, Prandtl, elasticity number, visc. ratio */
  double ve_nonlinearity;              /* PTT epsilon                                       */
  double alpha_evss;                   /* read but unused by the step                       */
  double body_force[2];
  double dt_coef_cfl, dt_coef_visc;
  double tol;                          /* PPE tolerance; the reference hard-codes 1e-8      */
  /* padded domain box passed to div_free (sph2D_incom.F90:64-67); all zero = derive it */
  double x_mint, x_maxt, y_mint, y_maxt;
  /* IBOUND */
  double b_node[VEBI_MAX_PATCHES][2];
  double b_edge[VEBI_MAX_PATCHES][2];
  double b_vel[VEBI_MAX_PATCHES];
  double b_thermal[VEBI_MAX_PATCHES];
  double c_centre[VEBI_MAX_CIRCLES][2];
  double c_radius[VEBI_MAX_CIRCLES];
  double c_omega[VEBI_MAX_CIRCLES];
  double c_vel[VEBI_MAX_CIRCLES][2];
  double c_thermal[VEBI_MAX_CIRCLES];
  int32_t b_type[VEBI_MAX_PATCHES];
  int32_t b_periodic_parent[VEBI_MAX_PATCHES];
  int32_t nb_patches, nb_circles;
  /* INDAT integers */
  int32_t i_open_domain, i_shift_coeff;
  int32_t npfb, nbS;
  int32_t const_mod;                   /* 1 Newtonian, 2 linear PTT / Oldroyd-B (Makefile:11-15) */
  int32_t itermax;                     /* PPE iteration cap; the reference hard-codes 1000       */
  int32_t nplink;                      /* neighbour / cell capacity; the reference uses 75       */
  int32_t nmirror_cap;                 /* mirror capacity; 0 = reference estimate 2*npfb         */
  int32_t precision;                   /* VEBI_PREC_*                                            */
  int32_t correct_velocity;            /* 1: run correct_velocity after the update; the reference
                                          has the call commented out (div_free.F90:105)          */
  int32_t ppe_warm_start;              /* 1: start BiCGSTAB from the previous step's P instead of
                                          x0 = 0 (ppe...:145); changes results, off by default   */
  int32_t ppe_precond;                 /* VEBI_PRECOND_*: preconditioner of the PPE BiCGSTAB     */
  int32_t reserved[4];
} vebi_params;

/* Per-step scalars the Fortran driver and `output` read after div_free
 * (sph2D_incom.F90:98-117, output.F90:84-85). */
typedef struct vebi_step_stats {
  double dt;            /* time step chosen by set_time_step (div_free.F90:126-146)  */
  double LS_residual;   /* sqrt(|r|^2/|r0|^2) at exit of the PPE solve               */
  double umax;          /* max |u| used by the CFL bound                             */
  double max_abs_u, max_abs_v, max_abs_p;   /* TIME file columns (output.F90:84)     */
  double rms_u;         /* secondary_properties diagnostic (div_free.F90:170-183)    */
  double ppe_rhs_mean;  /* DC removed from the PPE right-hand side                   */
  double stage_ms[VEBI_NSTAGES]; /* device time of each stage (0 unless timing on)    */
  double circle_force[2]; /* force of the fluid on the circles (cylinder), x and y: the
                             circle-mirror pair terms of the step (no reference counterpart;
                             0 without circles) */
  int32_t LS_iters;     /* BiCGSTAB iterations                                       */
  int32_t n_inbin;
  int32_t np, npfb, nmirror, maxneighbours;
  int32_t n_escapees;
  int32_t error;        /* first device-side error code of the step (0 = none)       */
  int32_t warnings;     /* VEBI_WARN_* bits                                          */
  int32_t gpu_launches; /* kernels this library launched during the step(s)          */
  int32_t refine_iters; /* mixed precision: outer refinement sweeps                  */
  int32_t LS_iters_total; /* vebi_run_steps: BiCGSTAB iterations summed over the steps */
  int32_t nsteps;       /* steps these statistics cover                              */
  int32_t n_near_pole;  /* diagnostic (no reference counterpart): particles whose conformation
                           eigenvalues are < 1e-7 apart, near the 1/(L2 - L1 + 1e-10) pole of the
                           log-conformation update (predictor_mod.F90:213) */
  int32_t n_near_pole_total; /* vebi_run_steps: the same summed over the steps             */
} vebi_step_stats;

typedef struct vebi_ctx vebi_ctx;

/* Allocate device state for up to npfb particles plus mirrors and build the cell grid
 * (cell_generator, cell_griddin.F90:13-24; kernel constants, input.F90:164-172;
 * corner angles, check_boundaries input.F90:182-273).  Replaces getdata's setup. */
int vebi_create(const vebi_params* params, vebi_ctx** out);

/* Copy the host particle state into the context: the arrays getdata fills
 * (input.F90:105-145).  tau_p and trace_conf may be NULL for const_mod == 1;
 * inbin may be NULL (all false).  ld >= npfb. */
int vebi_upload_state(vebi_ctx* ctx, const double* r, const double* u, const double* tau_p,
                      const double* theta, const double* trace_conf, const uint8_t* inbin,
                      int32_t ld);

/* One time step: the div_free equivalent (div_free.F90:22-124).  `secondary` = 1 runs
 * secondary_properties' vorticity/rms diagnostic (done at dump times, div_free.F90:154).
 * stats may be NULL. */
int vebi_step(vebi_ctx* ctx, double x_mint, double y_mint, double x_maxt, double y_maxt,
              int32_t secondary, vebi_step_stats* stats);

/* Run nsteps steps back to back on the context's stream (no host copies) and return
 * the device time between the first launch and the last completion in *ms.  With timing
 * on, last->stage_ms holds each stage's device time summed over the nsteps steps.
 * A failure in any of the steps is returned (the first failing status is kept on the device
 * until the next vebi_upload_state; the steps after it skip the PPE solve). */
int vebi_run_steps(vebi_ctx* ctx, double x_mint, double y_mint, double x_maxt, double y_maxt,
                   int32_t nsteps, double* ms, vebi_step_stats* last);

/* Copy particle fields back to the host, for dumps (output.F90:44-51,66-72).
 * Any pointer may be NULL to skip that field.  Fields of fluid/wall particles only
 * (1..npfb), in the host's layout with leading dimension ld. */
int vebi_download_state(vebi_ctx* ctx, double* r, double* u, double* tau_p, double* theta,
                        double* p, double* vort, double* a_out, double* trace_conf,
                        int32_t* n_surf, uint8_t* inbin, int32_t ld);

/* Free device state. */
int vebi_destroy(vebi_ctx* ctx);

/* Page-lock (pin) a host array the caller owns, e.g. the Fortran r/u/tau_p arrays, so the
 * transfers of vebi_upload_state / vebi_download_state run at full link speed; and undo it. */
int vebi_pin_host(void* ptr, int64_t bytes);
int vebi_unpin_host(void* ptr);

/* Turn per-stage CUDA-event timing on (1) or off (0). */
int vebi_set_timing(vebi_ctx* ctx, int32_t on);

/* Intermediate arrays of the last step, for parity tests against the CPU oracle:
 * name -> element size and count (vebi_debug_size) and a host copy (vebi_debug_get).
 * Names: see vebisph_gb300/solver.py (DEBUG_FIELDS). */
int vebi_debug_size(vebi_ctx* ctx, const char* name, int64_t* elem_bytes, int64_t* count);
int vebi_debug_get(vebi_ctx* ctx, const char* name, void* out, int64_t bytes);

/* Failure-detection check (no reference counterpart; the reference has no device waits):
 * runs the solvers' bounded grid barrier in a cooperative grid of `blocks` (2..64) blocks in
 * which one block never arrives, with a short poll limit (1..2^22 polls, about 64 ns each).
 * The waiting blocks give up, record VEBI_ERR_TIMEOUT and return; *status_out receives the
 * recorded status and *ms_out (optional) the kernel's duration.  Nothing hangs, and the
 * CUDA context stays usable. */
int vebi_test_barrier_timeout(int32_t blocks, int64_t spin_limit, int32_t* status_out, double* ms_out);

/* Self-check of the library's FP32 <-> FP64 conversions on the integer pipe against the GPU's
 * own conversions, on n seeded inputs (1..2^32) covering every class of value: the counts of
 * mismatching results go to *bad_narrow (FP64 -> FP32) and *bad_widen (FP32 -> FP64).  No
 * reference counterpart. */
int vebi_test_conversions(int64_t n, uint64_t seed, int64_t* bad_narrow, int64_t* bad_widen);

/* ---- A PPE solve that allocates nothing.  No counterpart in the reference. ------------
 * For callers that cannot call cudaMalloc -- a host framework whose allocator owns all device
 * memory, or a real-time loop that must not allocate -- this runs the step's BiCGSTAB
 * (SPARSE_PBICGSTAB_nonull when closed_domain != 0, else the Jacobi SPARSE_PBICGSTAB) on a
 * matrix the caller already holds in device memory, in the layout of vebi_debug_get's
 * ij_count / ppe_col / ppe_val / ppe_diag / ppe_B (ELL [k][i] with stride ell_stride >= n),
 * with x0 = 0, and writes x.  Its working vectors live in a file-scope device array of fixed
 * size (about 4.3 MB, held by every GPU that loads the library until the process exits), so:
 *  - n is at most VEBI_NOALLOC_MAX_ROWS; larger n returns VEBI_ERR_ARG;
 *  - all calls share that array: calls that overlap on the GPU race;
 *  - the first call on a device looks up the array's device address with that device
 *    current; make that first call before any stream capture begins.
 * `stream` is a cudaStream_t (NULL = legacy default stream).  When iters_out or residual_out
 * is non-NULL the call waits for the solve, reports them and returns the solve's device-side
 * status (VEBI_ERR_TIMEOUT when a grid barrier gave up); those pointers must be NULL while the
 * stream is being captured (VEBI_ERR_ARG otherwise).  With both NULL the call only enqueues
 * the solve and returns launch errors: a device-side failure then shows in x, which the
 * kernel fills with NaN. */
#define VEBI_NOALLOC_MAX_ROWS 65536
int vebi_ppe_solve_noalloc(const int32_t* ij_count, const int32_t* ppe_col, const double* ppe_val,
                           const double* ppe_diag, const double* rhs, double* x, int32_t n,
                           int64_t ell_stride, int32_t closed_domain, double tol, int32_t itermax,
                           void* stream, int32_t* iters_out, double* residual_out);

/* ---- Output files (output.F90:18-85) -------------------------------------------------
 * vebi_dump_async snapshots the particle fields after the last step and copies them to pinned
 * host memory on a stream of its own, overlapping the following steps.  vebi_dump_write waits
 * for those copies and writes, in the reference's gfortran list-directed layout:
 *  - part_path: a PART dump (output.F90:40-51; inbin particles skipped, no mirrors as
 *    output_mirrors is .false., div_free.F90:36);
 *  - restart_path: the TEMP_REC.dat restart record (output.F90:59-77).
 * Either path may be NULL.  With VEBI_DUMP_BACKGROUND the files are written on a host thread
 * and the call returns at once; vebi_dump_wait joins it (the next vebi_dump_async does too).
 * VEBI_DUMP_RESTART_READABLE (opt-in) writes the restart particle lines without theta, the
 * layout the reference's restart reader expects (input.F90:123-126): the reference writes
 * theta (output.F90:70) but does not read it back.
 * vebi_format_list formats one list-directed record ('r' real(8), 'i' integer(4) items) with
 * its newline, as the reference's TIME / LS / TIME_OUT lines (output.F90:56,84-85); returns the
 * length, or -1 when cap is too small. */
#define VEBI_DUMP_BACKGROUND 1
#define VEBI_DUMP_RESTART_READABLE 2
typedef struct vebi_dump_info {
  double time, dt, xb_min, xb_max, yb_min, yb_max, dx, av_conc, dv;
  int32_t itime, n_dump, np_inflow, flags;
} vebi_dump_info;
int vebi_dump_async(vebi_ctx* ctx);
int vebi_dump_write(vebi_ctx* ctx, const vebi_dump_info* info, const char* part_path, const char* restart_path);
int vebi_dump_wait(vebi_ctx* ctx);
int64_t vebi_format_list(const char* kinds, const double* reals, const int32_t* ints, char* out, int64_t cap);

/* ---- Batches of independent simulations ----------------------------------------------
 * No counterpart in the reference, which runs one simulation per process.  A batch owns n
 * contexts (one per simulation, each with its own device arrays); uneven particle counts and
 * parameters are allowed.  vebi_batch_step advances every instance by nsteps steps: each step
 * is one launch of a CUDA graph whose independent branches are the instances' captured steps,
 * so the instances overlap on the GPU, and the call waits once at the end.  Each instance
 * keeps its own PPE convergence (iterations and residual in stats[i], an array of n).  An
 * instance whose step fails reports its status in stats[i].error; the failure is sticky for
 * that instance until its next upload (its later steps skip the PPE solve) and the other
 * instances go on: the call returns VEBI_OK unless a CUDA call failed.  Instances are
 * reached with vebi_batch_get for upload/download/inspection; destroying the batch destroys
 * them. */
typedef struct vebi_batch vebi_batch;
int vebi_batch_create(const vebi_params* params, int32_t n, vebi_batch** out);
int vebi_batch_get(vebi_batch* b, int32_t i, vebi_ctx** ctx);
int vebi_batch_step(vebi_batch* b, int32_t nsteps, double* ms, vebi_step_stats* stats);
int vebi_batch_destroy(vebi_batch* b);

/* Rows of the PPE each solver thread owns (>= 1; default 1): the persistent solver runs on
 * ceil(npfb / (256 * rows_per_thread)) blocks, at most the co-resident maximum.  Fewer blocks
 * make a small instance leave room for other instances of a batch.  Re-captures the graph. */
int vebi_set_solver_grid(vebi_ctx* ctx, int32_t rows_per_thread);
/* Tile size of the multigrid V-cycle (VEBI_PRECOND_MULTIGRID; no reference counterpart): the
 * coarse levels of at most `rows` rows run in one thread block with block barriers instead of
 * across the grid with grid barriers (default 2048).  Results do not depend on it. */
int vebi_set_coarse_block_rows(vebi_ctx* ctx, int32_t rows);

/* Static description of the library build. */
const char* vebi_version(void);

/* Last error message of this thread (static storage). */
const char* vebi_last_error(void);

/* ---- Adjoint (reverse mode) of the step over a window --------------------------------
 * No counterpart in the reference, which has no adjoint.  The differentiated map advances the
 * fields (u, theta, tau) over nsteps steps with every step's geometry -- the advected positions
 * r* at which mirrors, pair list, kernel weights, correction matrices and PPE matrix are built,
 * and dt -- taken from the recorded base trajectory.
 *
 * vebi_adjoint_record runs nsteps ordinary steps from the context's state, keeping every step's
 * geometry and pressure (24 bytes per particle per step) and the fields every checkpoint_every
 * steps.  vebi_adjoint_replay runs the
 * differentiated map itself from the context's current fields (upload a perturbed state first:
 * finite differences go through it); replaying the unperturbed state reproduces the record.
 * vebi_adjoint_restore puts a checkpointed state back into the context.  vebi_adjoint_reverse
 * takes dJ/d(state after the window) -- seed_u (2 planes), seed_theta, seed_tau (4 planes),
 * leading dimension ld, any of them NULL for zero -- and returns dJ/d(state before the window)
 * in the same layout, dJ/dWi (Ra, Pr, beta fixed), and the transposed BiCGSTAB iterations.
 * It replays each segment from its checkpoint to rebuild the steps' intermediates, taking each
 * step's pressure from the record instead of solving the PPE again, so it leaves the context's
 * fields at an intermediate state.
 *
 * Scope: closed domains with wall and periodic patches (and their corners) and circles,
 * Newtonian or Oldroyd-B (ve_nonlinearity = 0), FP64 or mixed-precision contexts, no PPE warm
 * start, no correct_velocity; other contexts get VEBI_ERR_ARG from vebi_adjoint_create.  In a
 * mixed-precision context the window runs the mixed step and the VJP, in FP64, uses the FP32
 * weights that step used; its transposed solve is the context's mixed solver.  Destroy the
 * adjoint before its context. */
typedef struct vebi_adjoint vebi_adjoint;
/* Set the Weissenberg number of a context (El = Wi sqrt(Pr/Ra), Ra, Pr, beta unchanged): the
 * relaxation time of the log-conformation update and the polymeric coefficient
 * (1-beta)/(Re Wi).  For parameter continuation and for checking dJ/dWi. */
int vebi_set_weissenberg(vebi_ctx* ctx, double wi);

/* Divergence guard (opt-in; no reference counterpart -- the reference runs on until positions
 * turn NaN and are binned, put_in_bin.F90:27-47).  With u_limit > 0, a step whose fluid
 * velocity entering it, or whose new fluid or wall velocity, is non-finite or above u_limit
 * in magnitude fails with VEBI_ERR_DIVERGED; like every step failure the status is sticky
 * until the next vebi_upload_state.  In a batch this is each instance's own status
 * (stats[i].error), so a simulation that blows up cannot pass silently.  u_limit = 0 turns
 * the guard off (the default). */
int vebi_set_velocity_limit(vebi_ctx* ctx, double u_limit);
int vebi_adjoint_create(vebi_ctx* ctx, int32_t max_steps, int32_t checkpoint_every, vebi_adjoint** out);
int vebi_adjoint_record(vebi_adjoint* adj, int32_t nsteps, vebi_step_stats* last);
int vebi_adjoint_replay(vebi_adjoint* adj, int32_t nsteps, vebi_step_stats* last);
int vebi_adjoint_restore(vebi_adjoint* adj, int32_t step);
int vebi_adjoint_reverse(vebi_adjoint* adj, const double* seed_u, const double* seed_theta, const double* seed_tau,
                         int32_t ld, double* grad_u, double* grad_theta, double* grad_tau, double* grad_wi,
                         int32_t* ls_iters);
int vebi_adjoint_destroy(vebi_adjoint* adj);

#ifdef __cplusplus
}
#endif

#endif /* VEBI_H */
