/*
 * swm_gpu.h -- C ABI of the GB300 implementation of the SWM time-stepping
 * hot path (shallow-water C-grid tendencies + Adams-Bashforth, lateral
 * mixing, damping, forcing, tracer advection-diffusion, red-black SOR).
 *
 * The entry points mirror the Fortran module entry points of martinclaus/swm
 * they replace; each declaration cites the routine (path:line in the swm
 * source tree).  A Fortran host binds them with ISO_C_BINDING interfaces;
 * every function returns 0 on success or a positive SWM_GPU_E* code, and
 * swm_gpu_last_error() gives the message.
 *
 * Arrays are Fortran column-major (Nx, Ny) = C row-major [Ny][Nx], FP64,
 * indices 0-based; masks are int8 (1 = ocean).  Host pointers only: the
 * library owns every device buffer.
 */
#ifndef SWM_GPU_H
#define SWM_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
enum {
  SWM_GPU_OK = 0,
  SWM_GPU_EINVAL = 1,        /* bad argument / call order                         */
  SWM_GPU_ECUDA = 2,         /* CUDA runtime error                                */
  SWM_GPU_ENOMEM = 3,        /* device allocation failed                          */
  SWM_GPU_ENOT_CONVERGED = 4,/* SOR hit its iteration cap (the reference warns)   */
  SWM_GPU_EDEVICE = 5        /* device-side check failed (error word set)         */
};

/* ---- physics switches (include/model.h CPP defines) ---- */
enum {
  SWM_MODE_NONE = 0,          /* no linearisation define                          */
  SWM_MODE_NONLINEAR = 1,     /* FULLY_NONLINEAR                                  */
  SWM_MODE_LIN_REST = 2,      /* LINEARISED_STATE_OF_REST                         */
  SWM_MODE_LIN_MEAN = 3       /* LINEARISED_MEAN_STATE                            */
};
enum { SWM_MIX_LAPLACE = 0, SWM_MIX_BIHARMONIC = 1 /* project extension */ };

/* ---- execution paths ---- */
enum {
  SWM_PATH_PLAIN_FP64 = 0,    /* per-module FP64 kernels, bit-for-bit with the FP64 restatement */
  SWM_PATH_FUSED_FP64 = 1,    /* one fused FP64 stencil kernel per step            */
  SWM_PATH_FUSED_FP32C = 2    /* fused FP32 stencil, state kept as FP32 hi+lo pair */
};

typedef struct swm_gpu_config {
  int32_t nx, ny;               /* &domain_nl Nx, Ny                               */
  int32_t mode;                 /* SWM_MODE_*                                      */
  int32_t lateral_mixing;       /* LATERAL_MIXING                                  */
  int32_t quadratic_friction;   /* QUADRATIC_BOTTOM_FRICTION                       */
  int32_t barotropic;           /* BAROTROPIC                                      */
  int32_t mixing_kind;          /* SWM_MIX_*                                       */
  int32_t coriolis_approx;      /* &domain_nl coriolis_approx                      */
  int32_t tracer_nan_guard;     /* 1: 0/0 tracer coefficients taken as 0           */
  int32_t damping_additive;     /* 1: damping entries add (older selfcheck build)  */
  int32_t mask_psi_bs;          /* 1: basic-state psi zeroed on land (same)        */
  int32_t tracer_flux;          /* 0: reference centred tracer flux; 1: third-order
                                   upwind-biased flux (extension)                  */
  int32_t frozen_flow;          /* 1: SWM state held fixed after the initial
                                   conditions, only tracers step (extension)      */
  double dt, G, Ah, A, OMEGA, RHO0, lbc, theta0;
  double lon_s, lon_e, lat_s, lat_e;
  double H_overwrite;           /* 0 = unset                                       */
  double ab_chi, minD;
  double tau_scale;             /* TAU_SCALE (1.0 when undefined)                  */
  double bih;                   /* biharmonic coefficient (extension)              */
  int32_t path;                 /* SWM_PATH_*                                      */
  int32_t reserved;
} swm_gpu_config;

/* field ids for swm_gpu_get_field / swm_gpu_set_field (registry names of
   vars_module.f90:67-104 in brackets) */
enum {
  SWM_F_U = 0,        /* SWM_u(:,:,N0)    [SWM_U]   */
  SWM_F_V,            /* SWM_v(:,:,N0)    [SWM_V]   */
  SWM_F_ETA,          /* SWM_eta(:,:,N0)  [SWM_ETA] */
  SWM_F_D, SWM_F_DH, SWM_F_DU, SWM_F_DV,
  SWM_F_EDENS, SWM_F_POT, SWM_F_ZETA, SWM_F_MU, SWM_F_MV,
  SWM_F_H, SWM_F_HU, SWM_F_HV, SWM_F_HETA,
  SWM_F_IMPL_U, SWM_F_IMPL_V, SWM_F_IMPL_ETA,
  SWM_F_GAMMA_LIN_U, SWM_F_GAMMA_LIN_V, SWM_F_GAMMA_LIN_ETA, SWM_F_GAMMA_SQ_U, SWM_F_GAMMA_SQ_V,
  SWM_F_FX, SWM_F_FY, SWM_F_FETA,
  SWM_F_U_BS, SWM_F_V_BS, SWM_F_ZETA_BS,
  SWM_F_LATMIX_U, SWM_F_LATMIX_V,
  SWM_F_GU, SWM_F_GV, SWM_F_GETA,  /* newest increment G(:,:,NG0) */
  SWM_F_PSI,          /* computeStreamfunction (calc_lib.f90:727-780), formed on the device */
  SWM_F_NFIELDS
};

/* damping (swm_damping_nl) and forcing (swm_forcing_nl) kinds */
enum { SWM_TERM_GAMMA_LIN_U, SWM_TERM_GAMMA_LIN_V, SWM_TERM_GAMMA_LIN_ETA,
       SWM_TERM_GAMMA_SQ_U, SWM_TERM_GAMMA_SQ_V };
enum { SWM_DAMP_UNIFORM, SWM_DAMP_SPONGE, SWM_DAMP_FILE };
enum { SWM_SPONGE_N = 1, SWM_SPONGE_S = 2, SWM_SPONGE_W = 4, SWM_SPONGE_E = 8 };
enum { SWM_FRC_WIND, SWM_FRC_OSC, SWM_FRC_CUSTOM, SWM_FRC_HEAT, SWM_FRC_EMF };
enum { SWM_CMP_ZONAL, SWM_CMP_MERID, SWM_CMP_CONT, SWM_CMP_U2, SWM_CMP_V2, SWM_CMP_REY };

typedef struct swm_gpu_ctx swm_gpu_ctx;

/* ---- context ---- */
const char *swm_gpu_last_error(void);
int swm_gpu_create(const swm_gpu_config *cfg, swm_gpu_ctx **out);
int swm_gpu_destroy(swm_gpu_ctx *ctx);
/* waits for the context's stream; SWM_GPU_EDEVICE when a step kernel that
   stages its rows by bulk asynchronous copies (SWM_GB300_MARCH_PREFETCH=3)
   gave up waiting for a row (the same holds for
   swm_gpu_ensemble_synchronize) */
int swm_gpu_synchronize(swm_gpu_ctx *ctx);
/* the CUDA stream (cudaStream_t) every call of this context runs on */
void *swm_gpu_stream(swm_gpu_ctx *ctx);
/* number of kernels this context has launched so far */
int64_t swm_gpu_launch_count(swm_gpu_ctx *ctx);
/* Launch shape of the FP32 pair step kernel, as its autotuner picked it on
   the first step: rows per warp strip (the cost target of a row group), the
   cost of a row whose window holds land, and the blocks per launch; zeros
   before the first step or on other paths.  No reference counterpart. */
int swm_gpu_step_shape(swm_gpu_ctx *ctx, double *rows, double *masked_cost, int *blocks);
/* Host-only planner behind that shape: the tiles of the FP32 step kernel for
   an nx x ny basin (mixing 0 none, 1 Laplacian, 2 biharmonic) from its packed
   mask words (per point: bits 0-3 ocean at H, u, v, eta; bits 4-7 the same
   at i-1, bits 8-11 at i+1), cut for `rows` rows per warp with a masked row
   counted masked_cost.  Writes up to `capacity` tiles as (strip, first row,
   rows) triples, four per block, rows 0 for padding; returns the number of
   tiles, or -1 for bad arguments.  Runs no GPU code. */
int swm_gpu_plan_step_tiles(int mixing, int nx, int ny, const uint16_t *mask_words, double rows,
                            double masked_cost, int32_t *tiles, int capacity);
/* Columns of the basin one warp strip of the FP32 step kernel updates, for
   the mixing kind (0 none, 1 Laplacian, 2 biharmonic): the width the tiles
   of swm_gpu_plan_step_tiles are strips of.  No reference counterpart. */
int swm_gpu_step_strip_columns(int mixing);

/* ---- SWM_initSWM pieces (swm_module.f90:37-48) ---- */
/* initDomain (domain_module.f90:49-207): grids, masks, depth on all grids,
   metric and Coriolis; H may be NULL (closed 1 m basin), H_missing may be NULL */
int swm_gpu_domain(swm_gpu_ctx *ctx, const double *H, const int8_t *H_missing);
/* SWM_timestep_init (swm_nonlinear_timestep_module.f90:60-101); psi_bs only
   for SWM_MODE_LIN_MEAN, else NULL */
int swm_gpu_timestep_init(swm_gpu_ctx *ctx, const double *psi_bs);
/* getDampingCoefficient (swm_damping_module.f90:137-203), one swm_damping_nl
   record; file_data only for SWM_DAMP_FILE */
int swm_gpu_add_damping(swm_gpu_ctx *ctx, int term, int type, double value, double sl_length,
                        double sl_cutoff, int sponge_flags, const double *file_data);
/* tail of SWM_damping_init (swm_damping_module.f90:78-115) */
int swm_gpu_finish_damping(swm_gpu_ctx *ctx);
/* SWM_forcing_initStream (swm_forcing_module.f90:592-646); d2 = imaginary part
   for oscillating forcing; returns the stream id in *id */
int swm_gpu_add_stream(swm_gpu_ctx *ctx, int type, int component, double omega, int is_constant,
                       const double *d1, const double *d2, int *id);
/* time-interpolated record of a time-dependent stream (memchunk getChunkData
   output, swm_forcing_module.f90:319,356-357) -- one H2D copy */
int swm_gpu_set_stream_data(swm_gpu_ctx *ctx, int id, const double *d1, const double *d2);
/* same for a stream whose data is constant along each row: Ny values per
   part (one H2D copy of Ny doubles); d2 may be NULL */
int swm_gpu_set_stream_rows(swm_gpu_ctx *ctx, int id, const double *rows1, const double *rows2);
/* All records of part 1 or 2 (nrec x Nx x Ny) of a time-dependent stream,
   kept on the device; each step swm_gpu_stream_interp then forms the record
   in use on the device from the memchunk bracket the host computes (record
   indices r0, r1 and their times t0, t1; r1 < 0: exactly record r0) as
   getChunkData (memchunk_module.f90:214-246) does, instead of one H2D copy
   of the whole field per step and stream */
int swm_gpu_stream_records(swm_gpu_ctx *ctx, int id, int part, int nrec, const double *records);
int swm_gpu_stream_interp(swm_gpu_ctx *ctx, int id, int part, int r0, int r1, double t, double t0, double t1);
/* SWM_forcing_init (swm_forcing_module.f90:78-127) */
int swm_gpu_forcing_init(swm_gpu_ctx *ctx);
/* SWM_initialConditions (swm_module.f90:156-181) */
int swm_gpu_initial_conditions(swm_gpu_ctx *ctx, const double *eta, const double *u, const double *v);

/* ---- time loop (model.f90:159-196) ---- */
/* SWM_timestep -> SWM_timestep_step (swm_nonlinear_timestep_module.f90:164-180)
   followed by TRC_timestep (tracer_module.f90:109-123) when tracers exist */
int swm_gpu_step(swm_gpu_ctx *ctx, int64_t itt);
/* model_advance (model.f90:238-259): SWM_advance (swm_module.f90:86-139) and
   TRC_advance (tracer_module.f90:133-146) */
int swm_gpu_advance(swm_gpu_ctx *ctx, int64_t itt);
/* nsteps iterations of step+advance for itt = itt0+1 .. itt0+nsteps with no
   time-dependent file forcing in between.  From itt = 3 on, without tracers
   or oscillating forcing, blocks of six steps replay one captured CUDA graph
   (bit-identical to single steps) */
int swm_gpu_run(swm_gpu_ctx *ctx, int64_t itt0, int64_t nsteps);

/* nsteps monitored steps (itt0+1 .. itt0+nsteps) issued without a host wait
   per step: before step s the row profile rows1 + s*Ny (and rows2 + s*Ny for
   a second component, may be NULL) of stream stream_id goes to the device
   as swm_gpu_set_stream_rows does (rows1 NULL: no upload); after it the
   three domain integrals of swm_gpu_integrals go to out3 + 3*s.  Returns
   when the last result has landed; the arrays must stay untouched until
   then.  On the FP32 pair path with pinned (mapped) arrays each step is one
   kernel launch that reads its rows and writes its integrals in place; the
   integrals are then summed inside the step kernel, in another order than
   swm_gpu_integrals (agreement about 1e-13 relative).  Other paths and
   arrays take staged copies and the reduction of swm_gpu_integrals. */
int swm_gpu_run_monitor(swm_gpu_ctx *ctx, int64_t itt0, int64_t nsteps, int stream_id, const double *rows1,
                        const double *rows2, double *out3);

/* ---- host access (the registry pointers the diagnostics read) ---- */
int swm_gpu_get_field(swm_gpu_ctx *ctx, int field, double *host_out);
/* swm_gpu_set_field: the state (u, v, eta) at any time; static fields
   (depths, damping and drag factors, constant forcing, basic state) at any
   time on the plain path, and before the first step on the fused paths
   (SWM_GPU_EINVAL afterwards: those paths keep their own copies). */
int swm_gpu_set_field(swm_gpu_ctx *ctx, int field, const double *host_in);
/* Output without stalling the time loop (for a writer thread; the reference
   writes its diagnostics synchronously, io_module.f90:504-529): the copy of
   the field as of this point of the stream goes into host_out (pinned memory
   lets it overlap the following steps), and *ticket names it.  The buffer
   must stay valid until swm_gpu_wait(ticket) returns; swm_gpu_ready returns
   1 when done, 0 when not yet, -1 on error.  Tickets older than the last 64
   wait for a later copy. */
int swm_gpu_get_field_async(swm_gpu_ctx *ctx, int field, double *host_out, int64_t *ticket);
int swm_gpu_wait(swm_gpu_ctx *ctx, int64_t ticket);
int swm_gpu_ready(swm_gpu_ctx *ctx, int64_t ticket);
/* Page-lock (pin) a host array the caller owns, and release it: a pinned
   destination lets swm_gpu_get_field_async overlap the following steps.  A
   Fortran host pins its output arrays once (c_loc, size in bytes); the
   Python host's asynchronous writer pins its buffer pool.  Wait for every
   copy into the array before unpinning it.  Tickets and pinned arrays may
   be used from a writer thread while the host thread steps the model: the
   library's calls are thread-safe for one context as long as only one
   thread issues work on it. */
int swm_gpu_host_register(void *host, int64_t bytes);
int swm_gpu_host_unregister(void *host);
/* 1-D metric: which = 0 lat, 1 cos, 2 tan, 3 f; grid = 0 H, 1 u, 2 v, 3 eta */
int swm_gpu_get_metric(swm_gpu_ctx *ctx, int which, int grid, double *host_out);
int swm_gpu_get_mask(swm_gpu_ctx *ctx, int grid, int8_t *host_out);
/* computeStreamfunction (calc_lib.f90:727-780) of the current u, v, formed
   on the device in the reference's summation order */
int swm_gpu_streamfunction(swm_gpu_ctx *ctx, double *psi_out);
/* Time averaging of diagTask (diagTask.f90:266-338) on the device: add
   weight * field (square = 1: field^2) to the FP64 buffer of slot and weight
   to its count; swm_gpu_diag_mean returns buffer / count (and the count),
   then clears the slot.  One device field read per call, no host copy until
   the mean. */
int swm_gpu_diag_accumulate(swm_gpu_ctx *ctx, int slot, int field, int square, double weight);
int swm_gpu_diag_mean(swm_gpu_ctx *ctx, int slot, double *host_out, double *count_out);
/* Domain integrals of the current state over ocean points, each point
   weighted by the cell area A^2 cos(lat) dLambda dTheta at its own latitude
   (eta and u points: the eta rows; v points: the v rows).  FP64 state:
   summed in FP64; FP32 pair state: summed in (hi, lo) binary32 pairs (about
   46 bits) and combined in FP64:
   out[0] = volume anomaly sum(eta * area), out[1] = sum(0.5 G eta^2 area),
   out[2] = sum(0.5 u^2 area) over u points + sum(0.5 v^2 area) over v points.
   No counterpart in the reference (its diagnostics write fields only); this
   is the per-step scalar a monitoring loop reads back (16-24 bytes D2H). */
int swm_gpu_integrals(swm_gpu_ctx *ctx, double *out3);
/* The same sums copied into out3 (pinned host memory, valid until the
   ticket is waited on) without waiting: collect with swm_gpu_wait(ticket),
   so a monitoring loop can issue the next step first */
int swm_gpu_integrals_async(swm_gpu_ctx *ctx, double *out3, int64_t *ticket);
/* The same three integrals, bit for bit, computed without allocating any
   memory (no device, pinned or library allocation): all scratch is one fixed
   array inside the library, for hosts that cannot allocate inside their time
   loop (device memory fully reserved by their own pool, or other streams
   that an implicit device synchronisation of cudaMalloc/cudaFree would
   stall).  No counterpart in the reference.  Grids of at most
   SWM_NOALLOC_MAX_NY rows (SWM_GPU_EINVAL beyond).  The first call on a
   device looks up the array's device address; make that first call before
   any stream capture.  Every call waits on the context's stream for its
   result, so it is never valid on a stream under capture: it returns
   SWM_GPU_EINVAL there.  The array is shared by all contexts on a device:
   calls that overlap in time on one device race and must be serialised. */
#define SWM_NOALLOC_MAX_NY 8192
int swm_gpu_integrals_noalloc(swm_gpu_ctx *ctx, double *out3);

/* ---- ensemble of basins (extension; the reference runs one basin per
   process) ----
   Members are contexts created and initialised through the calls above on
   SWM_PATH_FUSED_FP32C, without tracers, sharing the lateral-mixing kind and
   the current step.  swm_gpu_ensemble_run steps all of them with one
   persistent launch per step that takes (member, strip, row group) tiles
   from a device queue; from itt = 3 on, blocks of six steps replay a CUDA
   graph.  Members stay usable through their own contexts between runs
   (get_field etc.).  The ensemble does not own the members: destroy it
   before them. */
typedef struct swm_gpu_ensemble swm_gpu_ensemble;
int swm_gpu_ensemble_create(swm_gpu_ctx *const *members, int n, swm_gpu_ensemble **out);
int swm_gpu_ensemble_destroy(swm_gpu_ensemble *ens);
/* steps itt0+1 .. itt0+nsteps of every member (SWM_timestep + model_advance) */
int swm_gpu_ensemble_run(swm_gpu_ensemble *ens, int64_t itt0, int64_t nsteps);
/* FP64 domain integrals of every member, 3 per member as swm_gpu_integrals */
int swm_gpu_ensemble_integrals(swm_gpu_ensemble *ens, double *out);
/* nsteps monitored steps of every member (itt0+1 .. itt0+nsteps) issued
   without a host wait per step, the batched form of swm_gpu_run_monitor:
   before step s, the row profiles rows + s*R (R = the sum of the members'
   Ny; member i's Ny rows follow those of members 0 .. i-1) become the
   members' zonal wind-stress rows (one H2D copy; rows may be NULL: no
   update; otherwise every member needs a time-dependent row-profile zonal
   wind stream); after it, the three integrals of swm_gpu_integrals of every
   member go to out + 3*n*s + 3*i (one D2H copy).  From itt = 3 on the step
   kernel forms the sums itself, in (hi, lo) binary32 pairs per tile added
   in FP64 in a fixed order (agreement with swm_gpu_ensemble_integrals about
   1e-13 relative); the start-up steps use swm_gpu_ensemble_integrals.
   Returns when the last result has landed; pinned arrays let the copies
   run asynchronously, and they must stay untouched until then. */
int swm_gpu_ensemble_run_monitor(swm_gpu_ensemble *ens, int64_t itt0, int64_t nsteps, const double *rows,
                                 double *out);
int swm_gpu_ensemble_synchronize(swm_gpu_ensemble *ens);
void *swm_gpu_ensemble_stream(swm_gpu_ensemble *ens);
int64_t swm_gpu_ensemble_launch_count(swm_gpu_ensemble *ens);
/* rows per warp strip the ensemble picked by timing its step */
int swm_gpu_ensemble_rows(swm_gpu_ensemble *ens);

/* ---- tracer (tracer_vars.f90:124-185, tracer_module.f90:58-342) ---- */
int trc_gpu_add(swm_gpu_ctx *ctx, double kappa_h, double cons, double gamma_c, const double *C,
                const double *C0, const double *gamma_field, const double *cons_field, int *id);
int trc_gpu_init(swm_gpu_ctx *ctx);   /* TRC_initCoeffs (tracer_module.f90:291-342) */
enum { TRC_F_CH, TRC_F_C, TRC_F_G, TRC_F_UHC, TRC_F_VHC, TRC_F_DIFF, TRC_F_IMPL };
int trc_gpu_get_field(swm_gpu_ctx *ctx, int tracer, int field, double *host_out);

/* ---- red-black SOR (ElSolv_SOR.f90) ---- */
int elsolv_sor_gpu_init(swm_gpu_ctx *ctx);   /* init_ElSolv_SOR (:44-66) */
/* main_ElSolv_SOR (:150-222); returns SWM_GPU_ENOT_CONVERGED when max_count
   sweeps did not bring the correction norm below eps */
int elsolv_sor_gpu_solve(swm_gpu_ctx *ctx, const double *B, double *chi, double eps, int first_guess,
                         int *iterations, double *anorm);
/* computeNonDivergentFlowField (calc_lib.f90:548-590) of the current model
   velocities on the device: computeDivergence (:607-622), main_ElSolv_SOR
   for chi (kept on the device between calls, like calc_lib::chi;
   first_guess = itt == 1; eps = EPS of calc_lib.h, 1e-4), computeGradient
   (:638-648); u_nd = u - d chi / (A cos dLambda), v_nd = v - d chi / (A
   dTheta).  Outputs may be NULL. */
int swm_gpu_nondivergent(swm_gpu_ctx *ctx, int first_guess, double eps, double *u_nd, double *v_nd, double *chi,
                         int *iterations);
/* Self-check of the division by a fixed divisor that the SOR half-sweep
   and the plain path use (a / b formed from the reciprocal of b by two
   Markstein corrections, other numerators by exact branches) against the
   division operator, on n pseudo-random pairs from seed: divisors over the
   exponent range it is used for, special significands and numerators
   outside that range included; *mismatches counts the pairs whose quotients
   differ in any bit (two NaNs count as equal).  Runs on the current device
   and waits. */
int swm_gpu_check_division(int64_t n, int64_t seed, int64_t *mismatches);

/* ---- variable-coefficient Helmholtz solver (extension of ElSolv_SOR) ----
   div(H^-1 grad psi) - lambda psi = rhs on an (nx, ny) grid of spacing dx,
   dy; a face coefficient is the mean of 1/H of its two cells over dx^2 (dy^2);
   cells with ocean == 0 hold psi = 0, and so does everything beyond the
   outer frame.  Red-black sweeps in the reference's colour order; stopping
   on the relative residual ||rhs - A psi|| / ||rhs||, checked every 16
   sweeps.  The reference's own solver (elsolv_sor_gpu_*) keeps its operator,
   relaxation schedule and absolute stopping rule. */
typedef struct swm_helm swm_helm;
int swm_helm_create(int nx, int ny, double dx, double dy, double lambda, const double *H, const int8_t *ocean,
                    swm_helm **out);
int swm_helm_destroy(swm_helm *h);
void *swm_helm_stream(swm_helm *h);
int64_t swm_helm_launch_count(swm_helm *h);
/* out = A psi on ocean cells, 0 elsewhere */
int swm_helm_apply(swm_helm *h, const double *psi, double *out);
/* FP64 sweeps; SWM_GPU_ENOT_CONVERGED when rtol is not reached in max_sweeps */
int swm_helm_solve_fp64(swm_helm *h, const double *rhs, double *psi, double omega, double rtol, int max_sweeps,
                        int *sweeps, double *relres);
/* FP32 sweeps on the correction equation, FP64 residual and accumulation
   (iterative refinement); each correction solve stops when its own residual
   has fallen by inner_tol */
int swm_helm_solve_mixed(swm_helm *h, const double *rhs, double *psi, double omega, double rtol, double inner_tol,
                         int max_sweeps, int *sweeps, int *outer, double *relres);
/* block shape of the sweep kernel by timing, and the relaxation factor in
   [omega_lo, omega_hi] (ngrid values) by trial solves of trial_sweeps */
int swm_helm_autotune(swm_helm *h, const double *rhs, double omega_lo, double omega_hi, int ngrid,
                      int trial_sweeps, double *omega, int *block_x, int *block_y);

#ifdef __cplusplus
}
#endif
#endif
