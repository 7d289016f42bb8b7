/*
 * gpmood.h -- C ABI of the GB300 GP-MOOD step library (libgpmood.so).
 *
 * One SSP-RK3 step of GP-MOOD for the 2-D compressible Euler equations:
 * GP-SE reconstruction (radius 2 -> 1 -> first order), HLLC face fluxes with
 * Gauss quadrature, a-posteriori MOOD detection with its order cascade, and
 * the CFL time step, all in FP64 on one GPU.
 *
 * The entry points replace the reference's Fortran subroutines one for one:
 *   gpmood_time_stepping  <- time_stepping(Uin, Uout)   gp-mood-code/time_stepper.f90:12-23
 *   gpmood_setdt          <- Setdt(Uin)                 gp-mood-code/physics.f90:78-129
 *   gpmood_boundary_c     <- Boundary_C(U)              gp-mood-code/BC.f90:10-421
 *   gpmood_create         <- GP_presim_sphere() + init_mesh()
 *                                                       gp-mood-code/GP_init.f90:26-357,
 *                                                       gp-mood-code/mesh_init.f90:10-20
 *   gpmood_advance        <- the main.f90:145-203 time loop (device-resident state)
 *   gpmood_params         <- the parameters.f90 knobs   gp-mood-code/problems/sedov_GPMOOD.f90:8-46
 *
 * Arrays cross the ABI in the reference's layout U(4, lb:le, nb:ne): the
 * variable index (rho, rho*u, rho*v, E) is fastest, then x, then y, with
 * ngc = 4 ghost layers (lb = 1-ngc, le = lf+ngc).  That is
 * 4*(lf+8)*(nf+8) doubles.
 *
 * Conventions: every int-returning call returns 0 on success or a negative
 * GPMOOD_E* code; gpmood_last_error() gives the message.  The library never
 * keeps a host pointer after a call returns.  One context per host thread;
 * each context owns one CUDA stream and all calls on it are synchronous at
 * return.  There is no CPU fallback: without a usable GPU gpmood_create
 * fails with GPMOOD_E_CUDA.
 */
#ifndef GPMOOD_H
#define GPMOOD_H

#ifdef __cplusplus
extern "C" {
#endif

/* Enumerations share the reference's values (gp-mood-code/constants.f90:17-34). */
#define GPMOOD_FOG         1     /* method: first-order Godunov (mod_FOG.f90); ngp 1 */
#define GPMOOD_GP_MOOD     2     /* method: GP-MOOD */
#define GPMOOD_GP_SE       202   /* method: unlimited GP (MOOD off) */
#define GPMOOD_NN_GP_MOOD  203   /* method: GP-MOOD with the MLP a-priori gate */
#define GPMOOD_POL_MOOD    200   /* method: MOOD with the third-order polynomial reconstruction
                                    (mod_pol_MOOD.f90, pol_presim); Mord 3, ngp 2 */
#define GPMOOD_UNLIM_POL   201   /* method: the same polynomial reconstruction without MOOD
                                    (mod_Unlim_Pol.f90); Mord 3, ngp 2 */
#define GPMOOD_NN_GP_MOOD_CC 204 /* method: the reference's network with its convex-combination
                                    reconstruction (mod_NN_GP_MOOD_CC.f90); Mord 3 */
#define GPMOOD_FE          8     /* integrator: Forward_Euler */
#define GPMOOD_SSP_RK2     9
#define GPMOOD_SSP_RK3     10
#define GPMOOD_SSP_RK4     12
#define GPMOOD_HLLC        100   /* numFlux */
#define GPMOOD_LLF         101
#define GPMOOD_HLL         102
#define GPMOOD_UNSPLIT     103
#define GPMOOD_NEUMANN     17    /* BC_type */
#define GPMOOD_PERIODIC    18
#define GPMOOD_REFLECTIVE  20
#define GPMOOD_DMR         35
#define GPMOOD_DIRICHLET   19    /* Shu-Osher inflow/outflow states (BC.f90:61-87) */
#define GPMOOD_MACH800     201   /* outflow, jet at 0.70 <= x <= 0.80 on y = 0 (BC.f90:137-179) */
#define GPMOOD_DOUBLE_MACH800 301 /* jets on y = 0 and y = Ly (BC.f90:181-237) */
#define GPMOOD_RMI         401   /* inflow left, outflow right, reflective top/bottom (BC.f90:239-281) */
#define GPMOOD_RT          402   /* reflective, hydrostatic ghosts in y, g = 0.1 (BC.f90:343-390) */
#define GPMOOD_KH          403   /* periodic in x, Neumann in y (BC.f90:392-414) */

/* Floating-point modes of the kernels. */
#define GPMOOD_FP_EXACT    0     /* reference operation order, no FMA contraction:
                                    bit-identical to the CPU restatement */
#define GPMOOD_FP_FAST     1     /* FMA contraction and reciprocal reuse */

/* Error codes. */
#define GPMOOD_OK           0
#define GPMOOD_E_ARG       -1    /* invalid argument or unsupported knob */
#define GPMOOD_E_CUDA      -2    /* CUDA runtime error (no GPU, OOM, launch failure) */
#define GPMOOD_E_MOOD_CAP  -3    /* MOOD loop exceeded max_mood_iters in a stage */
#define GPMOOD_E_DT        -4    /* time step not finite or not positive */
#define GPMOOD_E_STATE     -5    /* call order violated (e.g. no state set) */

/* Knobs of parameters.f90 (same names and meaning), plus GB300 run options. */
typedef struct gpmood_params {
    double cfl;           /* CFL                                      :8  */
    double ell_o_dx;      /* GP length scale in cells                  :14 */
    double lx, ly;        /* domain [0,Lx]x[0,Ly] (Lx_16, Ly_16)       :43-44 */
    double tmax;          /* final time                                :41 */
    int integrator;       /* GPMOOD_FE, _SSP_RK2, _SSP_RK3, _SSP_RK4   :9  */
    int method;           /* GPMOOD_FOG, GPMOOD_GP_MOOD, GPMOOD_POL_MOOD, GPMOOD_UNLIM_POL, GPMOOD_GP_SE,
                             GPMOOD_NN_GP_MOOD, GPMOOD_NN_GP_MOOD_CC */
    int mord;             /* maximal order 1, 3 or 5                   :15 */
    int ngp;              /* Gauss points per face, 1..5               :16 */
    int dmp, u2, u2_tol;  /* MOOD checks (logical -> 0/1)              :18-20 */
    int num_flux;         /* GPMOOD_HLLC, _LLF, _HLL, _UNSPLIT         :30 */
    int lf, nf;           /* interior cells in x and y                 :37-38 */
    int bc_type;          /* GPMOOD_NEUMANN/PERIODIC/REFLECTIVE/DMR/DIRICHLET/MACH800/
                             DOUBLE_MACH800/RMI/RT/KH                    :45 */
    int nmax;             /* step cap of the time loop                 :42 */
    int fp_mode;          /* GPMOOD_FP_EXACT or GPMOOD_FP_FAST */
    int max_mood_iters;   /* MOOD passes allowed per stage before GPMOOD_E_MOOD_CAP; 0 (default)
                             allows 2*lf*nf+2, more than a terminating loop can take */
    int nsteps_with_no_nn;/* gate off for the first steps (global_variables.f90:97) */
    int nn_reference;     /* method NN_GP_MOOD: 0 the BF16 36-64-64-1 gate (default);
                             1 the reference's own network and NN_DETECTION (mod_NN.f90:14-58,
                             mod_subroutine_NN_MOOD.f90): FP32 sigmoid MLP on the raw R+1
                             stencil, CellGPO 1 or 3, a-posteriori NaN/positivity checks only */
} gpmood_params;

/* Per-step and cumulative counters (global_variables.f90:71, main.f90:165-167). */
typedef struct gpmood_counters {
    long long detected_last_step;   /* count_detected_cell of the last step */
    long long detected_total;       /* summed over all steps */
    long long a_priori_last_step;   /* cells started at reduced order by the gate */
    long long mood_passes_last_step;/* passes summed over the 3 stages */
    long long max_passes_stage;     /* worst stage since create */
    long long steps;                /* steps taken through this context */
    long long status_flags;         /* OR of every step's flags.  bit 0: NaN/inadmissible
                                       state left in an order-1 cell (reported, the step
                                       still succeeds, as in the reference); bit 1: MOOD cap
                                       hit; bit 2: bad dt; bit 3: grid-barrier timeout;
                                       bit 4: tensor-core wait timeout; bit 5: TMA tile
                                       copy wait timeout */
    long long kernel_launches;      /* kernels launched through this context */
} gpmood_counters;

/* Per-kernel device time gathered with CUDA events when timing is on. */
typedef struct gpmood_timing {
    double flux_ms;          /* first-pass face kernels (GP recon + HLLC), all stages */
    long long flux_launches; /* first passes timed: one per RK stage (its face kernels) */
    long long flux_faces;    /* faces computed by those passes */
    double update_ms;        /* flux-difference update + DETECTION kernels */
    long long update_launches;
    double mood_ms;          /* MOOD passes 2, 3, ... (mark + faces + cells) */
    long long mood_passes;   /* passes 2, 3, ... run, all stages */
} gpmood_timing;

typedef struct gpmood_ctx gpmood_ctx;

/* Fill the reference defaults: CFL 0.8, SSP-RK3, GP-MOOD, ell/dx 12, Mord 5,
 * ngp 3, DMP/U2/U2_tol on, HLLC, 256x256 on [0,1]^2, Neumann, tmax 0.8. */
int  gpmood_default_params(gpmood_params* p);

/* Validate the knobs, run the GP weight precompute (host, binary128) and
 * allocate the device work arrays on the current CUDA device. */
int  gpmood_create(const gpmood_params* p, gpmood_ctx** out);
void gpmood_destroy(gpmood_ctx* ctx);

/* Last error message of ctx (or of the thread when ctx is NULL). */
int  gpmood_last_error(const gpmood_ctx* ctx, char* buf, int len);

/* The GP weights in use: zt[3][4][ngp][13] for ord 1,3,5 and faces iL,iT,iR,iB;
 * d2[2][5] = (GP_d2x_sp, GP_d2y_sp) of ord 3; inv_err[3] = GP_init.f90:250 check. */
int  gpmood_get_weights(const gpmood_ctx* ctx, double* zt, double* d2, double* inv_err);

/* GP_presim_sphere alone (GP_init.f90:26-357): the same weights for a set of
 * knobs, computed on the host without touching a GPU. */
int  gpmood_gp_weights(const gpmood_params* p, double* zt, double* d2, double* inv_err);

/* ---- reference-facing calls on host arrays (Fortran layout) ---- */

/* Boundary_C(U): refill the ghost layers of a host array in place. */
int  gpmood_boundary_c(gpmood_ctx* ctx, double* u_host, double t_rk);

/* Setdt(U) with dtfinal = tmax - t: dt over all cells including ghosts. */
int  gpmood_setdt(gpmood_ctx* ctx, const double* u_host, double dtfinal, double* dt_out);

/* time_stepping(Uin, Uout): one SSP-RK3 step at time t with step dt.
 * The reference refills the ghost layers of Uin in place; its caller then
 * overwrites Uin with Uout (main.f90:162), so uin_host is left untouched here. */
int  gpmood_time_stepping(gpmood_ctx* ctx, const double* uin_host, double* uout_host,
                          double t, double dt);

/* Setdt(U) then time_stepping(U, Uout) (main.f90:151-155) in one call: U
 * crosses to the GPU once and Uout once back, *dt_out receives the step
 * taken.  Same results as gpmood_setdt + gpmood_time_stepping on the same
 * arrays (same kernels on the same data). */
int  gpmood_setdt_time_stepping(gpmood_ctx* ctx, const double* uin_host, double* uout_host,
                                double t, double dtfinal, double* dt_out);

/* ---- device-resident stepping ---- */

/* Upload a state (Fortran layout) and the time; resets the step counter. */
int  gpmood_set_state(gpmood_ctx* ctx, const double* u_host, double t);
/* Download state, time and step count (any pointer may be NULL). */
int  gpmood_get_state(gpmood_ctx* ctx, double* u_host, double* t, int* niter);
/* The same two calls with a device array (padded layout) in place of the host one. */
int  gpmood_set_state_dev(gpmood_ctx* ctx, const double* d_u, double t);
int  gpmood_get_state_dev(gpmood_ctx* ctx, double* d_u);
/* CellGPO(1:lf,1:nf) after the last stage ("ordr" of output.f90:128), x fastest. */
int  gpmood_get_orders(gpmood_ctx* ctx, signed char* orders);
/* The main.f90 loop: up to nsteps steps of Setdt + time_stepping + t += dt,
 * stopping at tmax; *steps_done receives the steps taken (may be NULL). */
int  gpmood_advance(gpmood_ctx* ctx, int nsteps, int* steps_done);
int  gpmood_get_counters(const gpmood_ctx* ctx, gpmood_counters* out);

/* The gate's extras repair (BF16 gate, method NN_GP_MOOD with nn_reference 0);
 * no counterpart in the reference.  With on != 0, a cell the gate starts at
 * Mord-2 whose update from the uniform first pass passes DETECTION gets Mord
 * back before the stage continues: only cells that plain MOOD's first
 * DETECTION also flags start lowered, trading the gate's saved passes for a
 * solution closer to plain GP-MOOD.  Off by default. */
int  gpmood_set_nn_repair(gpmood_ctx* ctx, int on);

/* Test hook for the failure paths; no counterpart in the reference.  Every
 * spin-wait of the context's kernels is bounded (the grid barrier of the
 * cooperative MOOD loop, the gate's tensor-core MMA waits): after ~1 s a wait
 * gives up, sets a status bit (3 or 4 of gpmood_counters.status_flags) and the
 * step fails with GPMOOD_E_CUDA, leaving the context usable.  This call bounds
 * those waits to `polls` polls instead, so that a test can make them run out
 * without a faulty GPU; 0 restores the default.  The gate frees its tensor
 * memory only after the MMAs in flight have landed. */
int  gpmood_set_wait_limit(gpmood_ctx* ctx, int polls);

/* One step on device arrays (padded layout) on the context's stream; d_uin is
 * inout (its ghosts are refilled, as in the reference).  For callers that keep
 * the state on the GPU. */
int  gpmood_time_stepping_dev(gpmood_ctx* ctx, double* d_uin, double* d_uout,
                              double t, double dt);

/* One SSP-RK3 step that allocates no memory; it has no counterpart in the
 * reference.  For callers that cannot let a library allocate GPU memory: a
 * host that manages all device memory through its own pool, or a real-time
 * loop that must not stall in cudaMalloc.  d_uin (inout: ghosts refilled) and
 * d_uout are the caller's device arrays in the padded layout; every scratch
 * array lives in a static device buffer of ~10 MB that every GPU loading the
 * library holds until exit, so grids are limited to (lf+8)*(nf+8) <= 264*264
 * (GPMOOD_E_ARG beyond that).  The knobs are checked as gpmood_create checks
 * them; method GP_MOOD or GP_SE, SSP-RK3, Neumann, periodic, reflective or
 * DMR boundaries.  The first call on a device (and in each new CUDA context
 * on it) looks up that buffer's address, so make it before any stream
 * capture.  All calls share the buffer: calls that overlap on the GPU race.
 * stream is a cudaStream_t (NULL = legacy default stream); the call is
 * synchronous at return.  *status (may be NULL) receives the step's status
 * bits, those of gpmood_counters.status_flags: bit 0 (a NaN or inadmissible
 * state left in an order-1 cell) leaves the call successful, as in the
 * reference; a MOOD cap (bit 1) returns GPMOOD_E_MOOD_CAP after the whole step
 * ran, as gpmood_time_stepping does.  Errors: gpmood_last_error(NULL, ...). */
int  gpmood_time_stepping_noalloc(const gpmood_params* p, double* d_uin, double* d_uout,
                                  double t, double dt, void* stream, int* status);

/* ---- many independent problems of uneven size (one GPU) ---- */

/* No counterpart in the reference (which runs one problem per process).  A
 * batch steps nprob problems that share the knobs of p (method GP_MOOD or
 * GP_SE; Neumann, periodic or reflective BCs), problem i on lf[i] x nf[i]
 * cells of [0,Lx]x[0,Ly], each with its own CFL time step.  Every phase of an
 * RK stage is one persistent launch over all problems and the MOOD loop one
 * cooperative launch per stage; a step is replayed from a CUDA graph. */
typedef struct gpmood_batch gpmood_batch;
int  gpmood_batch_create(const gpmood_params* p, int nprob, const int* lf, const int* nf,
                         gpmood_batch** out);
void gpmood_batch_destroy(gpmood_batch* b);
/* Problem i's state, Fortran layout of (lf[i]+8)*(nf[i]+8)*4 doubles, and time. */
int  gpmood_batch_set_state(gpmood_batch* b, int i, const double* u_host, double t);
int  gpmood_batch_get_state(gpmood_batch* b, int i, double* u_host, double* t);
/* nsteps steps of every problem (Setdt + time_stepping + t += dt each). */
int  gpmood_batch_advance(gpmood_batch* b, int nsteps);
/* Time each face-tile shape on this batch and keep the fastest: *tile gets its
 * index, ms_per_tile[5] (may be NULL) the measured times.  Shapes 0-3 are
 * one-direction face tiles (32x8, 32x4, 16x16, 64x4); shape 4 is the fast
 * mode's two-direction cell tile (order 5, ngp 3 only; time 0 otherwise),
 * which is also the default there. */
int  gpmood_batch_autotune(gpmood_batch* b, int* tile, double* ms_per_tile);
/* Interior cells of all problems, steps taken, detected cells (all steps),
 * status bits, and 1 if steps replay a CUDA graph (-1: eager launches). */
int  gpmood_batch_stats(const gpmood_batch* b, long long* interior_cells, long long* steps,
                        long long* detected, long long* status, int* graphed);

/* ---- measurement ---- */

/* The context's cudaStream_t (as void*), for callers that time on it. */
void* gpmood_get_stream(const gpmood_ctx* ctx);
/* Turn per-kernel CUDA-event timing on (1) or off (0); on also clears it. */
int  gpmood_set_timing(gpmood_ctx* ctx, int on);
int  gpmood_get_timing(const gpmood_ctx* ctx, gpmood_timing* out);
/* FP64 FMA throughput of the current GPU in GFLOP/s (2 flops per FMA),
 * from a short dependent-chain microbenchmark; the FP64 roofline denominator. */
int  gpmood_probe_fp64(double* gflops);
/* Whether FP64 mma.sync adds to the FMA pipe: gflops3[0..2] = GFLOP/s of FMA
 * chains alone, m8n8k4 FP64 MMAs alone, and half the warps on each with equal
 * flops per half.  A mixed rate near the single ones means that the two share
 * the FP64 hardware.  Measurement only; no reference counterpart. */
int  gpmood_probe_fp64_pipes(double* gflops3);
/* The fast mode's reciprocal (Newton-Raphson from the hardware approximation)
 * on device arrays: d_y[i] = 1/d_x[i]; for testing its accuracy. */
int  gpmood_fast_rcp(const double* d_x, double* d_y, int n);
/* The fast mode's square root (from the hardware's approximate reciprocal
 * square root, one coupled Newton step and a final correction) on device
 * arrays: d_y[i] = sqrt(d_x[i]); for testing its accuracy. */
int  gpmood_fast_sqrt(const double* d_x, double* d_y, int n);

/* ---- a-priori MLP gate (method GPMOOD_NN_GP_MOOD) ---- */

/* The gate replaces compute_CellGPO_with_NN (gp-mood-code/mod_NN.f90:14-58):
 * 36 FP32 features per cell (rho, rho*u, rho*v, E on the 9-point radius-2
 * cross, each scaled by its stencil max-abs), a 36-64-64-1 MLP with ReLU and
 * a sigmoid output in BF16 with FP32 accumulation; a positive prediction starts
 * the cell at order mord-2; the a-posteriori DETECTION stays on unchanged. */

/* Load the 36-64-64-1 gate: w0[64][36], b0[64], w1[64][64], b1[64], w2[64], b2[1]
 * as one float array of 6593 values in that order (PyTorch flatten order, the
 * order of neural_network/save_NN_for_fortran.py:13-23).  With nn_reference = 1
 * the same call loads the reference's network instead: W0[len][L], b0[len],
 * W1[len][len], b1[len], W2[2][len], b2[2] with L = 52 (Mord 3) or 100
 * (Mord 5) and any hidden width len <= 128 (the file read by load_NN,
 * mod_NN.f90:60-110). */
int  gpmood_set_nn(gpmood_ctx* ctx, const float* params, int n);
/* The reference network's two outputs r(1), r(2) of every interior cell of
 * the device-resident state into d_logits[2*lf*nf] (0, 0 for constant
 * stencils); nn_reference = 1 only. */
int  gpmood_nn_ref_logits(gpmood_ctx* ctx, float* d_logits);
/* The gate's logit of every interior cell of the device-resident state into
 * d_logits[lf*nf] (0 for constant stencils; nn_reference = 0). */
int  gpmood_nn_gate_logits(gpmood_ctx* ctx, float* d_logits);
/* The gate fires when the logit exceeds this value (default 0, i.e. p > 0.5). */
int  gpmood_set_nn_threshold(gpmood_ctx* ctx, float logit_threshold);
/* Gate decision on the device-resident state: gated[lf*nf] = 1 where the cell
 * would start at reduced order (x fastest); *n_gated = their number. */
int  gpmood_nn_predict(gpmood_ctx* ctx, signed char* gated, long long* n_gated);
/* CellGPO(1:lf,1:nf) at the end of RK stage `stage` (0, 1, 2) of the last step. */
int  gpmood_get_stage_orders(gpmood_ctx* ctx, int stage, signed char* orders);
/* Features of the device-resident state into device arrays d_x[lf*nf][36] and
 * d_const[lf*nf] (1 = constant stencil, never gated). */
int  gpmood_nn_features(gpmood_ctx* ctx, float* d_x, signed char* d_const);
/* Collect training samples while stepping (mod_append_NN_dataset.f90:11-79):
 * after stage 1's MOOD loop of every step, each non-constant interior cell's
 * features go to d_x[i][36] and its label (1 if the loop lowered its order) to
 * d_y[i]; negatives are kept with probability keep_negative; d_count is a
 * device int holding the running count (samples past capacity are dropped).
 * d_x = NULL detaches. */
int  gpmood_nn_harvest(gpmood_ctx* ctx, float* d_x, float* d_y, int capacity, float keep_negative,
                       unsigned seed, int* d_count);
/* Training kernels on device arrays (BF16 operands, FP32 accumulation); stream
 * is a cudaStream_t (NULL = legacy default stream); synchronous at return. */
int  gpmood_nn_forward(const float* d_params, const float* d_x, int n, float* d_logits, void* stream);
/* Mean weighted binary cross-entropy with logits and its gradient. */
int  gpmood_nn_loss_grad(const float* d_params, const float* d_x, const float* d_y, int n,
                         float pos_weight, float* d_grad, float* d_loss, void* stream);
/* One bias-corrected Adam step (step counts from 1). */
int  gpmood_nn_adam(float* d_params, const float* d_grad, float* d_m, float* d_v, int step,
                    float lr, float beta1, float beta2, float eps, void* stream);

/* ---- adjoint of the step with frozen MOOD order masks ----
 *
 * No reference counterpart: gp-mood-code has no adjoint.  A recording holds,
 * for nsteps steps taken by gpmood_advance, every step's t and dt and the
 * padded CellGPO of its three RK stages (the frozen masks), plus a copy of the
 * state every `every` steps.  With masks and dt frozen a step is a smooth map
 * of the interior state; gpmood_adj_backward applies the transpose of its
 * Jacobian along the recorded trajectory, recomputing each segment of `every`
 * steps from its checkpoint.  Boundary types: Neumann, periodic, reflective.
 * Device arrays use the state's padded layout; ghost entries of the returned
 * adjoint are zero (stage 1 overwrites the input's ghosts).  The context must
 * outlive the recording; recording and replay leave its state untouched
 * except that recording advances it by nsteps. */
typedef struct gpmood_adjoint gpmood_adjoint;
int  gpmood_adj_record(gpmood_ctx* ctx, int nsteps, int every, gpmood_adjoint** out);
void gpmood_adj_destroy(gpmood_adjoint* a);
/* Steps recorded (fewer than asked if tmax was reached) and their t and dt
 * (arrays of at least that many doubles, or NULL). */
int  gpmood_adj_info(const gpmood_adjoint* a, int* nsteps, double* t, double* dt);
/* Padded CellGPO (ncell bytes) of RK stage `stage` of step `step`. */
int  gpmood_adj_orders(const gpmood_adjoint* a, int step, int stage, signed char* orders_host);
/* d_uN = the recorded steps applied to d_u0 with the frozen masks and dt. */
int  gpmood_adj_replay(gpmood_adjoint* a, const double* d_u0, double* d_uN);
/* d_lam0 = (d u_N / d u_0)^T d_lamN along the recorded trajectory. */
int  gpmood_adj_backward(gpmood_adjoint* a, const double* d_lamN, double* d_lam0);

#ifdef __cplusplus
}
#endif
#endif
