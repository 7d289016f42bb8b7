/*
 * gpmood_oracle.h -- CPU restatement of the GP-MOOD per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the CUDA path: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
 * may load it.  The product library (libgpmood) never links or calls it.
 *
 * Parity status: pinned to the reference's own recorded outputs.  No
 * Fortran compiler exists on either machine, but the reference's deprecated
 * code line recorded final states of real runs
 * (deprecated/plotter_revision/{2DRP_C3,Isentropic}/).  With that line's
 * Setdt and slow start (the setdt_kind / slow_start knobs below; its solver
 * step is gp-mood-code's), the restatement reproduces the 2DRP3 runs at 200^2
 * and 400^2 -- R1 and R2 GP, POL_MOOD, SSP-RK3 and SSP-RK4, 487 to 1037 steps
 * with MOOD active -- bit for bit with the same step counts, and the
 * isentropic-vortex runs from their recorded initial states to 1e-15
 * relative L1 (tests/test_reference_pins.py).  Further checks: the
 * reference's GP inversion self-check (gp-mood-code/GP_init.f90:250) and an
 * independent arbitrary-precision (mpmath) recomputation of every GP weight.
 *
 * Layout follows the reference: U(4, lb:le, nb:ne), variable fastest
 * (gp-mood-code/global_variables.f90:26), lb = 1-ngc, le = lf+ngc, ngc = 4.
 */
#ifndef GPMOOD_ORACLE_H
#define GPMOOD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Knobs of the reference's parameters.f90 (problems/sedov_GPMOOD.f90:8-46). */
typedef struct orc_params {
    double cfl;        /* CFL */
    double ell_o_dx;   /* GP length scale over dx */
    double lx, ly;     /* domain size, mesh starts at 0 (mesh_init.f90:14-20) */
    double tmax;
    int mord;          /* 1, 3 or 5 */
    int ngp;           /* Gauss points per face, 1..5 */
    int method;        /* 1 = FOG (ngp 1), 2 = GP_MOOD, 202 = GP_SE, 200 = POL_MOOD, 201 = Unlim_POL
                          (constants.f90:17);
                          POL_MOOD/Unlim_POL need mord 3 and ngp 2 */
    int dmp, u2, u2_tol;
    int lf, nf;        /* interior cells */
    int bc_type;       /* 17 Neumann, 18 Periodic, 20 Reflective, 35 DMR */
    int integrator;    /* 8 FE, 9 SSP_RK2, 10 SSP_RK3 (default for 0), 12 SSP_RK4 (constants.f90:19) */
    int num_flux;      /* 100 HLLC (default for 0), 101 LLF, 102 HLL, 103 unsplit (constants.f90:21) */
    /* Knobs of the deprecated code line, which recorded the reference's only
     * per-cell output snapshots (deprecated/plotter_revision/Isentropic/);
     * all zero = gp-mood-code's behaviour. */
    int setdt_kind;    /* 0: physics.f90:110, dt = min 1/(1/(dx/(|u|+c)) + 1/(dy/(|v|+c)));
                          1: deprecated/physics.f90:106-118, dt = min(dx/(|u|+c), dy/(|v|+c)) */
    int lf0, nf0;      /* deprecated dt_reduction base grid (deprecated/physics.f90:94-126); 0 = off */
    double slow_start; /* deprecated/main.f90 slow start: the first steps take dt_sim, which starts
                          at min(slow_start, 1e30) and doubles each step while it is below the CFL dt;
                          0 = off */
    int csd_kind;      /* shock detector gating the DMP test: 0 mod_subroutine_MOOD.f90:231
                          (divV < -max(dx,dy)^2, Mach > 0.2, gradP > 5); 1 the deprecated line's
                          "old CSD" (deprecated/mod_subroutine_MOOD.f90:104, divV < -5, gradP > 5);
                          2 none (the DMP test on every checked cell, the "noCSD" runs) */
} orc_params;

/* GP weights as produced by GP_presim_sphere (GP_init.f90:26-357).
 * zt[o][face][g][k]: o = 0,1,2 for ord = 1,3,5; face = iL,iT,iR,iB - 1;
 * g < ngp; k < stencil size of ord.  d2x/d2y are the ord=3 second-derivative
 * weights (GP_init.f90:267-268).  inv_err[o] is the inversion self-check. */
typedef struct orc_gp {
    double zt[3][4][5][13];
    double d2x[5], d2y[5];
    double gauss_w[5];
    double inv_err[3];
    int ixiy[13][2];
} orc_gp;

int  orc_gp_presim(const orc_params* p, orc_gp* out);

/* Physics kernels (physics.f90, mod_HLLC.f90). */
void orc_hllc(const double ul[4], const double ur[4], int dir, double F[4]);
void orc_hll(const double ul[4], const double ur[4], int dir, double F[4]);
void orc_llf(const double ul[4], const double ur[4], int dir, double F[4]);
void orc_unsplit(const double ul[4], const double ur[4], int dir, double F[4]);
double orc_pressure(const double u[4]);

/* Boundary_C (BC.f90:10-135, 283-341) on a full padded array. */
void orc_boundary(const orc_params* p, double* U, double t_rk);

/* Setdt (physics.f90:78-129): returns dt for the given dtfinal. */
double orc_setdt(const orc_params* p, const double* U, double dtfinal);

/* Stepping context: owns the reference's module-global work arrays. */
typedef struct orc_ctx orc_ctx;
orc_ctx* orc_create(const orc_params* p);
void     orc_destroy(orc_ctx* c);
const orc_gp* orc_weights(const orc_ctx* c);

/* time_stepping(Uin, Uout) with SSP-RK3 (time_stepper.f90:12, mod_SSP_RK3.f90:12-39).
 * Uin is inout (ghosts are refilled in place, as the reference does).
 * init_orders: NULL for plain GP-MOOD, else 3 arrays (one per RK stage) of
 *   lf*nf int8 starting orders for interior cells (a-priori gate).
 * stage_orders: NULL or 3 arrays of lf*nf int8 that receive CellGPO after each
 *   stage's MOOD loop.
 * counters[0..2]: detected cells, MOOD passes (all stages), max passes per stage. */
int orc_time_stepping(orc_ctx* c, double* Uin, double* Uout, double t, double dt,
                      const signed char* const* init_orders,
                      signed char* const* stage_orders, long long* counters);

/* One Forward_Euler stage (mod_FE.f90:20-190); exposed for unit tests. */
/* NN_GP_MOOD_CC_ reconstruction: blend column col with the row pairs
 * w[2n..2n+1], n = 0..nf+1 (copied); w = NULL switches it off. */
void orc_set_cc(orc_ctx* c, int col, const float* w);
int orc_forward_euler(orc_ctx* c, double* Uin, double* Uout, double dt, double t_rk,
                      const signed char* init_order, signed char* final_order,
                      long long* counters);

/* DETECTION building blocks for unit tests (mod_subroutine_MOOD.f90). */
int orc_shock_detector(const orc_params* p, const double* Uin, int l, int n);

/* Initial conditions over lb..lf x nb..nf (IC.f90:29-30), followed by Boundary_C. */
void orc_ic_rp2d3(const orc_params* p, double* U);
void orc_ic_sedov(const orc_params* p, double* U);
void orc_ic_dmr(const orc_params* p, double* U);
void orc_ic_vortex(const orc_params* p, double* U);

/* Full run: the main.f90:145-203 loop for at most nsteps steps (or to tmax).
 * Returns steps taken; *t_io holds t in/out. */
int orc_run(orc_ctx* c, double* U, double* t_io, int nsteps, long long* counters);

/* Number of OpenMP threads the oracle uses (1 without OpenMP), and a setter. */
int orc_num_threads(void);
void orc_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
