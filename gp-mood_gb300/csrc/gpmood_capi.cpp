// gpmood_capi.cpp -- the C ABI of libgpmood.so (declared in include/gpmood.h).
//
// Host orchestration of one SSP-RK3 step on the device.  All arrays of a
// context live in HBM for the context's lifetime; the only host<->device
// traffic of a step is the caller's own state copy (host-buffer calls) and one
// 4-byte troubled-cell count per MOOD pass.
#include <cuda_runtime.h>
#include <math.h>
#include <nvtx3/nvToolsExt.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <new>

#include "../../include/gpmood.h"
#include "gpm_common.h"
#include "nn_gate.h"
#include "nn_ref.h"

struct gpmood_ctx {
    gpmood_params p;
    GridGeom g;
    GpWeights w;
    double inv_err[3];
    const KernelTable* kt;
    cudaStream_t stream;
    size_t ncell;                 // padded cells
    double *dU, *dUr, *dU1, *dU2, *dFx, *dFy;
    int8_t* dOrder;
    unsigned* dStamp;
    int* dList[2];
    DevScalars* dSc;
    DevScalars* hSc;              // pinned mirror
    GridBar* dBar;                // barrier of the cooperative MOOD loop
    GridBar* hBar;                // pinned mirror
    int* hCount;                  // pinned troubled count
    double t;                     // host mirror of the time
    int niter;
    bool have_state;
    bool dt_pending;              // dSc->dtmin_bits holds Setdt of dU
    gpmood_counters ctr;
    NnGate* nn;                   // a-priori gate and training kernels
    NnRef* nnref;                 // the reference's own network (nn_reference = 1)
    bool cc;                      // method NN_GP_MOOD_CC (kept as NN_GP_MOOD + nn_reference + cc)
    float* dCcw;                  // NN_GP_MOOD_CC: values_NN(L, n, :) per row, 2*(nf+2) floats
    int8_t* dStageOrd;            // CellGPO at the end of each RK stage (GPM_MAXST x ncell)
    int nstages;                  // Forward_Euler calls per step: FE 1, SSP-RK2 2, SSP-RK3 3, SSP-RK4 5
    double* dRk4[5];              // SSP-RK4 work arrays U3, U4, FU3, FU4, Fl (U1, U2 are dU1, dU2)
    float *hvX, *hvY;             // attached training-sample buffers (device), or null
    int* hvCount;
    int hvCap;
    float hvKeep;
    unsigned hvSeed;
    int wait_limit;               // test hook: polls of the kernels' bounded waits (0: ~1 s)
    bool nn_repair;               // the gate's extras repair (gpmood_set_nn_repair)
    bool timing;                  // per-kernel CUDA-event timing
    bool trace;                   // GPMOOD_TRACE=1: one line per step on stderr
    cudaEvent_t ev[GPM_MAXST][4]; // per RK stage: flux, update, MOOD loop boundaries
    int flux_nl[GPM_MAXST];       // first-pass face launches of each RK stage
    gpmood_timing tm;
    char err[512];
};

double gpm_probe_fp64();
int gpm_probe_fp64_pipes(double* gflops);
extern "C" void gpm_pol_weights(GpWeights* w);
int gpm_fast_rcp_dev(const double* x, double* y, int n);
int gpm_fast_sqrt_dev(const double* x, double* y, int n);

int gpm_mood_solo_default() {
    static const int v = [] {
        const char* e = getenv("GPMOOD_MOOD_SOLO");
        return e && *e ? atoi(e) : 12;
    }();
    return v;
}

int gpm_flux_tma_default() {
    const char* e = getenv("GPMOOD_FLUX_TMA");
    return e && *e ? (atoi(e) != 0) : 1;
}

int gpm_solo_split_default() {
    const char* e = getenv("GPMOOD_SOLO_SPLIT");
    return e && *e ? (atoi(e) != 0) : 1;
}

namespace {

// NVTX range over a host scope (steps and stages show up on an Nsight Systems
// timeline; without a tool attached the calls do nothing).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

thread_local char g_err[512];

int fail(gpmood_ctx* c, int code, const char* fmt, ...) {
    char* dst = c ? c->err : g_err;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(dst, 512, fmt, ap);
    va_end(ap);
    if (c) memcpy(g_err, c->err, 512);
    return code;
}

#define CU(call)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return fail(c, GPMOOD_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

int check_launch(gpmood_ctx* c, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, GPMOOD_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return 0;
}

size_t state_bytes(const gpmood_ctx* c) { return c->ncell * 4 * sizeof(double); }

StageArgs stage_args(gpmood_ctx* c, const double* uin, double* uout, int stage, bool uniform) {
    StageArgs a;
    a.g = c->g;
    a.uin = uin;
    a.uout = uout;
    a.fx = c->dFx;
    a.fy = c->dFy;
    a.order = c->dOrder;
    a.stamp = c->dStamp;
    a.tlist[0] = c->dList[0];
    a.tlist[1] = c->dList[1];
    a.sc = c->dSc;
    a.uniform_order = uniform ? 1 : 0;
    a.stage = stage;
    a.ccw = nullptr;
    return a;
}

// One Forward_Euler stage (mod_FE.f90:20-190) from uin (device) into uout;
// `stage` counts the Forward_Euler calls of the step, bc_stage selects t_rk
// for time-dependent boundaries (0: t, 1: t+dt, 2: t+dt/2).  Nothing here
// waits for the GPU: pass counts and status come back once per step.
int run_stage(gpmood_ctx* c, double* uin, double* uout, int stage, int bc_stage) {
    static const char* const kName[GPM_MAXST] = {"Forward_Euler 1", "Forward_Euler 2", "Forward_Euler 3",
                                                 "Forward_Euler 4", "Forward_Euler 5"};
    NvtxRange range(kName[stage < GPM_MAXST ? stage : GPM_MAXST - 1]);
    cudaStream_t s = c->stream;
    const KernelTable& kt = *c->kt;
    cudaEvent_t* ev = c->ev[stage];
    bool uniform = true, fixup = false, nnref = false;
    CU(cudaMemsetAsync(c->dOrder, c->p.mord, c->ncell, s));  // CellGPO = mord, :48
    CU(cudaMemsetAsync(c->dSc->ntrb, 0, sizeof(c->dSc->ntrb), s));
    const bool nn_on = c->p.method == GPMOOD_NN_GP_MOOD && c->niter + 1 > c->p.nsteps_with_no_nn;  // :51
    if (nn_on && c->p.nn_reference) {
        // the reference's network sets every CellGPO to 1 or 3; it reads Uin
        // before Boundary_C, as mod_FE.f90:51-56 come before :64
        const int rc = nn_ref_orders(c->nnref, c->g, uin, c->dOrder, &c->dSc->apriori_step, nullptr,
                                     c->cc ? c->dCcw : nullptr, s);
        if (rc < 0) return fail(c, GPMOOD_E_CUDA, "NN gate: %s", cudaGetErrorString(cudaGetLastError()));
        c->ctr.kernel_launches += rc;
        nnref = true;
        uniform = false;
    }
    c->kt->bc(c->g, uin, c->dSc, bc_stage, s);  // Boundary_C(Uin), :64
    c->ctr.kernel_launches += 2;
    if (nn_on && !c->p.nn_reference) {  // gated cells start at mord-2 and are listed in tlist[1]
        const int rc = nn_gate_orders(c->nn, c->g, uin, c->dOrder, &c->dSc->apriori_step, c->dList[1],
                                      &c->dSc->ntrb[1], nullptr, &c->dSc->status, s);
        if (rc < 0) return fail(c, GPMOOD_E_CUDA, "NN gate: %s", cudaGetErrorString(cudaGetLastError()));
        c->ctr.kernel_launches += rc;
        fixup = true;
        uniform = false;
    }
    StageArgs a = stage_args(c, uin, uout, stage, uniform);
    if (nnref) a.g.dmp = 0;  // NN_DETECTION: NaN and positivity only (mod_subroutine_NN_MOOD.f90:22-35)
    if (nnref && c->cc) {    // NN_GP_MOOD_CC_ reconstruction (mod_Reconstruction.f90:26-31)
        a.ccw = c->dCcw;
        a.g.cc_col = nn_ref_inputs(c->p.mord);
    }
    if (c->timing) cudaEventRecord(ev[0], s);
    // First pass over every face at mord; the faces of gated cells are then
    // recomputed at min(CellGPO) of their two cells, which gives every stored
    // flux the value of a first pass at the gated orders.  The reference's
    // network sets every order, so its first pass reads them face by face.
    StageArgs au = a;
    au.uniform_order = nnref ? 0 : 1;
    c->flux_nl[stage] = kt.flux_all(au, c->w, s);
    if (fixup) {
        if (c->nn_repair) {
            kt.gate_repair(a, c->w, c->p.lf * c->p.nf, s);
            c->ctr.kernel_launches += 1;
        }
        kt.mood_faces(a, c->w, 1, c->p.lf * c->p.nf, s);
        c->ctr.kernel_launches += 1;
    }
    if (c->timing) cudaEventRecord(ev[1], s);
    kt.update_detect(a, c->w, 0, s);
    if (c->timing) cudaEventRecord(ev[2], s);
    c->ctr.kernel_launches += 1 + c->flux_nl[stage];
    int rc = check_launch(c, "first MOOD pass");
    if (rc) return rc;
    if (c->p.method == GPMOOD_GP_MOOD || c->p.method == GPMOOD_NN_GP_MOOD) {
        // passes 2, 3, ... run on the device in one cooperative launch (the loop
        // of mod_FE.f90:69-174 ends when DETECTION flags no cell)
        const long long cap = c->p.max_mood_iters > 0 ? c->p.max_mood_iters : 2LL * c->p.lf * c->p.nf + 2;
        const int max_pass = cap > 0x7fffffff ? 0x7fffffff : (int)cap;
        if (kt.mood_loop(a, c->w, c->dBar, max_pass, stage, s))
            return fail(c, GPMOOD_E_CUDA, "MOOD loop launch: %s", cudaGetErrorString(cudaGetLastError()));
        c->ctr.kernel_launches += 1;
    }
    if (c->timing) cudaEventRecord(ev[3], s);
    CU(cudaMemcpyAsync(c->dStageOrd + (size_t)stage * c->ncell, c->dOrder, c->ncell, cudaMemcpyDeviceToDevice, s));
    if (stage == 0 && c->hvX) {  // training samples of stage 1 (mod_FE.f90:176-181)
        if (nn_harvest(c->g, uin, c->dOrder, c->hvX, c->hvY, c->hvCap, c->hvCount, c->hvKeep,
                       c->hvSeed * 2654435761u + (unsigned)c->ctr.steps, s))
            return fail(c, GPMOOD_E_CUDA, "NN harvest: %s", cudaGetErrorString(cudaGetLastError()));
        c->ctr.kernel_launches += 1;
    }
    kt.bc(c->g, uout, c->dSc, bc_stage, s);  // the last DETECTION's Boundary_C(Uout)
    c->ctr.kernel_launches += 2;
    if (c->p.integrator == GPMOOD_SSP_RK4) {  // SSP_RK4_ takes the increment, mod_FE.f90:188
        const double* x[2] = {uout, uin};
        const double k[2] = {1.0, -1.0};
        kt.lincomb(c->g, uout, 2, x, k, 0, c->dSc, s);
        c->ctr.kernel_launches += 1;
    }
    return check_launch(c, "stage");
}

// SSP_RK4_, mod_SSP_RK4.f90:12-38, with the constants of constants.f90:46-51.
int run_rk4(gpmood_ctx* c, double* u, double* ur, bool with_cfl) {
    const KernelTable& kt = *c->kt;
    cudaStream_t s = c->stream;
    const double c1 = 0.391752226571890, a20 = 0.444370493651235, a21 = 0.555629506348765,
                 c2 = 0.368410593050371, a30 = 0.620101851488403, a32 = 0.379898148511597,
                 c3 = 0.251891774271694, a40 = 0.178079954393132, a43 = 0.821920045606868,
                 c4 = 0.544974750228521, f2 = 0.517231671970585, f3 = 0.096059710526147,
                 f4 = 0.386708617503269, ff3 = 0.063692468666290, ff4 = 0.226007483236906;
    double *U1 = c->dU1, *U2 = c->dU2, *U3 = c->dRk4[0], *U4 = c->dRk4[1], *FU3 = c->dRk4[2], *FU4 = c->dRk4[3],
           *Fl = c->dRk4[4];
    int rc;
    if ((rc = run_stage(c, u, Fl, 0, 0))) return rc;
    {
        const double* x[2] = {u, Fl};
        const double k[2] = {1.0, c1};
        kt.lincomb(c->g, U1, 2, x, k, 0, c->dSc, s);
    }
    if ((rc = run_stage(c, U1, Fl, 1, 0))) return rc;
    {
        const double* x[3] = {u, U1, Fl};
        const double k[3] = {a20, a21, c2};
        kt.lincomb(c->g, U2, 3, x, k, 0, c->dSc, s);
    }
    if ((rc = run_stage(c, U2, Fl, 2, 0))) return rc;
    {
        const double* x[3] = {u, U2, Fl};
        const double k[3] = {a30, a32, c3};
        kt.lincomb(c->g, U3, 3, x, k, 0, c->dSc, s);
    }
    if ((rc = run_stage(c, U3, FU3, 3, 0))) return rc;
    {
        const double* x[3] = {u, U3, FU3};
        const double k[3] = {a40, a43, c4};
        kt.lincomb(c->g, U4, 3, x, k, 0, c->dSc, s);
    }
    if ((rc = run_stage(c, U4, FU4, 4, 0))) return rc;
    {
        const double* x[5] = {U2, U3, FU3, U4, FU4};
        const double k[5] = {f2, f3, ff3, f4, ff4};
        kt.lincomb(c->g, ur, 5, x, k, with_cfl ? 1 : 0, c->dSc, s);
    }
    c->ctr.kernel_launches += 5;
    return check_launch(c, "SSP-RK4 combinations");
}

// One time_stepping call (time_stepper.f90:12-23) from u into ur with the
// configured integrator; t, dt, qx, qy already on the device.  with_cfl fuses
// the next step's Setdt into the final combination.  One host
// synchronisation per step, at its end.
int run_step(gpmood_ctx* c, double* u, double* ur, bool with_cfl) {
    NvtxRange range("time_stepping");
    cudaStream_t s = c->stream;
    CU(cudaMemsetAsync(&c->dSc->detected_step, 0, 2 * sizeof(unsigned long long), s));
    CU(cudaMemsetAsync(&c->dSc->status, 0, sizeof(int), s));  // this step's flags (counters keep them all)
    int rc = 0;
    if (c->p.integrator == GPMOOD_SSP_RK3) {  // SSP_RK3_, mod_SSP_RK3.f90:12-39
        rc = run_stage(c, u, c->dU1, 0, 0);
        if (rc) return rc;
        rc = run_stage(c, c->dU1, c->dU2, 1, 1);
        if (rc) return rc;
        c->kt->combine(c->g, u, c->dU2, 0.75, 0.25, 0, c->dSc, s);  // U2 = 0.75 Uin + 0.25 U2
        c->ctr.kernel_launches += 2;
        rc = run_stage(c, c->dU2, ur, 2, 2);
        if (rc) return rc;
        c->kt->combine(c->g, u, ur, 1. / 3, 2. / 3, with_cfl ? 1 : 0, c->dSc, s);  // Uout = Uin/3 + 2 Uout/3
    } else if (c->p.integrator == GPMOOD_SSP_RK2) {  // SSP_RK2_, mod_SSP_RK2.f90:12-24 (t_rk = t)
        rc = run_stage(c, u, c->dU1, 0, 0);
        if (rc) return rc;
        rc = run_stage(c, c->dU1, ur, 1, 0);
        if (rc) return rc;
        // 0.5*(Uin+Uout): both halvings are exact, so 0.5*Uin + 0.5*Uout rounds the same
        c->kt->combine(c->g, u, ur, 0.5, 0.5, with_cfl ? 1 : 0, c->dSc, s);
        c->ctr.kernel_launches += 1;
    } else if (c->p.integrator == GPMOOD_SSP_RK4) {
        rc = run_rk4(c, u, ur, with_cfl);
        if (rc) return rc;
    } else {  // FE: one Forward_Euler (time_stepper.f90:18)
        rc = run_stage(c, u, ur, 0, 0);
        if (rc) return rc;
        if (with_cfl) {
            c->kt->cfl(c->g, ur, c->dSc, s);
            c->ctr.kernel_launches += 1;
        }
    }
    rc = check_launch(c, "combine");
    if (rc) return rc;
    CU(cudaMemcpyAsync(c->hSc, c->dSc, sizeof(DevScalars), cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(c->hBar, c->dBar, sizeof(GridBar), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    const bool mood = c->p.method == GPMOOD_GP_MOOD || c->p.method == GPMOOD_NN_GP_MOOD;
    long long passes = 0;
    for (int st = 0; st < c->nstages; st++) {
        const long long np = mood ? c->hSc->passes_stage[st] : 1;
        passes += np;
        if (np > c->ctr.max_passes_stage) c->ctr.max_passes_stage = np;
        if (c->timing) {
            float f = 0.f, u_ = 0.f, m = 0.f;
            cudaEventElapsedTime(&f, c->ev[st][0], c->ev[st][1]);
            cudaEventElapsedTime(&u_, c->ev[st][1], c->ev[st][2]);
            cudaEventElapsedTime(&m, c->ev[st][2], c->ev[st][3]);
            c->tm.flux_ms += f;
            c->tm.flux_launches += 1;  // one first pass (all faces of the stage)
            c->tm.flux_faces += (long long)(c->p.lf + 1) * c->p.nf + (long long)c->p.lf * (c->p.nf + 1);
            c->tm.update_ms += u_;
            c->tm.update_launches += 1;
            c->tm.mood_ms += m;
            c->tm.mood_passes += np - 1;
        }
    }
    c->ctr.detected_last_step = (long long)c->hSc->detected_step;
    c->ctr.a_priori_last_step = (long long)c->hSc->apriori_step;
    c->ctr.detected_total += (long long)c->hSc->detected_step;
    c->ctr.mood_passes_last_step = passes;
    c->ctr.steps++;
    c->ctr.status_flags |= c->hSc->status;
    if (c->hBar->err) {
        c->ctr.status_flags |= GPM_STATUS_BARRIER;
        // the aborted loop left its pass stamps without advancing the stamp
        // epoch: clear both with the barrier, so that the next loop's pass ids
        // cannot collide with them
        cudaMemsetAsync(c->dBar, 0, sizeof(GridBar), s);
        if (c->wait_limit) cudaMemcpyAsync(&c->dBar->limit, &c->wait_limit, sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(c->dStamp, 0, c->ncell * sizeof(unsigned), s);
        cudaMemsetAsync(&c->dSc->stamp_epoch, 0, sizeof(unsigned), s);
        cudaStreamSynchronize(s);
        return fail(c, GPMOOD_E_CUDA, "MOOD loop: grid barrier timed out");
    }
    if (c->hSc->status & GPM_STATUS_TENSOR) return fail(c, GPMOOD_E_CUDA, "NN gate: tensor-core wait timed out");
    if (c->hSc->status & GPM_STATUS_TMA) return fail(c, GPMOOD_E_CUDA, "first pass: TMA tile copy wait timed out");
    if (c->hSc->status & GPM_STATUS_MOODCAP) {
        const long long cap = c->p.max_mood_iters > 0 ? c->p.max_mood_iters : 2LL * c->p.lf * c->p.nf + 2;
        return fail(c, GPMOOD_E_MOOD_CAP, "MOOD loop did not converge in %lld passes", cap);
    }
    return 0;
}

// Put t, dt and dt/dx, dt/dy computed on the host (IEEE, same bits) on the device.
int set_time(gpmood_ctx* c, double t, double dt) {
    c->hSc->t = t;
    c->hSc->dt = dt;
    c->hSc->qx = dt / c->g.dx;
    c->hSc->qy = dt / c->g.dy;
    CU(cudaMemcpyAsync(c->dSc, c->hSc, 4 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return 0;
}

int validate(const gpmood_params* p, char* why, size_t n) {
    if (!p) { snprintf(why, n, "params is NULL"); return -1; }
    if (p->integrator != GPMOOD_FE && p->integrator != GPMOOD_SSP_RK2 && p->integrator != GPMOOD_SSP_RK3 &&
        p->integrator != GPMOOD_SSP_RK4) {
        snprintf(why, n, "integrator %d unsupported (FE=8, SSP_RK2=9, SSP_RK3=10, SSP_RK4=12)", p->integrator); return -1; }
    if (p->method != GPMOOD_GP_MOOD && p->method != GPMOOD_GP_SE && p->method != GPMOOD_NN_GP_MOOD &&
        p->method != GPMOOD_NN_GP_MOOD_CC && p->method != GPMOOD_POL_MOOD && p->method != GPMOOD_UNLIM_POL &&
        p->method != GPMOOD_FOG) {
        snprintf(why, n, "method %d unsupported (FOG=1, GP_MOOD=2, POL_MOOD=200, Unlim_POL=201, GP_SE=202, "
                 "NN_GP_MOOD=203, NN_GP_MOOD_CC=204)", p->method);
        return -1; }
    if (p->method == GPMOOD_FOG && p->ngp != 1) {  // FOG_ sets Gauss point 1 only (mod_FOG.f90:22-24)
        snprintf(why, n, "FOG needs ngp 1"); return -1; }
    if ((p->method == GPMOOD_POL_MOOD || p->method == GPMOOD_UNLIM_POL) && (p->mord != 3 || p->ngp != 2)) {
        snprintf(why, n, "POL_MOOD and Unlim_POL need Mord 3 and ngp 2 (pol_presim's weights)"); return -1; }
    if (p->method == GPMOOD_NN_GP_MOOD_CC && p->mord != 3) {  // mod_NN_GP_MOOD_CC.f90:73 stops above order 3
        snprintf(why, n, "NN_GP_MOOD_CC needs Mord 3"); return -1; }
    if (p->num_flux < GPMOOD_HLLC || p->num_flux > GPMOOD_UNSPLIT) {
        snprintf(why, n, "numFlux %d unsupported (HLLC=100, LLF=101, HLL=102, unsplit=103)", p->num_flux); return -1; }
    if (!(p->mord == 1 || p->mord == 3 || p->mord == 5)) { snprintf(why, n, "Mord %d unsupported (1, 3, 5)", p->mord); return -1; }
    if (p->ngp < 1 || p->ngp > 5) { snprintf(why, n, "ngp %d out of 1..5", p->ngp); return -1; }
    if (p->lf < 4 || p->nf < 4 || p->lf > 65536 || p->nf > 65536) { snprintf(why, n, "grid %dx%d out of range", p->lf, p->nf); return -1; }
    if (p->bc_type != GPMOOD_NEUMANN && p->bc_type != GPMOOD_PERIODIC && p->bc_type != GPMOOD_REFLECTIVE &&
        p->bc_type != GPMOOD_DMR && p->bc_type != GPMOOD_DIRICHLET && p->bc_type != GPMOOD_MACH800 &&
        p->bc_type != GPMOOD_DOUBLE_MACH800 && p->bc_type != GPMOOD_RMI && p->bc_type != GPMOOD_RT &&
        p->bc_type != GPMOOD_KH) { snprintf(why, n, "BC_type %d unsupported", p->bc_type); return -1; }
    if (!(p->cfl > 0) || !(p->lx > 0) || !(p->ly > 0) || !(p->ell_o_dx > 0)) { snprintf(why, n, "CFL, Lx, Ly, ell_o_dx must be > 0"); return -1; }
    if (p->fp_mode != GPMOOD_FP_EXACT && p->fp_mode != GPMOOD_FP_FAST) { snprintf(why, n, "fp_mode %d unknown", p->fp_mode); return -1; }
    if (p->max_mood_iters < 0) { snprintf(why, n, "max_mood_iters must be >= 0 (0: no cap but termination)"); return -1; }
    if (p->nn_reference && p->mord != 3 && p->mord != 5) {
        snprintf(why, n, "nn_reference needs Mord 3 or 5 (the R+1 stencil of the reference's network)"); return -1; }
    return 0;
}

void free_all(gpmood_ctx* c) {
    if (!c) return;
    cudaFree(c->dU); cudaFree(c->dUr); cudaFree(c->dU1); cudaFree(c->dU2);
    cudaFree(c->dFx); cudaFree(c->dFy); cudaFree(c->dOrder); cudaFree(c->dStamp);
    cudaFree(c->dList[0]); cudaFree(c->dList[1]); cudaFree(c->dSc); cudaFree(c->dStageOrd); cudaFree(c->dBar);
    for (int i = 0; i < 5; i++) cudaFree(c->dRk4[i]);
    if (c->hBar) cudaFreeHost(c->hBar);
    if (c->hSc) cudaFreeHost(c->hSc);
    if (c->hCount) cudaFreeHost(c->hCount);
    if (c->nn) nn_gate_destroy(c->nn);
    if (c->nnref) nn_ref_destroy(c->nnref);
    if (c->dCcw) cudaFree(c->dCcw);
    for (int st = 0; st < GPM_MAXST; st++)
        for (int i = 0; i < 4; i++)
            if (c->ev[st][i]) cudaEventDestroy(c->ev[st][i]);
    if (c->stream) cudaStreamDestroy(c->stream);
}

}  // namespace

void gpm_set_thread_error(const char* msg) { snprintf(g_err, sizeof g_err, "%s", msg); }

int gpm_validate_params(const gpmood_params* p, char* why, size_t n) { return validate(p, why, n); }

extern "C" {

int gpmood_default_params(gpmood_params* p) {
    if (!p) return fail(nullptr, GPMOOD_E_ARG, "params is NULL");
    memset(p, 0, sizeof(*p));
    p->cfl = 0.8;
    p->ell_o_dx = 12.0;
    p->lx = 1.0;
    p->ly = 1.0;
    p->tmax = 0.8;
    p->integrator = GPMOOD_SSP_RK3;
    p->method = GPMOOD_GP_MOOD;
    p->mord = 5;
    p->ngp = 3;
    p->dmp = p->u2 = p->u2_tol = 1;
    p->num_flux = GPMOOD_HLLC;
    p->lf = p->nf = 256;
    p->bc_type = GPMOOD_NEUMANN;
    p->nmax = 1 << 30;
    p->fp_mode = GPMOOD_FP_EXACT;
    p->max_mood_iters = 0;
    p->nsteps_with_no_nn = 0;
    return 0;
}

int gpmood_create(const gpmood_params* p, gpmood_ctx** out) {
    gpmood_ctx* c = nullptr;
    if (!out) return fail(nullptr, GPMOOD_E_ARG, "out is NULL");
    *out = nullptr;
    char why[256];
    if (validate(p, why, sizeof why)) return fail(nullptr, GPMOOD_E_ARG, "%s", why);
    c = new (std::nothrow) gpmood_ctx();
    if (!c) return fail(nullptr, GPMOOD_E_ARG, "out of host memory");
    c->p = *p;
    c->cc = p->method == GPMOOD_NN_GP_MOOD_CC;
    if (c->cc) {  // the reference's network with its convex-combination reconstruction
        c->p.method = GPMOOD_NN_GP_MOOD;
        c->p.nn_reference = 1;
    }
    // POL_MOOD / Unlim_POL: GP_MOOD / GP_SE with the polynomial weights (below)
    const bool pol = p->method == GPMOOD_POL_MOOD || p->method == GPMOOD_UNLIM_POL;
    if (pol) c->p.method = p->method == GPMOOD_POL_MOOD ? GPMOOD_GP_MOOD : GPMOOD_GP_SE;
    // FOG: every face state is the cell value and no DETECTION runs (mod_FOG.f90,
    // mod_FE.f90:161), i.e. GP_SE at order 1 (its weight is 1); the order mask
    // then reads 1 where the reference's CellGPO keeps Mord untouched
    if (p->method == GPMOOD_FOG) {
        c->p.method = GPMOOD_GP_SE;
        c->p.mord = 1;
    }
    c->g.lf = p->lf;
    c->g.nf = p->nf;
    c->g.nx = p->lf + 2 * GPM_NGC;
    c->g.ny = p->nf + 2 * GPM_NGC;
    // dx = real(Lx_16/lf, PR) (global_variables.f90:86-88), rounded from binary128.
    c->g.dx = (double)((_Float128)p->lx / p->lf);
    c->g.dy = (double)((_Float128)p->ly / p->nf);
    c->g.bc_type = p->bc_type;
    c->g.ngp = p->ngp;
    c->g.mord = c->p.mord;
    c->g.method = c->p.method;
    c->g.num_flux = p->num_flux;
    c->g.mood_solo = gpm_mood_solo_default();
    c->g.flux_tma = gpm_flux_tma_default();
    c->g.solo_split = gpm_solo_split_default();
    c->g.cc_col = -1;
    c->nstages = p->integrator == GPMOOD_FE ? 1 : p->integrator == GPMOOD_SSP_RK2 ? 2 : p->integrator == GPMOOD_SSP_RK4 ? 5 : 3;
    c->g.dmp = p->dmp;
    c->g.u2 = p->u2;
    c->g.u2_tol = p->u2_tol;
    c->g.u2_fd = p->method == GPMOOD_POL_MOOD;
    c->ncell = (size_t)c->g.nx * c->g.ny;
    c->kt = p->fp_mode == GPMOOD_FP_FAST ? &gpm_fast::table : &gpm_exact::table;
    {
        const char* tr = getenv("GPMOOD_TRACE");
        c->trace = tr && tr[0] == '1';
    }
    if (gpm_gp_presim(p->ell_o_dx, p->lx, p->ly, p->lf, p->nf, p->mord, p->ngp, &c->w, c->inv_err)) {
        delete c;
        return fail(nullptr, GPMOOD_E_ARG, "GP precompute rejected the knobs");
    }
    if (pol) gpm_pol_weights(&c->w);
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev < 1) {
        delete c;
        return fail(nullptr, GPMOOD_E_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
    }
#define ALLOC(ptr, bytes)                                                                             \
    do {                                                                                              \
        cudaError_t e_ = cudaMalloc((void**)&(ptr), (bytes));                                         \
        if (e_ != cudaSuccess) {                                                                      \
            fail(c, GPMOOD_E_CUDA, "cudaMalloc(%zu): %s", (size_t)(bytes), cudaGetErrorString(e_));   \
            free_all(c);                                                                              \
            delete c;                                                                                 \
            return GPMOOD_E_CUDA;                                                                     \
        }                                                                                             \
    } while (0)
    const size_t sb = c->ncell * 4 * sizeof(double);
    ALLOC(c->dU, sb);
    ALLOC(c->dUr, sb);
    ALLOC(c->dU1, sb);
    ALLOC(c->dU2, sb);
    ALLOC(c->dFx, sb);
    ALLOC(c->dFy, sb);
    ALLOC(c->dOrder, c->ncell);
    ALLOC(c->dStamp, c->ncell * sizeof(unsigned));
    ALLOC(c->dList[0], c->ncell * sizeof(int));
    ALLOC(c->dList[1], c->ncell * sizeof(int));
    ALLOC(c->dSc, sizeof(DevScalars));
    ALLOC(c->dStageOrd, GPM_MAXST * c->ncell);
    if (p->integrator == GPMOOD_SSP_RK4)
        for (int i = 0; i < 5; i++) ALLOC(c->dRk4[i], sb);
    ALLOC(c->dBar, sizeof(GridBar));
#undef ALLOC
    if (cudaMallocHost((void**)&c->hSc, sizeof(DevScalars)) != cudaSuccess ||
        cudaMallocHost((void**)&c->hCount, sizeof(int)) != cudaSuccess ||
        cudaMallocHost((void**)&c->hBar, sizeof(GridBar)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        fail(c, GPMOOD_E_CUDA, "pinned memory / stream creation failed");
        free_all(c);
        delete c;
        return GPMOOD_E_CUDA;
    }
    for (int i = 0; i < 4 * GPM_MAXST; i++) {
        if (cudaEventCreate(&c->ev[i / 4][i % 4]) != cudaSuccess) {
            fail(c, GPMOOD_E_CUDA, "event creation failed");
            free_all(c);
            delete c;
            return GPMOOD_E_CUDA;
        }
    }
    memset(c->hSc, 0, sizeof(DevScalars));
    c->hSc->tmax = p->tmax;
    c->hSc->cfl = p->cfl;
    if (p->bc_type == GPMOOD_DIRICHLET)  // BC.f90:68: sin() on the host, as the CPU restatement does
        for (int j = 0; j < GPM_NGC; j++) {
            const int l = p->lf + 1 + j;
            const double x = l * c->g.dx - c->g.dx / 2, r = 1. + 0.2 * sin(5 * (x - 4.5));
            double* q = c->hSc->bcd[j];
            q[0] = r;
            q[1] = r * 0.;
            q[2] = r * 0.;
            q[3] = ((1. / (1.4 - 1.)) + 0.5 * r * (0. * 0. + 0. * 0.));  // p2c(r, 0, 0, 1), gamma = 1.4
        }
    c->hSc->dtmin_bits = 0x46293e5939a08ceaULL;  // bits of 1.0e30
    // Initialise on the context's own stream: it is non-blocking, so work on the
    // legacy default stream would not be ordered before its first kernels.
    cudaStream_t s0 = c->stream;
    if (cudaMemcpyAsync(c->dSc, c->hSc, sizeof(DevScalars), cudaMemcpyHostToDevice, s0) != cudaSuccess ||
        cudaMemsetAsync(c->dStamp, 0, c->ncell * sizeof(unsigned), s0) != cudaSuccess ||
        cudaMemsetAsync(c->dFx, 0, sb, s0) != cudaSuccess || cudaMemsetAsync(c->dFy, 0, sb, s0) != cudaSuccess ||
        cudaMemsetAsync(c->dU, 0, sb, s0) != cudaSuccess || cudaMemsetAsync(c->dUr, 0, sb, s0) != cudaSuccess ||
        cudaMemsetAsync(c->dU1, 0, sb, s0) != cudaSuccess || cudaMemsetAsync(c->dU2, 0, sb, s0) != cudaSuccess ||
        cudaMemsetAsync(c->dStageOrd, c->p.mord, GPM_MAXST * c->ncell, s0) != cudaSuccess ||
        cudaMemsetAsync(c->dBar, 0, sizeof(GridBar), s0) != cudaSuccess ||
        cudaStreamSynchronize(s0) != cudaSuccess) {
        fail(c, GPMOOD_E_CUDA, "device initialisation failed");
        free_all(c);
        delete c;
        return GPMOOD_E_CUDA;
    }
    c->nn = nn_gate_create(c->g);
    c->nnref = nn_ref_create();
    if (c->cc && cudaMalloc(&c->dCcw, sizeof(float) * 2 * (size_t)(p->nf + 2)) != cudaSuccess) c->dCcw = nullptr;
    if (!c->nn || !c->nnref || (c->cc && !c->dCcw)) {
        fail(c, GPMOOD_E_CUDA, "NN gate allocation failed");
        free_all(c);
        delete c;
        return GPMOOD_E_CUDA;
    }
    *out = c;
    return 0;
}

void gpmood_destroy(gpmood_ctx* c) {
    if (!c) return;
    cudaStreamSynchronize(c->stream);
    free_all(c);
    delete c;
}

int gpmood_last_error(const gpmood_ctx* c, char* buf, int len) {
    if (!buf || len <= 0) return GPMOOD_E_ARG;
    snprintf(buf, (size_t)len, "%s", c ? c->err : g_err);
    return 0;
}

int gpmood_get_weights(const gpmood_ctx* c, double* zt, double* d2, double* inv_err) {
    if (!c) return fail(nullptr, GPMOOD_E_ARG, "ctx is NULL");
    const int ngp = c->p.ngp;
    if (zt)
        for (int o = 0; o < 3; o++)
            for (int f = 0; f < 4; f++)
                for (int g = 0; g < ngp; g++)
                    for (int m = 0; m < 13; m++) zt[((o * 4 + f) * ngp + g) * 13 + m] = c->w.zt[o][f][g][m];
    if (d2)
        for (int m = 0; m < 5; m++) {
            d2[m] = c->w.d2x[m];
            d2[5 + m] = c->w.d2y[m];
        }
    if (inv_err)
        for (int o = 0; o < 3; o++) inv_err[o] = c->inv_err[o];
    return 0;
}

int gpmood_gp_weights(const gpmood_params* p, double* zt, double* d2, double* inv_err) {
    char why[256];
    if (validate(p, why, sizeof why)) return fail(nullptr, GPMOOD_E_ARG, "%s", why);
    GpWeights w;
    double ie[3];
    if (gpm_gp_presim(p->ell_o_dx, p->lx, p->ly, p->lf, p->nf, p->mord, p->ngp, &w, ie))
        return fail(nullptr, GPMOOD_E_ARG, "GP precompute rejected the knobs");
    if (p->method == GPMOOD_POL_MOOD || p->method == GPMOOD_UNLIM_POL) gpm_pol_weights(&w);
    const int ngp = p->ngp;
    if (zt)
        for (int o = 0; o < 3; o++)
            for (int f = 0; f < 4; f++)
                for (int g = 0; g < ngp; g++)
                    for (int m = 0; m < 13; m++) zt[((o * 4 + f) * ngp + g) * 13 + m] = w.zt[o][f][g][m];
    if (d2)
        for (int m = 0; m < 5; m++) {
            d2[m] = w.d2x[m];
            d2[5 + m] = w.d2y[m];
        }
    if (inv_err)
        for (int o = 0; o < 3; o++) inv_err[o] = ie[o];
    return 0;
}

int gpmood_boundary_c(gpmood_ctx* c, double* u_host, double t_rk) {
    if (!c || !u_host) return fail(c, GPMOOD_E_ARG, "NULL argument");
    CU(cudaMemcpyAsync(c->dU2, u_host, state_bytes(c), cudaMemcpyHostToDevice, c->stream));
    int rc = set_time(c, t_rk, 0.0);
    if (rc) return rc;
    c->kt->bc(c->g, c->dU2, c->dSc, 0, c->stream);
    rc = check_launch(c, "Boundary_C");
    if (rc) return rc;
    CU(cudaMemcpyAsync(u_host, c->dU2, state_bytes(c), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return 0;
}

int gpmood_setdt(gpmood_ctx* c, const double* u_host, double dtfinal, double* dt_out) {
    if (!c || !u_host || !dt_out) return fail(c, GPMOOD_E_ARG, "NULL argument");
    CU(cudaMemcpyAsync(c->dU2, u_host, state_bytes(c), cudaMemcpyHostToDevice, c->stream));
    c->kt->cfl(c->g, c->dU2, c->dSc, c->stream);
    c->kt->dt_finalize(c->g, c->dSc, dtfinal < 0.0 ? 0.0 : dtfinal, c->stream);
    c->ctr.kernel_launches += 2;
    int rc = check_launch(c, "Setdt");
    if (rc) return rc;
    CU(cudaMemcpyAsync(c->hSc, c->dSc, sizeof(DevScalars), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    *dt_out = c->hSc->dt;
    c->dt_pending = false;
    if (c->hSc->status & GPM_STATUS_DT) return fail(c, GPMOOD_E_DT, "Setdt produced dt = %g", c->hSc->dt);
    return 0;
}

int gpmood_time_stepping(gpmood_ctx* c, const double* uin_host, double* uout_host, double t, double dt) {
    if (!c || !uin_host || !uout_host) return fail(c, GPMOOD_E_ARG, "NULL argument");
    if (!(dt > 0) || !isfinite(dt)) return fail(c, GPMOOD_E_DT, "dt = %g", dt);
    CU(cudaMemcpyAsync(c->dU, uin_host, state_bytes(c), cudaMemcpyHostToDevice, c->stream));
    int rc = set_time(c, t, dt);
    if (rc) return rc;
    rc = run_step(c, c->dU, c->dUr, false);
    if (rc) return rc;
    CU(cudaMemcpyAsync(uout_host, c->dUr, state_bytes(c), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    c->have_state = false;  // dU no longer mirrors a set_state upload
    return 0;
}

int gpmood_setdt_time_stepping(gpmood_ctx* c, const double* uin_host, double* uout_host, double t, double dtfinal,
                               double* dt_out) {
    if (!c || !uin_host || !uout_host || !dt_out) return fail(c, GPMOOD_E_ARG, "NULL argument");
    CU(cudaMemcpyAsync(c->dU, uin_host, state_bytes(c), cudaMemcpyHostToDevice, c->stream));
    c->have_state = false;  // dU no longer mirrors a set_state upload
    c->kt->cfl(c->g, c->dU, c->dSc, c->stream);
    c->kt->dt_finalize(c->g, c->dSc, dtfinal < 0.0 ? 0.0 : dtfinal, c->stream);
    c->ctr.kernel_launches += 2;
    int rc = check_launch(c, "Setdt");
    if (rc) return rc;
    CU(cudaMemcpyAsync(c->hSc, c->dSc, sizeof(DevScalars), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    const double dt = c->hSc->dt;
    *dt_out = dt;
    c->dt_pending = false;
    if ((c->hSc->status & GPM_STATUS_DT) || !(dt > 0) || !isfinite(dt))
        return fail(c, GPMOOD_E_DT, "Setdt produced dt = %g", dt);
    rc = set_time(c, t, dt);
    if (rc) return rc;
    rc = run_step(c, c->dU, c->dUr, false);
    if (rc) return rc;
    CU(cudaMemcpyAsync(uout_host, c->dUr, state_bytes(c), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return 0;
}

int gpmood_time_stepping_dev(gpmood_ctx* c, double* d_uin, double* d_uout, double t, double dt) {
    if (!c || !d_uin || !d_uout) return fail(c, GPMOOD_E_ARG, "NULL argument");
    if (!(dt > 0) || !isfinite(dt)) return fail(c, GPMOOD_E_DT, "dt = %g", dt);
    int rc = set_time(c, t, dt);
    if (rc) return rc;
    return run_step(c, d_uin, d_uout, false);
}

int gpmood_set_state(gpmood_ctx* c, const double* u_host, double t) {
    if (!c || !u_host) return fail(c, GPMOOD_E_ARG, "NULL argument");
    CU(cudaMemcpyAsync(c->dU, u_host, state_bytes(c), cudaMemcpyHostToDevice, c->stream));
    int rc = set_time(c, t, 0.0);
    if (rc) return rc;
    CU(cudaStreamSynchronize(c->stream));
    c->t = t;
    c->niter = 0;
    c->have_state = true;
    c->dt_pending = false;
    return 0;
}

int gpmood_get_state(gpmood_ctx* c, double* u_host, double* t, int* niter) {
    if (!c) return fail(nullptr, GPMOOD_E_ARG, "ctx is NULL");
    if (!c->have_state) return fail(c, GPMOOD_E_STATE, "no device-resident state (call gpmood_set_state)");
    if (u_host) {
        CU(cudaMemcpyAsync(u_host, c->dU, state_bytes(c), cudaMemcpyDeviceToHost, c->stream));
        CU(cudaStreamSynchronize(c->stream));
    }
    if (t) *t = c->t;
    if (niter) *niter = c->niter;
    return 0;
}

int gpmood_set_state_dev(gpmood_ctx* c, const double* d_u, double t) {
    if (!c || !d_u) return fail(c, GPMOOD_E_ARG, "NULL argument");
    CU(cudaMemcpyAsync(c->dU, d_u, state_bytes(c), cudaMemcpyDeviceToDevice, c->stream));
    int rc = set_time(c, t, 0.0);
    if (rc) return rc;
    CU(cudaStreamSynchronize(c->stream));
    c->t = t;
    c->niter = 0;
    c->have_state = true;
    c->dt_pending = false;
    return 0;
}

int gpmood_get_state_dev(gpmood_ctx* c, double* d_u) {
    if (!c || !d_u) return fail(c, GPMOOD_E_ARG, "NULL argument");
    if (!c->have_state) return fail(c, GPMOOD_E_STATE, "no device-resident state (call gpmood_set_state)");
    CU(cudaMemcpyAsync(d_u, c->dU, state_bytes(c), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return 0;
}

int gpmood_get_orders(gpmood_ctx* c, signed char* orders) {
    if (!c || !orders) return fail(c, GPMOOD_E_ARG, "NULL argument");
    // CellGPO(1:lf, 1:nf): interior rows of the padded order array.
    CU(cudaMemcpy2DAsync(orders, (size_t)c->p.lf, c->dOrder + (size_t)(GPM_NGC) * c->g.nx + GPM_NGC,
                         (size_t)c->g.nx, (size_t)c->p.lf, (size_t)c->p.nf, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return 0;
}

int gpmood_advance(gpmood_ctx* c, int nsteps, int* steps_done) {
    if (!c) return fail(nullptr, GPMOOD_E_ARG, "ctx is NULL");
    if (!c->have_state) return fail(c, GPMOOD_E_STATE, "no device-resident state (call gpmood_set_state)");
    if (c->p.method == GPMOOD_NN_GP_MOOD && (c->p.nn_reference ? !nn_ref_loaded(c->nnref) : !nn_gate_loaded(c->nn)))
        return fail(c, GPMOOD_E_STATE, "method NN_GP_MOOD needs the network's parameters (gpmood_set_nn)");
    if (steps_done) *steps_done = 0;
    int done = 0;
    while (done < nsteps && c->t < c->p.tmax && c->niter < c->p.nmax) {  // main.f90:145
        if (!c->dt_pending) {  // Setdt(U) (main.f90:151); later steps fuse it into the last combine
            c->kt->cfl(c->g, c->dU, c->dSc, c->stream);
            c->ctr.kernel_launches += 1;
        }
        c->kt->dt_finalize(c->g, c->dSc, -1.0, c->stream);
        c->ctr.kernel_launches += 1;
        int rc = run_step(c, c->dU, c->dUr, true);
        if (rc) return rc;
        if (c->hSc->status & GPM_STATUS_DT) return fail(c, GPMOOD_E_DT, "Setdt produced dt = %g", c->hSc->dt);
        c->kt->advance_t(c->dSc, c->stream);  // t = t + dt
        c->ctr.kernel_launches += 1;
        double* tmp = c->dU;                   // U = Ur
        c->dU = c->dUr;
        c->dUr = tmp;
        c->t = c->hSc->t + c->hSc->dt;
        c->niter++;
        if (c->trace)
            fprintf(stderr, "[gpmood] step %d t=%.9e dt=%.9e detected=%lld passes=%lld status=%d\n", c->niter,
                    c->t, c->hSc->dt, c->ctr.detected_last_step, c->ctr.mood_passes_last_step, c->hSc->status);
        c->dt_pending = true;
        done++;
        if (steps_done) *steps_done = done;
    }
    CU(cudaStreamSynchronize(c->stream));
    return check_launch(c, "advance");
}

int gpmood_get_counters(const gpmood_ctx* c, gpmood_counters* out) {
    if (!c || !out) return fail(nullptr, GPMOOD_E_ARG, "NULL argument");
    *out = c->ctr;
    return 0;
}

void* gpmood_get_stream(const gpmood_ctx* c) { return c ? (void*)c->stream : nullptr; }

int gpmood_set_timing(gpmood_ctx* c, int on) {
    if (!c) return fail(nullptr, GPMOOD_E_ARG, "ctx is NULL");
    c->timing = on != 0;
    memset(&c->tm, 0, sizeof(c->tm));
    return 0;
}

int gpmood_get_timing(const gpmood_ctx* c, gpmood_timing* out) {
    if (!c || !out) return fail(nullptr, GPMOOD_E_ARG, "NULL argument");
    *out = c->tm;
    return 0;
}

int gpmood_probe_fp64(double* gflops) {
    if (!gflops) return fail(nullptr, GPMOOD_E_ARG, "NULL argument");
    const double g = gpm_probe_fp64();
    if (!(g > 0)) return fail(nullptr, GPMOOD_E_CUDA, "FP64 probe failed: %s", cudaGetErrorString(cudaGetLastError()));
    *gflops = g;
    return 0;
}

int gpmood_probe_fp64_pipes(double* gflops3) {
    if (!gflops3) return fail(nullptr, GPMOOD_E_ARG, "NULL argument");
    if (gpm_probe_fp64_pipes(gflops3))
        return fail(nullptr, GPMOOD_E_CUDA, "FP64 pipe probe failed: %s", cudaGetErrorString(cudaGetLastError()));
    return 0;
}

int gpmood_fast_rcp(const double* d_x, double* d_y, int n) {
    if ((!d_x || !d_y) && n > 0) return fail(nullptr, GPMOOD_E_ARG, "NULL argument");
    if (gpm_fast_rcp_dev(d_x, d_y, n)) return fail(nullptr, GPMOOD_E_CUDA, "fast_rcp: %s", cudaGetErrorString(cudaGetLastError()));
    return 0;
}

int gpmood_fast_sqrt(const double* d_x, double* d_y, int n) {
    if ((!d_x || !d_y) && n > 0) return fail(nullptr, GPMOOD_E_ARG, "NULL argument");
    if (gpm_fast_sqrt_dev(d_x, d_y, n)) return fail(nullptr, GPMOOD_E_CUDA, "fast_sqrt: %s", cudaGetErrorString(cudaGetLastError()));
    return 0;
}

int gpmood_set_nn(gpmood_ctx* c, const float* params, int n) {
    if (!c || !params) return fail(c, GPMOOD_E_ARG, "NULL argument");
    if (c->p.nn_reference) {
        const int rc = nn_ref_set(c->nnref, params, n, c->p.mord, c->stream);
        if (rc == -1)
            return fail(c, GPMOOD_E_ARG, "%d values is no reference network for Mord %d (len^2 + (L+4) len + 2, L = %d)",
                        n, c->p.mord, nn_ref_inputs(c->p.mord));
        if (rc) return fail(c, GPMOOD_E_CUDA, "reference network upload failed");
        CU(cudaStreamSynchronize(c->stream));
        return 0;
    }
    if (n != NN_GATE_NPARAMS) return fail(c, GPMOOD_E_ARG, "expected %d gate parameters, got %d", NN_GATE_NPARAMS, n);
    if (nn_gate_set(c->nn, params, c->stream)) return fail(c, GPMOOD_E_CUDA, "NN gate upload failed");
    CU(cudaStreamSynchronize(c->stream));
    return 0;
}

int gpmood_nn_ref_logits(gpmood_ctx* c, float* d_logits) {
    if (!c || !d_logits) return fail(c, GPMOOD_E_ARG, "NULL argument");
    if (!c->have_state) return fail(c, GPMOOD_E_STATE, "no device-resident state (call gpmood_set_state)");
    if (!c->p.nn_reference || !nn_ref_loaded(c->nnref)) return fail(c, GPMOOD_E_STATE, "no reference network loaded");
    CU(cudaMemsetAsync(&c->dSc->apriori_step, 0, sizeof(unsigned long long), c->stream));
    if (nn_ref_orders(c->nnref, c->g, c->dU, c->dOrder, &c->dSc->apriori_step, d_logits, c->cc ? c->dCcw : nullptr,
                      c->stream) < 0)
        return fail(c, GPMOOD_E_CUDA, "reference network: %s", cudaGetErrorString(cudaGetLastError()));
    CU(cudaStreamSynchronize(c->stream));
    return 0;
}

int gpmood_nn_gate_logits(gpmood_ctx* c, float* d_logits) {
    if (!c || !d_logits) return fail(c, GPMOOD_E_ARG, "NULL argument");
    if (!c->have_state) return fail(c, GPMOOD_E_STATE, "no device-resident state (call gpmood_set_state)");
    if (c->p.nn_reference || !nn_gate_loaded(c->nn)) return fail(c, GPMOOD_E_STATE, "no gate parameters loaded");
    CU(cudaMemsetAsync(c->dOrder, c->p.mord, c->ncell, c->stream));
    CU(cudaMemsetAsync(&c->dSc->apriori_step, 0, sizeof(unsigned long long), c->stream));
    CU(cudaMemsetAsync(c->dSc->ntrb, 0, sizeof(c->dSc->ntrb), c->stream));
    if (nn_gate_orders(c->nn, c->g, c->dU, c->dOrder, &c->dSc->apriori_step, c->dList[1], &c->dSc->ntrb[1], d_logits,
                       &c->dSc->status, c->stream) < 0)
        return fail(c, GPMOOD_E_CUDA, "NN gate: %s", cudaGetErrorString(cudaGetLastError()));
    int st = 0;
    CU(cudaMemcpyAsync(&st, &c->dSc->status, sizeof st, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    if (st & GPM_STATUS_TENSOR) return fail(c, GPMOOD_E_CUDA, "NN gate: tensor-core wait timed out");
    return 0;
}

int gpmood_set_wait_limit(gpmood_ctx* c, int polls) {
    if (!c) return fail(nullptr, GPMOOD_E_ARG, "ctx is NULL");
    if (polls < 0) return fail(c, GPMOOD_E_ARG, "polls must be >= 0 (0: the default bound)");
    c->wait_limit = polls;
    CU(cudaMemcpyAsync(&c->dBar->limit, &c->wait_limit, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    if (c->nn) nn_gate_set_wait_limit(c->nn, polls);
    return 0;
}

int gpmood_set_nn_repair(gpmood_ctx* c, int on) {
    if (!c) return fail(nullptr, GPMOOD_E_ARG, "ctx is NULL");
    c->nn_repair = on != 0;
    return 0;
}

int gpmood_set_nn_threshold(gpmood_ctx* c, float thr) {
    if (!c) return fail(nullptr, GPMOOD_E_ARG, "ctx is NULL");
    nn_gate_set_threshold(c->nn, thr);
    return 0;
}

int gpmood_nn_predict(gpmood_ctx* c, signed char* gated, long long* n_gated) {
    if (!c || !gated) return fail(c, GPMOOD_E_ARG, "NULL argument");
    if (!c->have_state) return fail(c, GPMOOD_E_STATE, "no device-resident state (call gpmood_set_state)");
    const bool ref = c->p.nn_reference != 0;
    if (ref ? !nn_ref_loaded(c->nnref) : !nn_gate_loaded(c->nn))
        return fail(c, GPMOOD_E_STATE, "no network parameters (gpmood_set_nn)");
    CU(cudaMemsetAsync(c->dOrder, c->p.mord, c->ncell, c->stream));
    CU(cudaMemsetAsync(&c->dSc->apriori_step, 0, sizeof(unsigned long long), c->stream));
    CU(cudaMemsetAsync(c->dSc->ntrb, 0, sizeof(c->dSc->ntrb), c->stream));
    if ((ref ? nn_ref_orders(c->nnref, c->g, c->dU, c->dOrder, &c->dSc->apriori_step, nullptr,
                             c->cc ? c->dCcw : nullptr, c->stream)
             : nn_gate_orders(c->nn, c->g, c->dU, c->dOrder, &c->dSc->apriori_step, c->dList[1], &c->dSc->ntrb[1],
                              nullptr, &c->dSc->status, c->stream)) < 0)
        return fail(c, GPMOOD_E_CUDA, "NN gate: %s", cudaGetErrorString(cudaGetLastError()));
    CU(cudaMemcpy2DAsync(gated, (size_t)c->p.lf, c->dOrder + (size_t)GPM_NGC * c->g.nx + GPM_NGC, (size_t)c->g.nx,
                         (size_t)c->p.lf, (size_t)c->p.nf, cudaMemcpyDeviceToHost, c->stream));
    unsigned long long cnt = 0;
    int st = 0;
    CU(cudaMemcpyAsync(&cnt, &c->dSc->apriori_step, sizeof cnt, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(&st, &c->dSc->status, sizeof st, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    if (st & GPM_STATUS_TENSOR) return fail(c, GPMOOD_E_CUDA, "NN gate: tensor-core wait timed out");
    const size_t nint = (size_t)c->p.lf * c->p.nf;
    for (size_t i = 0; i < nint; i++) gated[i] = (ref ? gated[i] == 1 : gated[i] < c->p.mord) ? 1 : 0;
    if (n_gated) *n_gated = (long long)cnt;
    return 0;
}

int gpmood_get_stage_orders(gpmood_ctx* c, int stage, signed char* orders) {
    if (!c || !orders) return fail(c, GPMOOD_E_ARG, "NULL argument");
    if (stage < 0 || stage >= c->nstages) return fail(c, GPMOOD_E_ARG, "stage must be in 0..%d", c->nstages - 1);
    CU(cudaMemcpy2DAsync(orders, (size_t)c->p.lf,
                         c->dStageOrd + (size_t)stage * c->ncell + (size_t)GPM_NGC * c->g.nx + GPM_NGC,
                         (size_t)c->g.nx, (size_t)c->p.lf, (size_t)c->p.nf, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return 0;
}

int gpmood_nn_features(gpmood_ctx* c, float* d_x, signed char* d_const) {
    if (!c || !d_x) return fail(c, GPMOOD_E_ARG, "NULL argument");
    if (!c->have_state) return fail(c, GPMOOD_E_STATE, "no device-resident state (call gpmood_set_state)");
    if (nn_features(c->g, c->dU, d_x, reinterpret_cast<int8_t*>(d_const), c->stream))
        return fail(c, GPMOOD_E_CUDA, "features: %s", cudaGetErrorString(cudaGetLastError()));
    CU(cudaStreamSynchronize(c->stream));
    return 0;
}

int gpmood_nn_harvest(gpmood_ctx* c, float* d_x, float* d_y, int capacity, float keep_negative, unsigned seed,
                      int* d_count) {
    if (!c) return fail(nullptr, GPMOOD_E_ARG, "ctx is NULL");
    if (!d_x) {
        c->hvX = nullptr;
        c->hvY = nullptr;
        c->hvCount = nullptr;
        return 0;
    }
    if (!d_y || !d_count || capacity <= 0 || !(keep_negative >= 0.f && keep_negative <= 1.f))
        return fail(c, GPMOOD_E_ARG, "harvest needs d_y, d_count, capacity > 0 and keep_negative in [0,1]");
    c->hvX = d_x;
    c->hvY = d_y;
    c->hvCount = d_count;
    c->hvCap = capacity;
    c->hvKeep = keep_negative;
    c->hvSeed = seed;
    return 0;
}

int gpmood_nn_forward(const float* d_params, const float* d_x, int n, float* d_logits, void* stream) {
    if (!d_params || !d_x || !d_logits || n <= 0) return fail(nullptr, GPMOOD_E_ARG, "bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nn_forward(d_params, d_x, n, d_logits, s)) return fail(nullptr, GPMOOD_E_CUDA, "nn forward launch failed");
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(nullptr, GPMOOD_E_CUDA, "nn forward: %s", cudaGetErrorString(e));
    return 0;
}

int gpmood_nn_loss_grad(const float* d_params, const float* d_x, const float* d_y, int n, float pos_weight,
                        float* d_grad, float* d_loss, void* stream) {
    if (!d_params || !d_x || !d_y || !d_grad || !d_loss || n <= 0) return fail(nullptr, GPMOOD_E_ARG, "bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nn_loss_grad(d_params, d_x, d_y, n, pos_weight, d_grad, d_loss, s))
        return fail(nullptr, GPMOOD_E_CUDA, "nn loss/grad launch failed");
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(nullptr, GPMOOD_E_CUDA, "nn loss/grad: %s", cudaGetErrorString(e));
    return 0;
}

int gpmood_nn_adam(float* d_params, const float* d_grad, float* d_m, float* d_v, int step, float lr, float beta1,
                   float beta2, float eps, void* stream) {
    if (!d_params || !d_grad || !d_m || !d_v || step < 1) return fail(nullptr, GPMOOD_E_ARG, "bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nn_adam(d_params, d_grad, d_m, d_v, step, lr, beta1, beta2, eps, s))
        return fail(nullptr, GPMOOD_E_CUDA, "adam launch failed");
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(nullptr, GPMOOD_E_CUDA, "adam: %s", cudaGetErrorString(e));
    return 0;
}

}  // extern "C"

// ===========================================================================
// Adjoint of the step with frozen MOOD order masks (adjoint.cu for the stage
// VJP).  A step n -> n+1 with stage inputs X0 = U_n, X1, X2 is
//   X1 = S0(X0),  X2 = 3/4 X0 + 1/4 S1(X1),  U_{n+1} = 1/3 X0 + 2/3 S2(X2)
// (mod_SSP_RK3.f90:12-39), each S a Forward_Euler stage at its recorded
// orders and the step's dt.  Backward:
//   l2 = S2^T(2/3 l),  l1 = S1^T(1/4 l2),  l_n = 1/3 l + 3/4 l2 + S0^T(l1).
#include "adjoint.h"

struct gpmood_adjoint {
    gpmood_ctx* c;
    int nsteps, every, nck;
    double *t, *dt;              // host, per step
    int8_t* dOrd;                // nsteps x 3 x ncell frozen CellGPO
    double* dCk;                 // nck checkpoints (U_{k*every})
    double* dSeg;                // 3*every+1 stage inputs of one segment
    double *dLam, *dLamB, *dTA, *dAcc, *dTmp, *dMu, *dFace;
    DevScalars* dStepSc;         // per step: t, dt, dt/dx, dt/dy of the recording
};

namespace {

double* adj_state(gpmood_adjoint* a, double* base, int i) { return base + (size_t)i * a->c->ncell * 4; }

// One Forward_Euler stage at frozen orders: Boundary_C(uin), fluxes at
// min(CellGPO) per face, flux-difference update without DETECTION, Boundary_C(uout).
void adj_frozen_stage(gpmood_adjoint* a, int step, double* uin, double* uout, const int8_t* ord, int stage) {
    gpmood_ctx* c = a->c;
    const KernelTable& kt = *c->kt;
    DevScalars* sc = a->dStepSc + step;
    StageArgs sa = stage_args(c, uin, uout, stage, false);
    sa.g.method = GPMOOD_GP_SE;  // no DETECTION
    sa.order = const_cast<int8_t*>(ord);
    sa.sc = sc;
    kt.bc(c->g, uin, sc, stage, c->stream);
    kt.flux_all(sa, c->w, c->stream);
    kt.update_detect(sa, c->w, 0, c->stream);
    kt.bc(c->g, uout, sc, stage, c->stream);
}

const int8_t* adj_ord(const gpmood_adjoint* a, int step, int stage) {
    return a->dOrd + ((size_t)step * 3 + stage) * a->c->ncell;
}

// Step `step` from x0 (its ghosts are refreshed in place) into next, keeping
// the stage inputs X1, X2 in x1, x2.
int adj_replay_step(gpmood_adjoint* a, int step, double* x0, double* x1, double* x2, double* next) {
    gpmood_ctx* c = a->c;
    adj_frozen_stage(a, step, x0, x1, adj_ord(a, step, 0), 0);
    adj_frozen_stage(a, step, x1, x2, adj_ord(a, step, 1), 1);
    c->kt->combine(c->g, x0, x2, 0.75, 0.25, 0, a->dStepSc, c->stream);
    adj_frozen_stage(a, step, x2, next, adj_ord(a, step, 2), 2);
    c->kt->combine(c->g, x0, next, 1. / 3, 2. / 3, 0, a->dStepSc, c->stream);
    return check_launch(c, "adjoint replay");
}

// lam_in = S^T(lam_out) at the stage input x with the frozen orders of (step, stage).
int adj_stage_vjp(gpmood_adjoint* a, int step, int stage, const double* x, const double* lam_out, double* lam_in) {
    gpmood_ctx* c = a->c;
    AdjArgs aa;
    aa.g = c->g;
    aa.u_in = x;
    aa.order = adj_ord(a, step, stage);
    aa.lam_out = lam_out;
    aa.lam_in = lam_in;
    aa.face_adj = a->dFace;
    aa.mu_pad = a->dMu;
    aa.qx = a->dt[step] / c->g.dx;
    aa.qy = a->dt[step] / c->g.dy;
    if (gpm_adj_stage(aa, c->w, c->stream)) return fail(c, GPMOOD_E_CUDA, "adjoint stage launch failed");
    return 0;
}

void adj_free(gpmood_adjoint* a) {
    if (!a) return;
    delete[] a->t;
    delete[] a->dt;
    cudaFree(a->dOrd); cudaFree(a->dCk); cudaFree(a->dSeg);
    cudaFree(a->dLam); cudaFree(a->dLamB); cudaFree(a->dTA); cudaFree(a->dAcc); cudaFree(a->dTmp);
    cudaFree(a->dMu); cudaFree(a->dFace); cudaFree(a->dStepSc);
    delete a;
}

}  // namespace

extern "C" {

int gpmood_adj_record(gpmood_ctx* c, int nsteps, int every, gpmood_adjoint** out) {
    if (!c || !out) return fail(c, GPMOOD_E_ARG, "NULL argument");
    *out = nullptr;
    if (nsteps < 1 || every < 1) return fail(c, GPMOOD_E_ARG, "nsteps and every must be >= 1");
    if (!c->have_state) return fail(c, GPMOOD_E_STATE, "no device-resident state (call gpmood_set_state)");
    if (c->p.bc_type == GPMOOD_DMR)
        return fail(c, GPMOOD_E_ARG, "adjoint: BC_type DMR (time-dependent inflow) is not supported");
    if (c->p.integrator != GPMOOD_SSP_RK3 || c->p.num_flux != GPMOOD_HLLC)
        return fail(c, GPMOOD_E_ARG, "adjoint: only SSP_RK3 with HLLC");
    gpmood_adjoint* a = new (std::nothrow) gpmood_adjoint();
    if (!a) return fail(c, GPMOOD_E_ARG, "out of host memory");
    a->c = c;
    a->every = every;
    a->nck = (nsteps + every - 1) / every;
    a->t = new (std::nothrow) double[nsteps];
    a->dt = new (std::nothrow) double[nsteps];
    const size_t sb = state_bytes(c);
    bool ok = a->t && a->dt;
#define AALLOC(ptr, bytes) ok = ok && cudaMalloc((void**)&(ptr), (bytes)) == cudaSuccess
    AALLOC(a->dOrd, (size_t)nsteps * 3 * c->ncell);
    AALLOC(a->dCk, (size_t)a->nck * sb);
    AALLOC(a->dSeg, (size_t)(3 * every + 1) * sb);
    AALLOC(a->dLam, sb);
    AALLOC(a->dLamB, sb);
    AALLOC(a->dTA, sb);
    AALLOC(a->dAcc, sb);
    AALLOC(a->dTmp, sb);
    AALLOC(a->dMu, sb);
    AALLOC(a->dFace, 2 * c->ncell * 8 * GPM_MAXGP * sizeof(double));
    AALLOC(a->dStepSc, (size_t)nsteps * sizeof(DevScalars));
#undef AALLOC
    if (ok) {  // adjoint buffers keep zero ghosts for their whole life
        cudaStream_t s = c->stream;
        ok = cudaMemsetAsync(a->dLam, 0, sb, s) == cudaSuccess && cudaMemsetAsync(a->dLamB, 0, sb, s) == cudaSuccess &&
             cudaMemsetAsync(a->dTA, 0, sb, s) == cudaSuccess && cudaMemsetAsync(a->dAcc, 0, sb, s) == cudaSuccess &&
             cudaMemsetAsync(a->dTmp, 0, sb, s) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess;
    }
    if (!ok) {
        adj_free(a);
        return fail(c, GPMOOD_E_CUDA, "adjoint: allocation failed");
    }
    int done = 0;
    for (int s = 0; s < nsteps; s++) {
        if (s % every == 0) {
            cudaError_t e = cudaMemcpyAsync(adj_state(a, a->dCk, s / every), c->dU, sb, cudaMemcpyDeviceToDevice, c->stream);
            if (e != cudaSuccess) { adj_free(a); return fail(c, GPMOOD_E_CUDA, "adjoint checkpoint: %s", cudaGetErrorString(e)); }
        }
        int one = 0;
        int rc = gpmood_advance(c, 1, &one);
        if (rc) { adj_free(a); return rc; }
        if (!one) break;  // tmax or nmax reached
        a->t[s] = c->hSc->t;
        a->dt[s] = c->hSc->dt;
        cudaError_t e = cudaMemcpyAsync(a->dOrd + (size_t)s * 3 * c->ncell, c->dStageOrd, 3 * c->ncell,
                                        cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) { adj_free(a); return fail(c, GPMOOD_E_CUDA, "adjoint orders: %s", cudaGetErrorString(e)); }
        done++;
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) { adj_free(a); return fail(c, GPMOOD_E_CUDA, "adjoint record sync"); }
    if (done == 0) { adj_free(a); return fail(c, GPMOOD_E_STATE, "adjoint: no step taken (t >= tmax)"); }
    // per-step scalars on the device, so that replays never wait on the host
    DevScalars* hs = new (std::nothrow) DevScalars[done]();
    if (!hs) { adj_free(a); return fail(c, GPMOOD_E_ARG, "out of host memory"); }
    for (int s = 0; s < done; s++) {
        hs[s].t = a->t[s];
        hs[s].dt = a->dt[s];
        hs[s].qx = a->dt[s] / c->g.dx;  // the division of k_dt_finalize
        hs[s].qy = a->dt[s] / c->g.dy;
    }
    const cudaError_t es = cudaMemcpy(a->dStepSc, hs, (size_t)done * sizeof(DevScalars), cudaMemcpyHostToDevice);
    delete[] hs;
    if (es != cudaSuccess) { adj_free(a); return fail(c, GPMOOD_E_CUDA, "adjoint scalars: %s", cudaGetErrorString(es)); }
    a->nsteps = done;
    a->nck = (done + every - 1) / every;
    *out = a;
    return 0;
}

void gpmood_adj_destroy(gpmood_adjoint* a) { adj_free(a); }

int gpmood_adj_info(const gpmood_adjoint* a, int* nsteps, double* t, double* dt) {
    if (!a) return fail(nullptr, GPMOOD_E_ARG, "adjoint is NULL");
    if (nsteps) *nsteps = a->nsteps;
    if (t) memcpy(t, a->t, (size_t)a->nsteps * sizeof(double));
    if (dt) memcpy(dt, a->dt, (size_t)a->nsteps * sizeof(double));
    return 0;
}

int gpmood_adj_orders(const gpmood_adjoint* a, int step, int stage, signed char* orders_host) {
    if (!a || !orders_host) return fail(a ? a->c : nullptr, GPMOOD_E_ARG, "NULL argument");
    gpmood_ctx* c = a->c;
    if (step < 0 || step >= a->nsteps || stage < 0 || stage > 2) return fail(c, GPMOOD_E_ARG, "step/stage out of range");
    CU(cudaMemcpyAsync(orders_host, adj_ord(a, step, stage), c->ncell, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return 0;
}

int gpmood_adj_replay(gpmood_adjoint* a, const double* d_u0, double* d_uN) {
    if (!a || !d_u0 || !d_uN) return fail(a ? a->c : nullptr, GPMOOD_E_ARG, "NULL argument");
    gpmood_ctx* c = a->c;
    const size_t sb = state_bytes(c);
    double *x0 = adj_state(a, a->dSeg, 0), *x1 = adj_state(a, a->dSeg, 1), *x2 = adj_state(a, a->dSeg, 2);
    double* nx = adj_state(a, a->dSeg, 3);
    CU(cudaMemcpyAsync(x0, d_u0, sb, cudaMemcpyDeviceToDevice, c->stream));
    for (int s = 0; s < a->nsteps; s++) {
        int rc = adj_replay_step(a, s, x0, x1, x2, nx);
        if (rc) return rc;
        double* tmp = x0;
        x0 = nx;
        nx = tmp;
    }
    CU(cudaMemcpyAsync(d_uN, x0, sb, cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return 0;
}

int gpmood_adj_backward(gpmood_adjoint* a, const double* d_lamN, double* d_lam0) {
    if (!a || !d_lamN || !d_lam0) return fail(a ? a->c : nullptr, GPMOOD_E_ARG, "NULL argument");
    gpmood_ctx* c = a->c;
    cudaStream_t st = c->stream;
    const size_t sb = state_bytes(c);
    const KernelTable& kt = *c->kt;
    // U_N's ghosts are Boundary_C of its interior: fold their adjoint in.
    CU(cudaMemcpyAsync(a->dMu, d_lamN, sb, cudaMemcpyDeviceToDevice, st));
    CU(cudaMemsetAsync(a->dTmp, 0, sb, st));
    if (gpm_adj_fold(c->g, a->dMu, a->dTmp, a->dLam, st)) return fail(c, GPMOOD_E_CUDA, "adjoint fold launch failed");
    for (int seg = a->nck - 1; seg >= 0; seg--) {
        const int s0 = seg * a->every, s1 = s0 + a->every < a->nsteps ? s0 + a->every : a->nsteps;
        // recompute the segment's stage inputs from its checkpoint
        CU(cudaMemcpyAsync(adj_state(a, a->dSeg, 0), adj_state(a, a->dCk, seg), sb, cudaMemcpyDeviceToDevice, st));
        for (int s = s0; s < s1; s++) {
            const int i = 3 * (s - s0);
            int rc = adj_replay_step(a, s, adj_state(a, a->dSeg, i), adj_state(a, a->dSeg, i + 1),
                                     adj_state(a, a->dSeg, i + 2), adj_state(a, a->dSeg, i + 3));
            if (rc) return rc;
        }
        for (int s = s1 - 1; s >= s0; s--) {
            const int i = 3 * (s - s0);
            const double *x0 = adj_state(a, a->dSeg, i), *x1 = adj_state(a, a->dSeg, i + 1);
            const double* x2 = adj_state(a, a->dSeg, i + 2);
            CU(cudaMemcpyAsync(a->dTA, a->dLam, sb, cudaMemcpyDeviceToDevice, st));
            kt.combine(c->g, a->dLam, a->dTA, 0.0, 2. / 3, 0, a->dStepSc, st);      // TA = 2/3 l
            int rc = adj_stage_vjp(a, s, 2, x2, a->dTA, a->dLamB);             // l2
            if (rc) return rc;
            CU(cudaMemcpyAsync(a->dAcc, a->dLam, sb, cudaMemcpyDeviceToDevice, st));
            kt.combine(c->g, a->dLamB, a->dAcc, 0.75, 1. / 3, 0, a->dStepSc, st);  // acc = 1/3 l + 3/4 l2
            CU(cudaMemcpyAsync(a->dTA, a->dLamB, sb, cudaMemcpyDeviceToDevice, st));
            kt.combine(c->g, a->dLamB, a->dTA, 0.0, 0.25, 0, a->dStepSc, st);     // TA = 1/4 l2
            rc = adj_stage_vjp(a, s, 1, x1, a->dTA, a->dLamB);                 // l1
            if (rc) return rc;
            rc = adj_stage_vjp(a, s, 0, x0, a->dLamB, a->dTmp);                // S0^T(l1)
            if (rc) return rc;
            kt.combine(c->g, a->dAcc, a->dTmp, 1.0, 1.0, 0, a->dStepSc, st);      // l_s = acc + S0^T(l1)
            double* tmp = a->dLam;
            a->dLam = a->dTmp;
            a->dTmp = tmp;
            rc = check_launch(c, "adjoint step");
            if (rc) return rc;
        }
    }
    CU(cudaMemcpyAsync(d_lam0, a->dLam, sb, cudaMemcpyDeviceToDevice, st));
    CU(cudaStreamSynchronize(st));
    return 0;
}

}  // extern "C"
