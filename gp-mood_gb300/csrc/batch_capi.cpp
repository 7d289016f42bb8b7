// batch_capi.cpp -- C ABI of the batched path: many independent problems of
// uneven size stepped together on one GPU (include/gpmood.h, gpmood_batch_*).
//
// Each phase of an RK stage is one persistent launch over every problem's
// work items and the MOOD loop is one cooperative launch per stage, so a step
// is a fixed sequence of ~30 launches.  That sequence is captured once into a
// CUDA graph per state-buffer parity (U -> Ur and Ur -> U) and replayed; every
// problem advances with its own CFL time step.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "../../include/gpmood.h"
#include "batch_common.h"

void gpm_set_thread_error(const char* msg);

struct gpmood_batch {
    gpmood_params p;
    int nprob;
    std::vector<BProb> hprob;
    long long ncell = 0, ninterior = 0;
    int max_nx = 0;
    BProb* dprob = nullptr;
    GpWeights* dwtab = nullptr;
    BScal* dsc = nullptr;
    BScal* hsc = nullptr;  // pinned
    double *U = nullptr, *Ur = nullptr, *U1 = nullptr, *U2 = nullptr, *Fx = nullptr, *Fy = nullptr;
    int8_t* order = nullptr;
    unsigned* stamp = nullptr;
    int2* list[2] = {nullptr, nullptr};
    int* ntrb = nullptr;
    int* hntrb = nullptr;  // pinned
    GridBar* bar = nullptr;
    GridBar* hbar = nullptr;  // pinned
    int4* ftiles[GPM_NTILES] = {};
    int nft[GPM_NTILES] = {};
    int4* etiles = nullptr;  // edge items of the two-direction cell tiles
    int net = 0;
    int2* cblocks = nullptr;
    int ncb = 0;
    int2* pblocks = nullptr;
    int npb = 0;
    int tile = 0;
    bool xy_ok = false;  // the two-direction cell tile applies (fast mode, order 5, ngp 3)
    const BatchTable* bt = nullptr;
    void (*set_max_nx)(int) = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_state = 0;  // 0 not built, 1 built, -1 capture unsupported (eager launches)
    bool dt_pending = false;
    int parity = 0;  // 0: state in U, 1: state in Ur
    long long steps = 0, detected = 0, status = 0;
    char err[512] = {};
};

namespace {

int bfail(gpmood_batch* b, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (b) memcpy(b->err, buf, sizeof buf);
    gpm_set_thread_error(buf);
    return code;
}

#define BCU(call)                                                                                       \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return bfail(b, GPMOOD_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

BatchArgs make_args(gpmood_batch* b, const double* uin, double* uout, int stage) {
    BatchArgs a;
    memset(&a, 0, sizeof a);
    a.prob = b->dprob;
    a.wtab = b->dwtab;
    a.sc = b->dsc;
    a.nprob = b->nprob;
    a.bc_type = b->p.bc_type;
    a.ngp = b->p.ngp;
    a.mord = b->p.mord;
    a.method = b->p.method;
    a.dmp = b->p.dmp;
    a.u2 = b->p.u2;
    a.u2_tol = b->p.u2_tol;
    a.num_flux = b->p.num_flux;
    a.uin = uin;
    a.uout = uout;
    a.fx = b->Fx;
    a.fy = b->Fy;
    a.order = b->order;
    a.stamp = b->stamp;
    a.tlist[0] = b->list[0];
    a.tlist[1] = b->list[1];
    a.ntrb = b->ntrb;
    a.ftiles = b->ftiles[b->tile];
    a.nftiles = b->nft[b->tile];
    a.etiles = b->etiles;
    a.netiles = b->net;
    a.cblocks = b->cblocks;
    a.ncblocks = b->ncb;
    a.pblocks = b->pblocks;
    a.npblocks = b->npb;
    a.stage = stage;
    a.tile = b->tile;
    a.mood_solo = gpm_mood_solo_default();
    return a;
}

int batch_stage(gpmood_batch* b, double* uin, double* uout, int stage) {
    cudaStream_t s = b->stream;
    const BatchArgs a = make_args(b, uin, uout, stage);
    b->bt->bc(a, uin, s);
    BCU(cudaMemsetAsync(b->order, b->p.mord, (size_t)b->ncell, s));
    BCU(cudaMemsetAsync(b->ntrb, 0, 2 * sizeof(int), s));
    b->bt->flux(a, s);
    b->bt->update(a, s);
    if (b->p.method == GPMOOD_GP_MOOD) {
        const long long cap = b->p.max_mood_iters > 0 ? b->p.max_mood_iters : 2LL * b->ninterior + 2;
        BCU(cudaMemsetAsync(b->bar, 0, sizeof(GridBar), s));
        if (b->bt->mood_loop(a, b->bar, cap > 0x7fffffff ? 0x7fffffff : (int)cap, s))
            return bfail(b, GPMOOD_E_CUDA, "batched MOOD loop launch: %s", cudaGetErrorString(cudaGetLastError()));
    }
    b->bt->bc(a, uout, s);
    return 0;
}

// One SSP-RK3 step of every problem from u into ur (Setdt of u already reduced).
int batch_step(gpmood_batch* b, double* u, double* ur) {
    cudaStream_t s = b->stream;
    const BatchArgs a0 = make_args(b, u, ur, 0);
    b->bt->dt_finalize(a0, s);
    int rc = batch_stage(b, u, b->U1, 0);
    if (!rc) rc = batch_stage(b, b->U1, b->U2, 1);
    if (rc) return rc;
    b->bt->combine(a0, u, b->U2, 0.75, 0.25, 0, s);
    rc = batch_stage(b, b->U2, ur, 2);
    if (rc) return rc;
    b->bt->combine(a0, u, ur, 1. / 3, 2. / 3, 1, s);  // with the next step's per-problem Setdt
    b->bt->advance_t(a0, s);
    return 0;
}

int build_graphs(gpmood_batch* b) {
    for (int par = 0; par < 2; par++) {
        if (b->graph[par]) {
            cudaGraphExecDestroy(b->graph[par]);
            b->graph[par] = nullptr;
        }
    }
    for (int par = 0; par < 2; par++) {
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return -1;
        const int rc = par == 0 ? batch_step(b, b->U, b->Ur) : batch_step(b, b->Ur, b->U);
        const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (rc || e != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return -1;
        }
        const cudaError_t ei = cudaGraphInstantiate(&b->graph[par], g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            cudaGetLastError();
            return -1;
        }
    }
    return 0;
}

void free_batch(gpmood_batch* b) {
    for (int par = 0; par < 2; par++)
        if (b->graph[par]) cudaGraphExecDestroy(b->graph[par]);
    cudaFree(b->dprob); cudaFree(b->dwtab); cudaFree(b->dsc);
    cudaFree(b->U); cudaFree(b->Ur); cudaFree(b->U1); cudaFree(b->U2); cudaFree(b->Fx); cudaFree(b->Fy);
    cudaFree(b->order); cudaFree(b->stamp); cudaFree(b->list[0]); cudaFree(b->list[1]);
    cudaFree(b->ntrb); cudaFree(b->bar); cudaFree(b->cblocks); cudaFree(b->pblocks);
    for (int k = 0; k < GPM_NTILES; k++) cudaFree(b->ftiles[k]);
    cudaFree(b->etiles);
    if (b->hsc) cudaFreeHost(b->hsc);
    if (b->hntrb) cudaFreeHost(b->hntrb);
    if (b->hbar) cudaFreeHost(b->hbar);
    if (b->stream) cudaStreamDestroy(b->stream);
}

}  // namespace

extern "C" {

int gpmood_batch_create(const gpmood_params* p, int nprob, const int* lf, const int* nf, gpmood_batch** out) {
    gpmood_batch* b = nullptr;
    if (!p || !lf || !nf || !out || nprob < 1) return bfail(nullptr, GPMOOD_E_ARG, "bad batch arguments");
    *out = nullptr;
    if (p->method != GPMOOD_GP_MOOD && p->method != GPMOOD_GP_SE)
        return bfail(nullptr, GPMOOD_E_ARG, "batched method must be GP_MOOD (2) or GP_SE (202)");
    if (p->bc_type != GPMOOD_NEUMANN && p->bc_type != GPMOOD_PERIODIC && p->bc_type != GPMOOD_REFLECTIVE)
        return bfail(nullptr, GPMOOD_E_ARG, "batched BC_type must be Neumann, periodic or reflective");
    if (p->integrator != GPMOOD_SSP_RK3 || p->num_flux < GPMOOD_HLLC || p->num_flux > GPMOOD_UNSPLIT ||
        !(p->mord == 1 || p->mord == 3 || p->mord == 5) ||
        p->ngp < 1 || p->ngp > 5 || (p->fp_mode != GPMOOD_FP_EXACT && p->fp_mode != GPMOOD_FP_FAST) ||
        p->max_mood_iters < 0 || !(p->cfl > 0) || !(p->lx > 0) || !(p->ly > 0) || !(p->ell_o_dx > 0))
        return bfail(nullptr, GPMOOD_E_ARG, "unsupported batch knobs");
    for (int i = 0; i < nprob; i++)
        if (lf[i] < 4 || nf[i] < 4 || lf[i] > 16384 || nf[i] > 16384)
            return bfail(nullptr, GPMOOD_E_ARG, "problem %d: grid %dx%d out of range", i, lf[i], nf[i]);
    b = new (std::nothrow) gpmood_batch();
    if (!b) return bfail(nullptr, GPMOOD_E_ARG, "out of host memory");
    b->p = *p;
    b->nprob = nprob;
    b->bt = p->fp_mode == GPMOOD_FP_FAST ? &gpm_fast::batch_table : &gpm_exact::batch_table;
    b->xy_ok = p->fp_mode == GPMOOD_FP_FAST && p->mord == 5 && p->ngp == 3 && p->num_flux == GPMOOD_HLLC;
    b->tile = b->xy_ok ? GPM_TILE_XY : 0;  // the single-problem path's first pass
    b->set_max_nx = p->fp_mode == GPMOOD_FP_FAST ? gpm_fast::batch_set_max_nx : gpm_exact::batch_set_max_nx;

    // problems, weight classes (one GP weight set per distinct grid size)
    std::vector<std::pair<int, int>> sizes;
    std::vector<GpWeights> wts;
    b->hprob.resize(nprob);
    long long off = 0;
    for (int i = 0; i < nprob; i++) {
        BProb& q = b->hprob[i];
        q.off = off;
        q.lf = lf[i];
        q.nf = nf[i];
        q.nx = lf[i] + 2 * GPM_NGC;
        q.ny = nf[i] + 2 * GPM_NGC;
        q.dx = gpm_cell_size(p->lx, lf[i]);
        q.dy = gpm_cell_size(p->ly, nf[i]);
        auto it = std::find(sizes.begin(), sizes.end(), std::make_pair(lf[i], nf[i]));
        if (it == sizes.end()) {
            GpWeights w;
            double ie[3];
            if (gpm_gp_presim(p->ell_o_dx, p->lx, p->ly, lf[i], nf[i], p->mord, p->ngp, &w, ie)) {
                delete b;
                return bfail(nullptr, GPMOOD_E_ARG, "GP precompute rejected the knobs");
            }
            sizes.push_back(std::make_pair(lf[i], nf[i]));
            wts.push_back(w);
            q.wc = (int)wts.size() - 1;
        } else {
            q.wc = (int)(it - sizes.begin());
        }
        q.pad = 0;
        off += (long long)q.nx * q.ny;
        b->ninterior += (long long)lf[i] * nf[i];
        b->max_nx = std::max(b->max_nx, std::max(q.nx, q.ny));
    }
    b->ncell = off;

    // work lists; big problems first so the persistent CTAs finish together
    std::vector<int> ord(nprob);
    for (int i = 0; i < nprob; i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
        return (long long)lf[x] * nf[x] > (long long)lf[y] * nf[y];
    });
    std::vector<int4> ft[GPM_NTILES];
    std::vector<int4> et;  // edge items of the two-direction cell tiles
    for (int i : ord) {  // two-direction cell tiles over the interior, and 32-face edge items
        for (int n0 = 1; n0 <= nf[i]; n0 += kTileTY[GPM_TILE_XY])
            for (int l0 = 1; l0 <= lf[i]; l0 += kTileTX[GPM_TILE_XY]) ft[GPM_TILE_XY].push_back(make_int4(i, 2, l0, n0));
        for (int k0 = 0; k0 < lf[i] + nf[i]; k0 += 32)  // one warp of edge faces per item
            et.push_back(make_int4(i, 3, k0, 0));
    }
    for (int k = 0; k < GPM_NTILES; k++) {
        if (k == GPM_TILE_XY) continue;
        for (int i : ord) {
            const int TX = kTileTX[k], TY = kTileTY[k];
            for (int n0 = 1; n0 <= nf[i]; n0 += TY)
                for (int l0 = 0; l0 <= lf[i]; l0 += TX) ft[k].push_back(make_int4(i, 0, l0, n0));
            for (int n0 = 0; n0 <= nf[i]; n0 += TY)
                for (int l0 = 1; l0 <= lf[i]; l0 += TX) ft[k].push_back(make_int4(i, 1, l0, n0));
        }
    }
    std::vector<int2> cb, pb;
    for (int i : ord) {
        for (int k = 0; k < lf[i] * nf[i]; k += 256) cb.push_back(make_int2(i, k));
        for (int k = 0; k < b->hprob[i].nx * b->hprob[i].ny; k += 256) pb.push_back(make_int2(i, k));
    }
    b->ncb = (int)cb.size();
    b->npb = (int)pb.size();

#define BALLOC(ptr, bytes)                                                                                  \
    do {                                                                                                    \
        if (cudaMalloc((void**)&(ptr), (bytes)) != cudaSuccess) {                                           \
            bfail(b, GPMOOD_E_CUDA, "cudaMalloc(%zu) failed", (size_t)(bytes));                             \
            free_batch(b);                                                                                  \
            delete b;                                                                                       \
            return GPMOOD_E_CUDA;                                                                           \
        }                                                                                                   \
    } while (0)
    const size_t sb = (size_t)b->ncell * 32;
    BALLOC(b->dprob, sizeof(BProb) * nprob);
    BALLOC(b->dwtab, sizeof(GpWeights) * wts.size());
    BALLOC(b->dsc, sizeof(BScal) * nprob);
    BALLOC(b->U, sb);
    BALLOC(b->Ur, sb);
    BALLOC(b->U1, sb);
    BALLOC(b->U2, sb);
    BALLOC(b->Fx, sb);
    BALLOC(b->Fy, sb);
    BALLOC(b->order, (size_t)b->ncell);
    BALLOC(b->stamp, (size_t)b->ncell * sizeof(unsigned));
    BALLOC(b->list[0], (size_t)b->ninterior * sizeof(int2));
    BALLOC(b->list[1], (size_t)b->ninterior * sizeof(int2));
    BALLOC(b->ntrb, 8 * sizeof(int));
    BALLOC(b->bar, sizeof(GridBar));
    BALLOC(b->cblocks, sizeof(int2) * cb.size());
    BALLOC(b->pblocks, sizeof(int2) * pb.size());
    for (int k = 0; k < GPM_NTILES; k++) {
        BALLOC(b->ftiles[k], sizeof(int4) * ft[k].size());
        b->nft[k] = (int)ft[k].size();
    }
    BALLOC(b->etiles, sizeof(int4) * et.size());
    b->net = (int)et.size();
#undef BALLOC
    if (cudaMallocHost((void**)&b->hsc, sizeof(BScal) * nprob) != cudaSuccess ||
        cudaMallocHost((void**)&b->hntrb, 8 * sizeof(int)) != cudaSuccess ||
        cudaMallocHost((void**)&b->hbar, sizeof(GridBar)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        bfail(b, GPMOOD_E_CUDA, "pinned memory / stream creation failed");
        free_batch(b);
        delete b;
        return GPMOOD_E_CUDA;
    }
    for (int i = 0; i < nprob; i++) {
        BScal& sc = b->hsc[i];
        memset(&sc, 0, sizeof sc);
        sc.tmax = p->tmax;
        sc.cfl = p->cfl;
        sc.dtmin_bits = 0x46293e5939a08ceaULL;  // bits of 1.0e30
    }
    cudaStream_t s = b->stream;
    bool ok = cudaMemcpyAsync(b->dprob, b->hprob.data(), sizeof(BProb) * nprob, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(b->dwtab, wts.data(), sizeof(GpWeights) * wts.size(), cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(b->dsc, b->hsc, sizeof(BScal) * nprob, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(b->cblocks, cb.data(), sizeof(int2) * cb.size(), cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(b->pblocks, pb.data(), sizeof(int2) * pb.size(), cudaMemcpyHostToDevice, s) == cudaSuccess;
    for (int k = 0; ok && k < GPM_NTILES; k++)
        ok = cudaMemcpyAsync(b->ftiles[k], ft[k].data(), sizeof(int4) * ft[k].size(), cudaMemcpyHostToDevice, s) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(b->etiles, et.data(), sizeof(int4) * et.size(), cudaMemcpyHostToDevice, s) == cudaSuccess;
    ok = ok && cudaMemsetAsync(b->U, 0, sb, s) == cudaSuccess && cudaMemsetAsync(b->Ur, 0, sb, s) == cudaSuccess &&
         cudaMemsetAsync(b->U1, 0, sb, s) == cudaSuccess && cudaMemsetAsync(b->U2, 0, sb, s) == cudaSuccess &&
         cudaMemsetAsync(b->Fx, 0, sb, s) == cudaSuccess && cudaMemsetAsync(b->Fy, 0, sb, s) == cudaSuccess &&
         cudaMemsetAsync(b->stamp, 0, (size_t)b->ncell * sizeof(unsigned), s) == cudaSuccess &&
         cudaMemsetAsync(b->ntrb, 0, 8 * sizeof(int), s) == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess;
    if (!ok) {
        bfail(b, GPMOOD_E_CUDA, "batch initialisation failed: %s", cudaGetErrorString(cudaGetLastError()));
        free_batch(b);
        delete b;
        return GPMOOD_E_CUDA;
    }
    b->set_max_nx(b->max_nx);
    *out = b;
    return 0;
}

void gpmood_batch_destroy(gpmood_batch* b) {
    if (!b) return;
    cudaStreamSynchronize(b->stream);
    free_batch(b);
    delete b;
}

int gpmood_batch_set_state(gpmood_batch* b, int i, const double* u_host, double t) {
    if (!b || !u_host || i < 0 || i >= b->nprob) return bfail(b, GPMOOD_E_ARG, "bad arguments");
    const BProb& q = b->hprob[i];
    double* dst = (b->parity == 0 ? b->U : b->Ur) + 4 * q.off;
    BCU(cudaMemcpyAsync(dst, u_host, (size_t)q.nx * q.ny * 32, cudaMemcpyHostToDevice, b->stream));
    BCU(cudaMemcpyAsync(&b->dsc[i].t, &t, sizeof(double), cudaMemcpyHostToDevice, b->stream));
    BCU(cudaStreamSynchronize(b->stream));
    b->dt_pending = false;
    return 0;
}

int gpmood_batch_get_state(gpmood_batch* b, int i, double* u_host, double* t) {
    if (!b || i < 0 || i >= b->nprob) return bfail(b, GPMOOD_E_ARG, "bad arguments");
    const BProb& q = b->hprob[i];
    const double* src = (b->parity == 0 ? b->U : b->Ur) + 4 * q.off;
    if (u_host) BCU(cudaMemcpyAsync(u_host, src, (size_t)q.nx * q.ny * 32, cudaMemcpyDeviceToHost, b->stream));
    BCU(cudaMemcpyAsync(b->hsc, b->dsc, sizeof(BScal) * b->nprob, cudaMemcpyDeviceToHost, b->stream));
    BCU(cudaStreamSynchronize(b->stream));
    if (t) *t = b->hsc[i].t;
    return 0;
}

int gpmood_batch_advance(gpmood_batch* b, int nsteps) {
    if (!b || nsteps < 0) return bfail(b, GPMOOD_E_ARG, "bad arguments");
    cudaStream_t s = b->stream;
    for (int k = 0; k < nsteps; k++) {
        double* u = b->parity == 0 ? b->U : b->Ur;
        double* ur = b->parity == 0 ? b->Ur : b->U;
        if (!b->dt_pending) {  // Setdt of every problem (later steps fuse it into the last combine)
            b->bt->cfl(make_args(b, u, ur, 0), u, s);
        }
        BCU(cudaMemsetAsync(b->ntrb + 3, 0, 3 * sizeof(int), s));
        if (b->graph_state == 0) b->graph_state = build_graphs(b) == 0 ? 1 : -1;
        if (b->graph_state == 1) {
            BCU(cudaGraphLaunch(b->graph[b->parity], s));
        } else {
            const int rc = batch_step(b, u, ur);
            if (rc) return rc;
        }
        BCU(cudaMemcpyAsync(b->hntrb, b->ntrb, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
        BCU(cudaMemcpyAsync(b->hbar, b->bar, sizeof(GridBar), cudaMemcpyDeviceToHost, s));
        BCU(cudaStreamSynchronize(s));
        b->parity ^= 1;
        b->dt_pending = true;
        b->steps++;
        b->detected += b->hntrb[4];
        if (b->hntrb[6]) b->status |= GPM_STATUS_NAN;  // a NaN or inadmissible state left at order 1
        if (b->hbar->err) {  // clear the barrier and the aborted loop's pass stamps; the batch stays usable
            cudaMemsetAsync(b->bar, 0, sizeof(GridBar), s);
            cudaMemsetAsync(b->stamp, 0, (size_t)b->ncell * sizeof(unsigned), s);
            cudaStreamSynchronize(s);
            b->status |= GPM_STATUS_BARRIER;
            return bfail(b, GPMOOD_E_CUDA, "batched MOOD loop: grid barrier timed out");
        }
        if (b->hntrb[3]) {
            b->status |= GPM_STATUS_MOODCAP;
            return bfail(b, GPMOOD_E_MOOD_CAP, "batched MOOD loop hit max_mood_iters");
        }
    }
    return 0;
}

int gpmood_batch_autotune(gpmood_batch* b, int* tile, double* ms_per_tile) {
    if (!b) return bfail(nullptr, GPMOOD_E_ARG, "batch is NULL");
    cudaStream_t s = b->stream;
    cudaEvent_t e0, e1;
    BCU(cudaEventCreate(&e0));
    BCU(cudaEventCreate(&e1));
    double* u = b->parity == 0 ? b->U : b->Ur;
    const BatchArgs a0 = make_args(b, u, b->U1, 0);
    b->bt->bc(a0, u, s);
    int best = 0;
    float best_ms = 1e30f;
    for (int k = 0; k < GPM_NTILES; k++) {
        if (k == GPM_TILE_XY && !b->xy_ok) {
            if (ms_per_tile) ms_per_tile[k] = 0.0;
            continue;
        }
        b->tile = k;
        const BatchArgs a = make_args(b, u, b->U1, 0);
        b->bt->flux(a, s);  // warm-up
        float tot = 0.f;
        for (int r = 0; r < 3; r++) {
            cudaEventRecord(e0, s);
            b->bt->flux(a, s);
            cudaEventRecord(e1, s);
            BCU(cudaEventSynchronize(e1));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            tot += ms;
        }
        const float ms = tot / 3;
        if (ms_per_tile) ms_per_tile[k] = ms;
        if (ms < best_ms) {
            best_ms = ms;
            best = k;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    BCU(cudaGetLastError());
    b->tile = best;
    b->graph_state = 0;  // recapture with the chosen tile
    if (tile) *tile = best;
    return 0;
}

int gpmood_batch_stats(const gpmood_batch* b, long long* interior_cells, long long* steps, long long* detected,
                       long long* status, int* graphed) {
    if (!b) return bfail(nullptr, GPMOOD_E_ARG, "batch is NULL");
    if (interior_cells) *interior_cells = b->ninterior;
    if (steps) *steps = b->steps;
    if (detected) *detected = b->detected;
    if (status) *status = b->status;
    if (graphed) *graphed = b->graph_state;
    return 0;
}

}  // extern "C"
