// noalloc.cu -- one GP-MOOD time step that allocates no memory.
//
// Some callers cannot let a library allocate device memory: a host that owns
// all GPU memory through its own pool (a cudaMalloc would bypass the pool's
// accounting and implicitly synchronise the device), or a real-time loop that
// must not stall in the allocator.  For them gpmood_time_stepping_noalloc runs
// the same SSP-RK3 step as gpmood_time_stepping_dev -- the same kernels,
// including the cooperative MOOD loop -- with every scratch array (RK stage
// buffers, face-flux stores, order mask, MOOD stamps and lists, device
// scalars, the loop's grid barrier) carved out of the file-scope array below
// instead of being allocated.  The caller still passes the input and output
// states.  Nothing here calls cudaMalloc, cudaFree or an allocating library
// routine, and the host side uses no heap either (fixed static tables).
//
// The array is sized for grids of at most GPM_NOALLOC_MAX_CELLS padded cells
// ((lf+8)*(nf+8) <= 264*264, e.g. 256x256), about 10 MB; every GPU that loads
// the library holds it until the process exits.  All calls share it and it
// keeps the last call's contents, so calls that overlap on the GPU (other
// streams, other host threads) race; what must start at zero (the MOOD
// stamps, the grid barrier, the device scalars) is cleared at the start of
// every call.
#include <mutex>
#include <stdio.h>
#include <string.h>

#include <cuda.h>

#include "../../include/gpmood.h"
#include "gpm_common.h"

#define GPM_NOALLOC_MAX_CELLS (264 * 264)
// Bytes per padded cell: U1, U2, Fx, Fy (4 doubles each), order (1), stamp (4), two lists (4 + 4).
#define GPM_NOALLOC_CELL_BYTES (4 * 32 + 1 + 4 + 4 + 4)
#define GPM_NOALLOC_BYTES ((size_t)GPM_NOALLOC_MAX_CELLS * GPM_NOALLOC_CELL_BYTES + 16 * 256)

static __device__ __align__(256) unsigned char g_noalloc_scratch[GPM_NOALLOC_BYTES];

// The knob checks of gpmood_create (gpmood_capi.cpp).
int gpm_validate_params(const gpmood_params* p, char* why, size_t n);

namespace {

// The message goes to the thread's error buffer, read by gpmood_last_error(NULL, ...).
int nerr(int code, const char* msg, const char* detail = nullptr) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s%s%s", msg, detail ? ": " : "", detail ? detail : "");
    gpm_set_thread_error(buf);
    return code;
}

// ---- set-up: the device address of g_noalloc_scratch -----------------------
// In host code the array's name is a host-side stand-in, not a device address,
// so the address is looked up with cudaGetSymbolAddress once per device, with
// that device current, and kept.  The table is keyed on the device and on the
// current context's unique id (cuCtxGetId): a context created after
// cudaDeviceReset, or a non-primary context a host makes current, gets its
// own look-up instead of a stale address.
typedef CUresult(CUDAAPI* CtxGetCurrentFn)(CUcontext*);
typedef CUresult(CUDAAPI* CtxGetIdFn)(CUcontext, unsigned long long*);

struct AddrSlot {
    int dev;
    unsigned long long ctx_id;
    void* ptr;
};
constexpr int kAddrSlots = 64;
AddrSlot g_addr[kAddrSlots];
int g_naddr = 0;
std::mutex g_addr_mu;

int current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_cur = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    if (!get_cur || !get_id) return -1;
    CUcontext ctx = nullptr;
    if (get_cur(&ctx) != CUDA_SUCCESS || !ctx) return -1;
    return get_id(ctx, id) == CUDA_SUCCESS ? 0 : -1;
}

int scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return nerr(GPMOOD_E_CUDA, "cudaGetDevice", cudaGetErrorString(e));
    unsigned long long id = 0;
    const bool have_id = current_context_id(&id) == 0;  // false before the thread's first CUDA work
    std::lock_guard<std::mutex> lock(g_addr_mu);
    if (have_id)
        for (int i = 0; i < g_naddr; i++)
            if (g_addr[i].dev == dev && g_addr[i].ctx_id == id) {
                *out = g_addr[i].ptr;
                return 0;
            }
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);  // initialises the primary context if none is current
    if (e != cudaSuccess || !ptr) return nerr(GPMOOD_E_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch)", cudaGetErrorString(e));
    if (!have_id && current_context_id(&id)) return nerr(GPMOOD_E_CUDA, "no current CUDA context");
    const int slot = g_naddr < kAddrSlots ? g_naddr++ : (int)(id % kAddrSlots);
    g_addr[slot] = AddrSlot{dev, id, ptr};
    *out = ptr;
    return 0;
}

// ---- GP weights, computed once per knob set ---------------------------------
// The binary128 precompute takes milliseconds, far more than a step on a small
// grid, so the last few knob sets' weights are kept in a fixed table.
struct WeightSlot {
    bool used;
    double ell_o_dx, lx, ly;
    int lf, nf, mord, ngp;
    unsigned long long last;
    GpWeights w;
};
constexpr int kWeightSlots = 4;
WeightSlot g_w[kWeightSlots];
unsigned long long g_wclock = 0;
std::mutex g_w_mu;

int weights_for(const gpmood_params* p, GpWeights* out) {
    std::lock_guard<std::mutex> lock(g_w_mu);
    int victim = 0;
    for (int i = 0; i < kWeightSlots; i++) {
        WeightSlot& s = g_w[i];
        if (s.used && s.ell_o_dx == p->ell_o_dx && s.lx == p->lx && s.ly == p->ly && s.lf == p->lf &&
            s.nf == p->nf && s.mord == p->mord && s.ngp == p->ngp) {
            s.last = ++g_wclock;
            *out = s.w;
            return 0;
        }
        if (!s.used || (g_w[victim].used && s.last < g_w[victim].last)) victim = i;
    }
    WeightSlot& s = g_w[victim];
    double inv_err[3];
    if (gpm_gp_presim(p->ell_o_dx, p->lx, p->ly, p->lf, p->nf, p->mord, p->ngp, &s.w, inv_err)) {
        s.used = false;
        return -1;
    }
    s.used = true;
    s.ell_o_dx = p->ell_o_dx;
    s.lx = p->lx;
    s.ly = p->ly;
    s.lf = p->lf;
    s.nf = p->nf;
    s.mord = p->mord;
    s.ngp = p->ngp;
    s.last = ++g_wclock;
    *out = s.w;
    return 0;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Carve {
    double *u1, *u2, *fx, *fy;
    int8_t* order;
    unsigned* stamp;
    int* list[2];
    DevScalars* sc;
    GridBar* bar;
};

Carve carve(unsigned char* base, size_t ncell) {
    Carve c;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base + off;
        off = align256(off + bytes);
        return p;
    };
    c.sc = reinterpret_cast<DevScalars*>(take(sizeof(DevScalars)));
    c.bar = reinterpret_cast<GridBar*>(take(sizeof(GridBar)));
    c.u1 = reinterpret_cast<double*>(take(ncell * 32));
    c.u2 = reinterpret_cast<double*>(take(ncell * 32));
    c.fx = reinterpret_cast<double*>(take(ncell * 32));
    c.fy = reinterpret_cast<double*>(take(ncell * 32));
    c.stamp = reinterpret_cast<unsigned*>(take(ncell * 4));
    c.list[0] = reinterpret_cast<int*>(take(ncell * 4));
    c.list[1] = reinterpret_cast<int*>(take(ncell * 4));
    c.order = reinterpret_cast<int8_t*>(take(ncell));
    return c;
}

#define NCU(call)                                                                      \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) return nerr(GPMOOD_E_CUDA, #call, cudaGetErrorString(e_)); \
    } while (0)

// One Forward_Euler stage (mod_FE.f90:20-190): Boundary_C(Uin), the first pass
// over all faces, the update with DETECTION, then passes 2, 3, ... in one
// cooperative launch; nothing waits for the GPU.
int stage_noalloc(const KernelTable& kt, const GridGeom& g, const GpWeights& w, const Carve& s, double* uin,
                  double* uout, int stage, int max_pass, cudaStream_t st) {
    kt.bc(g, uin, s.sc, stage, st);
    NCU(cudaMemsetAsync(s.order, g.mord, (size_t)g.nx * g.ny, st));
    NCU(cudaMemsetAsync(s.sc->ntrb, 0, sizeof(s.sc->ntrb), st));
    StageArgs a;
    a.g = g;
    a.uin = uin;
    a.uout = uout;
    a.fx = s.fx;
    a.fy = s.fy;
    a.order = s.order;
    a.stamp = s.stamp;
    a.tlist[0] = s.list[0];
    a.tlist[1] = s.list[1];
    a.sc = s.sc;
    a.uniform_order = 1;
    a.stage = stage;
    a.ccw = nullptr;
    kt.flux_all(a, w, st);
    kt.update_detect(a, w, 0, st);
    NCU(cudaGetLastError());
    if (g.method == GPMOOD_GP_MOOD && kt.mood_loop(a, w, s.bar, max_pass, stage, st))
        return nerr(GPMOOD_E_CUDA, "MOOD loop launch", cudaGetErrorString(cudaGetLastError()));
    kt.bc(g, uout, s.sc, stage, st);  // the last DETECTION's Boundary_C(Uout)
    NCU(cudaGetLastError());
    return 0;
}

}  // namespace

extern "C" int gpmood_time_stepping_noalloc(const gpmood_params* p, double* d_uin, double* d_uout, double t,
                                            double dt, void* stream, int* status) {
    if (status) *status = 0;
    if (!p || !d_uin || !d_uout) return nerr(GPMOOD_E_ARG, "NULL argument");
    char why[256];
    if (gpm_validate_params(p, why, sizeof why)) return nerr(GPMOOD_E_ARG, why);
    if (p->integrator != GPMOOD_SSP_RK3 || (p->method != GPMOOD_GP_MOOD && p->method != GPMOOD_GP_SE) ||
        (p->bc_type != GPMOOD_NEUMANN && p->bc_type != GPMOOD_PERIODIC && p->bc_type != GPMOOD_REFLECTIVE &&
         p->bc_type != GPMOOD_DMR))
        return nerr(GPMOOD_E_ARG, "gpmood_time_stepping_noalloc supports SSP-RK3, GP_MOOD or GP_SE, and Neumann, "
                                  "periodic, reflective or DMR boundaries");
    if (!(dt > 0) || dt != dt || dt > 1e300) return nerr(GPMOOD_E_DT, "dt must be finite and > 0");
    const size_t ncell = (size_t)(p->lf + 2 * GPM_NGC) * (size_t)(p->nf + 2 * GPM_NGC);
    if (ncell > GPM_NOALLOC_MAX_CELLS) {
        snprintf(why, sizeof why, "(lf+8)*(nf+8) = %zu exceeds the %d padded cells of the static scratch", ncell,
                 GPM_NOALLOC_MAX_CELLS);
        return nerr(GPMOOD_E_ARG, "grid too large for gpmood_time_stepping_noalloc", why);
    }
    void* base = nullptr;
    if (int rc = scratch_address(&base)) return rc;
    const Carve s = carve(static_cast<unsigned char*>(base), ncell);

    GridGeom g;
    memset(&g, 0, sizeof g);
    g.lf = p->lf;
    g.nf = p->nf;
    g.nx = p->lf + 2 * GPM_NGC;
    g.ny = p->nf + 2 * GPM_NGC;
    g.dx = gpm_cell_size(p->lx, p->lf);
    g.dy = gpm_cell_size(p->ly, p->nf);
    g.bc_type = p->bc_type;
    g.ngp = p->ngp;
    g.mord = p->mord;
    g.method = p->method;
    g.num_flux = p->num_flux;
    g.dmp = p->dmp;
    g.u2 = p->u2;
    g.u2_tol = p->u2_tol;
    g.mood_solo = gpm_mood_solo_default();
    g.flux_tma = gpm_flux_tma_default();
    g.solo_split = gpm_solo_split_default();
    g.cc_col = -1;
    GpWeights w;
    if (weights_for(p, &w)) return nerr(GPMOOD_E_ARG, "GP precompute rejected the knobs");
    const KernelTable& kt = p->fp_mode == GPMOOD_FP_FAST ? gpm_fast::table : gpm_exact::table;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    DevScalars h;
    memset(&h, 0, sizeof h);
    h.t = t;
    h.dt = dt;
    h.qx = dt / g.dx;
    h.qy = dt / g.dy;
    h.tmax = p->tmax;
    h.cfl = p->cfl;
    h.dtmin_bits = 0x46293e5939a08ceaULL;  // bits of 1.0e30
    NCU(cudaMemcpyAsync(s.sc, &h, sizeof h, cudaMemcpyHostToDevice, st));
    NCU(cudaMemsetAsync(s.bar, 0, sizeof(GridBar), st));
    NCU(cudaMemsetAsync(s.stamp, 0, ncell * sizeof(unsigned), st));  // pass stamps restart every call
    // 0 allows 2*lf*nf+2 passes, more than a terminating MOOD loop can take
    const long long cap = p->max_mood_iters > 0 ? p->max_mood_iters : 2LL * p->lf * p->nf + 2;
    const int max_pass = cap > 0x7fffffff ? 0x7fffffff : (int)cap;
    int rc = stage_noalloc(kt, g, w, s, d_uin, s.u1, 0, max_pass, st);
    if (!rc) rc = stage_noalloc(kt, g, w, s, s.u1, s.u2, 1, max_pass, st);
    if (!rc) {
        kt.combine(g, d_uin, s.u2, 0.75, 0.25, 0, s.sc, st);
        rc = stage_noalloc(kt, g, w, s, s.u2, d_uout, 2, max_pass, st);
    }
    if (!rc) kt.combine(g, d_uin, d_uout, 1. / 3, 2. / 3, 0, s.sc, st);
    // the step's status word and the barrier flag: one wait per call
    GridBar hb;
    NCU(cudaGetLastError());
    NCU(cudaMemcpyAsync(&h, s.sc, sizeof h, cudaMemcpyDeviceToHost, st));
    NCU(cudaMemcpyAsync(&hb, s.bar, sizeof hb, cudaMemcpyDeviceToHost, st));
    NCU(cudaStreamSynchronize(st));
    if (rc) return rc;
    if (status) *status = h.status | (hb.err ? GPM_STATUS_BARRIER : 0);
    if (hb.err) return nerr(GPMOOD_E_CUDA, "MOOD loop grid barrier timed out");
    if (h.status & GPM_STATUS_MOODCAP) return nerr(GPMOOD_E_MOOD_CAP, "MOOD loop did not converge");
    return 0;
}
