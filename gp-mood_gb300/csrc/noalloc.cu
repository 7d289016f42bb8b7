// noalloc.cu -- one GP-MOOD time step that allocates no memory.
//
// Some callers cannot let a library allocate device memory: a host that owns
// all GPU memory through its own pool (a cudaMalloc would bypass the pool's
// accounting and implicitly synchronise the device), or a real-time loop that
// must not stall in the allocator.  For them gpmood_time_stepping_noalloc runs
// the same SSP-RK3 step as gpmood_time_stepping_dev, with every scratch array
// (RK stage buffers, face-flux stores, order mask, MOOD stamps and lists,
// device scalars) carved out of the file-scope array below instead of being
// allocated.  The caller still passes the input and output states.
//
// The array is sized for grids of at most GPM_NOALLOC_MAX_CELLS padded cells
// ((lf+8)*(nf+8) <= 264*264, e.g. 256x256), about 10 MB; every GPU that loads
// the library holds it until the process exits.  All calls share it and it
// keeps the last call's contents, so calls that overlap on the GPU (other
// streams, other host threads) race; the stamps that must start at zero are
// cleared at the start of every call.
#include <stdio.h>
#include <string.h>

#include "../../include/gpmood.h"
#include "gpm_common.h"

#define GPM_NOALLOC_MAX_CELLS (264 * 264)
// Bytes per padded cell: U1, U2, Fx, Fy (4 doubles each), order (1), stamp (4), two lists (4 + 4).
#define GPM_NOALLOC_CELL_BYTES (4 * 32 + 1 + 4 + 4 + 4)
#define GPM_NOALLOC_BYTES ((size_t)GPM_NOALLOC_MAX_CELLS * GPM_NOALLOC_CELL_BYTES + 16 * 256)

static __device__ __align__(256) unsigned char g_noalloc_scratch[GPM_NOALLOC_BYTES];

namespace {

// Device address of g_noalloc_scratch per device, set once with that device current.
void* g_scratch_addr[64];

// The message goes to the thread's error buffer, read by gpmood_last_error(NULL, ...).
int nerr(int code, const char* msg, const char* detail = nullptr) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s%s%s", msg, detail ? ": " : "", detail ? detail : "");
    gpm_set_thread_error(buf);
    return code;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Carve {
    double *u1, *u2, *fx, *fy;
    int8_t* order;
    unsigned* stamp;
    int* list[2];
    DevScalars* sc;
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

int stage_noalloc(const KernelTable& kt, const GridGeom& g, const GpWeights& w, const Carve& s, double* uin,
                  double* uout, int stage, int max_iters, unsigned* pass_id, cudaStream_t st) {
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
    if (g.method == GPMOOD_GP_MOOD) {
        int cur = 0, npass = 1;
        for (;;) {
            int nt = 0;
            NCU(cudaMemcpyAsync(&nt, &s.sc->ntrb[cur], sizeof(int), cudaMemcpyDeviceToHost, st));
            NCU(cudaStreamSynchronize(st));
            if (nt == 0) break;
            if (npass >= max_iters) return nerr(GPMOOD_E_MOOD_CAP, "MOOD loop did not converge");
            npass++;
            kt.mood_mark(a, cur, nt, st);
            kt.mood_faces(a, w, cur, nt, st);
            kt.mood_cells(a, w, cur, nt, ++*pass_id, st);
            NCU(cudaGetLastError());
            cur ^= 1;
        }
    }
    kt.bc(g, uout, s.sc, stage, st);
    NCU(cudaGetLastError());
    return 0;
}

}  // namespace

extern "C" int gpmood_time_stepping_noalloc(const gpmood_params* p, double* d_uin, double* d_uout, double t,
                                            double dt, void* stream) {
    if (!p || !d_uin || !d_uout) return nerr(GPMOOD_E_ARG, "NULL argument");
    if (p->integrator != GPMOOD_SSP_RK3 || p->num_flux < GPMOOD_HLLC || p->num_flux > GPMOOD_UNSPLIT ||
        (p->method != GPMOOD_GP_MOOD && p->method != GPMOOD_GP_SE) || !(p->mord == 1 || p->mord == 3 || p->mord == 5) ||
        p->ngp < 1 || p->ngp > 5 || p->lf < 4 || p->nf < 4 ||
        (p->bc_type != GPMOOD_NEUMANN && p->bc_type != GPMOOD_PERIODIC && p->bc_type != GPMOOD_REFLECTIVE &&
         p->bc_type != GPMOOD_DMR) ||
        (p->fp_mode != GPMOOD_FP_EXACT && p->fp_mode != GPMOOD_FP_FAST) || p->max_mood_iters < 0)
        return nerr(GPMOOD_E_ARG, "unsupported knobs (GP_MOOD/GP_SE, SSP-RK3, Mord 1/3/5, ngp 1..5)");
    if (!(dt > 0) || dt != dt || dt > 1e300) return nerr(GPMOOD_E_DT, "dt must be finite and > 0");
    const size_t ncell = (size_t)(p->lf + 2 * GPM_NGC) * (size_t)(p->nf + 2 * GPM_NGC);
    if (ncell > GPM_NOALLOC_MAX_CELLS) {
        char why[128];
        snprintf(why, sizeof why, "(lf+8)*(nf+8) = %zu exceeds the %d padded cells of the static scratch", ncell,
                 GPM_NOALLOC_MAX_CELLS);
        return nerr(GPMOOD_E_ARG, "grid too large for gpmood_time_stepping_noalloc", why);
    }

    int dev = 0;
    NCU(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return nerr(GPMOOD_E_CUDA, "device index out of range");
    if (!g_scratch_addr[dev]) {  // once per device, with that device current
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) return nerr(GPMOOD_E_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch)", cudaGetErrorString(e));
        g_scratch_addr[dev] = ptr;
    }
    const Carve s = carve(static_cast<unsigned char*>(g_scratch_addr[dev]), ncell);

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
    g.cc_col = -1;
    GpWeights w;
    double inv_err[3];
    if (gpm_gp_presim(p->ell_o_dx, p->lx, p->ly, p->lf, p->nf, p->mord, p->ngp, &w, inv_err))
        return nerr(GPMOOD_E_ARG, "GP precompute rejected the knobs");
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
    NCU(cudaMemsetAsync(s.stamp, 0, ncell * sizeof(unsigned), st));  // pass ids restart at 1 every call
    unsigned pass_id = 0;
    // 0 allows 2*lf*nf+2 passes, more than a terminating MOOD loop can take
    const int max_iters = p->max_mood_iters > 0 ? p->max_mood_iters : 2 * p->lf * p->nf + 2;
    int rc = stage_noalloc(kt, g, w, s, d_uin, s.u1, 0, max_iters, &pass_id, st);
    if (!rc) rc = stage_noalloc(kt, g, w, s, s.u1, s.u2, 1, max_iters, &pass_id, st);
    if (!rc) {
        kt.combine(g, d_uin, s.u2, 0.75, 0.25, 0, s.sc, st);
        rc = stage_noalloc(kt, g, w, s, s.u2, d_uout, 2, max_iters, &pass_id, st);
    }
    if (!rc) {
        kt.combine(g, d_uin, d_uout, 1. / 3, 2. / 3, 0, s.sc, st);
        NCU(cudaGetLastError());
        NCU(cudaStreamSynchronize(st));
    }
    return rc;
}
