// stage_kernels.cu -- the kernels of one GP-MOOD Runge-Kutta stage.
//
// Compiled twice into libgpmood.so:
//   -DGPM_EXACT=1 --fmad=false  -> namespace gpm_exact (bit-identical to the
//                                  reference's operation order)
//   -DGPM_EXACT=0 --fmad=true   -> namespace gpm_fast
//
// One stage (Forward_Euler, gp-mood-code/mod_FE.f90:20-190) runs as:
//   k_bc_x / k_bc_y       Boundary_C(Uin)                      BC.f90:10-421
//   k_flux_tile<x|y>      every face: GP recon + HLLC + quadrature, stored
//                         (the first MOOD pass, mod_FE.f90:73-145)
//   k_update_detect       Uout = Uin + flux differences, DETECTION on every
//                         cell, troubled cells stream-compacted into a list
//   while the list is not empty (the MOOD loop, mod_FE.f90:69-174):
//     k_mood_mark         order cascade 5->3->1 of the troubled cells
//     k_mood_faces        recompute the 4 faces of each troubled cell
//     k_mood_cells        recompute Uout of the 5-point cross of each
//                         troubled cell, re-run DETECTION there -> next list
//   k_bc_x / k_bc_y       Boundary_C(Uout)
//   k_combine             SSP-RK3 combination (mod_SSP_RK3.f90:28,33), with
//                         the next step's Setdt reduction fused into the last
//
// Why the list-based loop equals the reference's full-grid loop: after a
// DETECTION pass the reference flags exactly the faces of troubled cells and
// the cells of their 5-point crosses (mod_subroutine_MOOD.f90:133-182), resets
// those cells to Uin, and in the next pass recomputes flagged faces and
// re-applies stored fluxes to flagged cells only.  Every other cell keeps its
// Uout.  A stored flux always equals the flux at the current orders (a face is
// recomputed whenever an adjacent order drops), so recomputing a flagged
// cell's Uout from Uin and its four current face fluxes, in the reference's
// accumulation order, reproduces the reference bit for bit.
#include "physics.cuh"

#if GPM_EXACT
#define GPM_NS gpm_exact
#else
#define GPM_NS gpm_fast
#endif

namespace GPM_NS {

constexpr int TX = 32, TY = 8;           // faces per CTA tile
constexpr int HX = TX + 5, HY = TY + 5;  // cells staged per tile (halo 2 below, 3 above)

__device__ __forceinline__ size_t cidx(const GridGeom& g, int l, int n) {
    return (size_t)(n + 3) * (size_t)g.nx + (size_t)(l + 3);
}

// ---------------------------------------------------------------------------
// Boundary_C, BC.f90:10-421.  Pass 1 fills the ghost columns of interior rows,
// pass 2 the ghost rows of every column (so corners come from pass 1 values,
// as in the reference's loop nest).

__device__ __forceinline__ void p2c(double r, double u, double v, double p, double* out) {
    out[0] = r;
    out[1] = r * u;
    out[2] = r * v;
    out[3] = ((p / (GPM_GAMMA - 1.)) + 0.5 * r * (u * u + v * v));
}

__device__ __forceinline__ void f_dmr(double x, double y, double* r) {  // IC.f90:336-355
    const double xmin = 1. / 6;
    const double ymin = (x - xmin) * sqrt(3.);
    if (y > ymin) p2c(8., 7.1447096, -4.125, 116.5, r);
    else p2c(1.4, 0.0, 0.0, 1.0, r);
}

__global__ void k_bc_x(GridGeom g, double* __restrict__ u, const DevScalars* __restrict__ sc, int stage) {
    const int n = 1 + blockIdx.x * blockDim.y + threadIdx.y;   // interior row
    const int k = threadIdx.x;                                  // 0..7: 4 left + 4 right ghosts
    if (n > g.nf || k >= 2 * GPM_NGC) return;
    const bool right = k >= GPM_NGC;
    const int j = right ? k - GPM_NGC : k;                      // 0..3
    const int l = right ? g.lf + 1 + j : -j;                    // right: lf+1..lf+4, left: 0..-3
    double* dst = u + 4 * cidx(g, l, n);
    if (g.bc_type == 17) {  // Neumann
        const double* src = u + 4 * cidx(g, right ? g.lf : 1, n);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    } else if (g.bc_type == 18) {  // Periodic
        const int ls = right ? 1 + j : g.lf - j;
        const double* src = u + 4 * cidx(g, ls, n);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    } else if (g.bc_type == 20) {  // Reflective: mirror, flip normal momentum
        const int ls = right ? g.lf - j : 1 + j;
        const double* src = u + 4 * cidx(g, ls, n);
        dst[0] = src[0]; dst[1] = -src[1]; dst[2] = src[2]; dst[3] = src[3];
    } else if (g.bc_type == 35) {  // DMR: exact pre/post-shock states
        f_dmr(l * g.dx - g.dx / 2, n * g.dy - g.dy / 2, dst);
    }
}

__global__ void k_bc_y(GridGeom g, double* __restrict__ u, const DevScalars* __restrict__ sc, int stage) {
    const int l = -3 + blockIdx.x * blockDim.y + threadIdx.y;  // every column incl. ghosts
    const int k = threadIdx.x;
    if (l > g.lf + GPM_NGC || k >= 2 * GPM_NGC) return;
    const bool top = k >= GPM_NGC;
    const int j = top ? k - GPM_NGC : k;
    const int n = top ? g.nf + 1 + j : -j;
    double* dst = u + 4 * cidx(g, l, n);
    if (g.bc_type == 17) {
        const double* src = u + 4 * cidx(g, l, top ? g.nf : 1);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    } else if (g.bc_type == 18) {
        const int ns = top ? 1 + j : g.nf - j;
        const double* src = u + 4 * cidx(g, l, ns);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    } else if (g.bc_type == 20) {
        const int ns = top ? g.nf - j : 1 + j;
        const double* src = u + 4 * cidx(g, l, ns);
        dst[0] = src[0]; dst[1] = src[1]; dst[2] = -src[2]; dst[3] = src[3];
    } else if (g.bc_type == 35) {
        const double x = l * g.dx - g.dx / 2;
        if (top) {
            // t_rk of the stage (mod_SSP_RK3.f90:22,26,29)
            const double t_rk = stage == 0 ? sc->t : (stage == 1 ? sc->t + sc->dt : sc->t + 0.5 * sc->dt);
            const double xmin = 1. / 6 + 10. * t_rk / (0.5 * sqrt(3.)) + 1. / sqrt(3.);
            if (x < xmin) p2c(8., 7.1447096, -4.125, 116.5, dst);
            else p2c(1.4, 0.0, 0.0, 1.0, dst);
        } else if (x > 1. / 6) {
            const double* src = u + 4 * cidx(g, l, 1 + j);
            dst[0] = src[0]; dst[1] = src[1]; dst[2] = -src[2]; dst[3] = src[3];
        } else {
            p2c(8., 7.1447096, -4.125, 116.5, dst);
        }
    }
}

void launch_bc(const GridGeom& g, double* u, const DevScalars* sc, int stage, cudaStream_t s) {
    const dim3 blk(8, 32);
    k_bc_x<<<(g.nf + 31) / 32, blk, 0, s>>>(g, u, sc, stage);
    k_bc_y<<<(g.nx + 31) / 32, blk, 0, s>>>(g, u, sc, stage);
}

// ---------------------------------------------------------------------------
// First MOOD pass: every face of the stage.  One thread per face; the CTA
// stages its (TX+5) x (TY+5) cells of Uin in shared memory, then each thread
// reconstructs the two face states at every Gauss point (13-point GP dot
// products), solves HLLC and integrates along the face.

template <int DIR, int NP, int NGP>
__device__ __forceinline__ void face_from_tile(const GpWeights& w, int o, const Cell (*tile)[HX], int tx, int ty,
                                               double* F) {
    constexpr int FL = DIR == 0 ? 2 : 1;  // iR (x) / iT (y) face of the low cell
    constexpr int FH = DIR == 0 ? 0 : 3;  // iL (x) / iB (y) face of the high cell
    double uL[NGP][4], uR[NGP][4];
    {
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = tile[ty + st_oy(m)][tx + st_ox(m)];
        gp_recon<NP, NGP>(&w.zt[o][FL][0][0], q, uL);
    }
    {
        constexpr int hx = DIR == 0 ? 1 : 0, hy = DIR == 0 ? 0 : 1;
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = tile[ty + hy + st_oy(m)][tx + hx + st_ox(m)];
        gp_recon<NP, NGP>(&w.zt[o][FH][0][0], q, uR);
    }
    quad_flux<DIR, NGP>(uL, uR, w.gw, F);
}

template <int DIR, int NGP, int UORD>  // UORD: uniform order (1,3,5) or 0 = per-face from the order array
__global__ void __launch_bounds__(TX * TY) k_flux_tile(StageArgs a, const __grid_constant__ GpWeights w) {
    __shared__ Cell tile[HY][HX];
    const GridGeom& g = a.g;
    const int lmin = DIR == 0 ? 0 : 1, nmin = DIR == 0 ? 1 : 0;
    const int l0 = lmin + blockIdx.x * TX, n0 = nmin + blockIdx.y * TY;
    const int tid = threadIdx.y * TX + threadIdx.x;
    for (int i = tid; i < HX * HY; i += TX * TY) {
        const int cy = i / HX, cx = i - cy * HX;
        const int l = l0 - 2 + cx, n = n0 - 2 + cy;
        if (l >= -3 && l <= g.lf + 4 && n >= -3 && n <= g.nf + 4) tile[cy][cx] = ld_cell(a.uin + 4 * cidx(g, l, n));
    }
    __syncthreads();
    const int l = l0 + threadIdx.x, n = n0 + threadIdx.y;
    if (l > g.lf || n > g.nf) return;
    const int tx = threadIdx.x + 2, ty = threadIdx.y + 2;
    double F[4];
    if (UORD != 0) {
        face_from_tile<DIR, np_of(UORD == 0 ? 1 : UORD), NGP>(w, UORD / 2, tile, tx, ty, F);
    } else {
        const size_t c0 = cidx(g, l, n), c1 = DIR == 0 ? c0 + 1 : c0 + g.nx;
        const int o = min((int)a.order[c0], (int)a.order[c1]);
        if (o >= 5) face_from_tile<DIR, 13, NGP>(w, 2, tile, tx, ty, F);
        else if (o >= 3) face_from_tile<DIR, 5, NGP>(w, 1, tile, tx, ty, F);
        else face_from_tile<DIR, 1, NGP>(w, 0, tile, tx, ty, F);
    }
    double* out = (DIR == 0 ? a.fx : a.fy) + 4 * cidx(g, l, n);
    st_cell(out, Cell{F[0], F[1], F[2], F[3]});
}

template <int DIR, int NGP>
void launch_flux_dir(const StageArgs& a, const GpWeights& w, cudaStream_t s) {
    const int nl = DIR == 0 ? a.g.lf + 1 : a.g.lf;
    const int nn = DIR == 0 ? a.g.nf : a.g.nf + 1;
    const dim3 grid((nl + TX - 1) / TX, (nn + TY - 1) / TY), blk(TX, TY);
    if (!a.uniform_order) k_flux_tile<DIR, NGP, 0><<<grid, blk, 0, s>>>(a, w);
    else if (a.g.mord == 5) k_flux_tile<DIR, NGP, 5><<<grid, blk, 0, s>>>(a, w);
    else if (a.g.mord == 3) k_flux_tile<DIR, NGP, 3><<<grid, blk, 0, s>>>(a, w);
    else k_flux_tile<DIR, NGP, 1><<<grid, blk, 0, s>>>(a, w);
}

template <int NGP>
void launch_flux_ngp(const StageArgs& a, const GpWeights& w, cudaStream_t s) {
    launch_flux_dir<0, NGP>(a, w, s);
    launch_flux_dir<1, NGP>(a, w, s);
}

void launch_flux_all(const StageArgs& a, const GpWeights& w, cudaStream_t s) {
    switch (a.g.ngp) {
    case 1: launch_flux_ngp<1>(a, w, s); break;
    case 2: launch_flux_ngp<2>(a, w, s); break;
    case 3: launch_flux_ngp<3>(a, w, s); break;
    case 4: launch_flux_ngp<4>(a, w, s); break;
    default: launch_flux_ngp<5>(a, w, s); break;
    }
}

// ---------------------------------------------------------------------------
// Flux-difference update of one cell in the reference's accumulation order
// (the n-outer, l-inner face loop of mod_FE.f90:75-145 visits, for cell
// (l,n): the y face below, the x face to the left, the x face to the right,
// the y face above).
__device__ __forceinline__ Cell cell_update(const GridGeom& g, const double* __restrict__ uin,
                                            const double* __restrict__ fx, const double* __restrict__ fy,
                                            size_t c, double qx, double qy) {
    const Cell u = ld_cell(uin + 4 * c);
    const Cell fb = ld_cell_cg(fy + 4 * (c - g.nx));
    const Cell fl = ld_cell_cg(fx + 4 * (c - 1));
    const Cell fr = ld_cell_cg(fx + 4 * c);
    const Cell ft = ld_cell_cg(fy + 4 * c);
    Cell o;
    o.r = u.r + qy * fb.r;    o.mx = u.mx + qy * fb.mx;   o.my = u.my + qy * fb.my;   o.e = u.e + qy * fb.e;
    o.r = o.r + qx * fl.r;    o.mx = o.mx + qx * fl.mx;   o.my = o.my + qx * fl.my;   o.e = o.e + qx * fl.e;
    o.r = o.r - qx * fr.r;    o.mx = o.mx - qx * fr.mx;   o.my = o.my - qx * fr.my;   o.e = o.e - qx * fr.e;
    o.r = o.r - qy * ft.r;    o.mx = o.mx - qy * ft.mx;   o.my = o.my - qy * ft.my;   o.e = o.e - qy * ft.e;
    return o;
}

// Warp-aggregated append of flagged cells to a list.
__device__ __forceinline__ void list_append(bool flag, int* __restrict__ list, int* __restrict__ count, int value) {
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, flag);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(act) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(act, base, leader);
    if (flag) list[base + __popc(m & ((1u << lane) - 1))] = value;
}

__global__ void __launch_bounds__(256) k_update_detect(StageArgs a, const __grid_constant__ GpWeights w, int cur) {
    const GridGeom& g = a.g;
    const int l = 1 + blockIdx.x * 32 + threadIdx.x, n = 1 + blockIdx.y * 8 + threadIdx.y;
    if (l > g.lf || n > g.nf) return;
    const size_t c = cidx(g, l, n);
    const double qx = a.sc->qx, qy = a.sc->qy;
    const Cell uo = cell_update(g, a.uin, a.fx, a.fy, c, qx, qy);
    st_cell(a.uout + 4 * c, uo);
    bool trb = false;
    if (g.method == 2 || g.method == 203) {
        const int o = a.uniform_order ? g.mord : (int)a.order[c];
        if (o > 1) trb = mood_troubled(uo, a.uin + 4 * c, g.nx, g, w.d2x, w.d2y);
    }
    list_append(trb, a.tlist[cur], &a.sc->ntrb[cur], (int)c);
}

void launch_update_detect(const StageArgs& a, const GpWeights& w, int cur, cudaStream_t s) {
    const dim3 grid((a.g.lf + 31) / 32, (a.g.nf + 7) / 8), blk(32, 8);
    k_update_detect<<<grid, blk, 0, s>>>(a, w, cur);
}

// ---------------------------------------------------------------------------
// MOOD passes 2, 3, ... on the troubled list only.

constexpr int LIST_CTAS_PER_SM = 4;

__global__ void k_mood_mark(StageArgs a, int cur) {
    const int nt = a.sc->ntrb[cur];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
        const int c = a.tlist[cur][i];
        const int o = a.order[c];
        a.order[c] = (int8_t)(o == 3 ? 1 : (o > 3 ? 3 : o));  // mod_subroutine_MOOD.f90:159-163
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(&a.sc->detected_step, (unsigned long long)nt);
        a.sc->ntrb[cur ^ 1] = 0;
    }
}

// One face of the face list at its current order (min of the two cells),
// with stencils read straight from global memory.
template <int DIR, int NP, int NGP>
__device__ __forceinline__ void face_global(const GridGeom& g, const GpWeights& w, int o, const double* __restrict__ uin,
                                            size_t c0, double* F) {
    constexpr int FL = DIR == 0 ? 2 : 1;
    constexpr int FH = DIR == 0 ? 0 : 3;
    const ptrdiff_t row = g.nx;
    const size_t c1 = DIR == 0 ? c0 + 1 : c0 + g.nx;
    double uL[NGP][4], uR[NGP][4];
    {
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = ld_cell(uin + 4 * (c0 + st_ox(m) + row * st_oy(m)));
        gp_recon<NP, NGP>(&w.zt[o][FL][0][0], q, uL);
    }
    {
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = ld_cell(uin + 4 * (c1 + st_ox(m) + row * st_oy(m)));
        gp_recon<NP, NGP>(&w.zt[o][FH][0][0], q, uR);
    }
    quad_flux<DIR, NGP>(uL, uR, w.gw, F);
}

template <int DIR, int NGP>
__device__ __forceinline__ void face_any_order(const StageArgs& a, const GpWeights& w, size_t c0) {
    const GridGeom& g = a.g;
    const size_t c1 = DIR == 0 ? c0 + 1 : c0 + g.nx;
    const int o = min((int)a.order[c0], (int)a.order[c1]);
    double F[4];
    if (o >= 5) face_global<DIR, 13, NGP>(g, w, 2, a.uin, c0, F);
    else if (o >= 3) face_global<DIR, 5, NGP>(g, w, 1, a.uin, c0, F);
    else face_global<DIR, 1, NGP>(g, w, 0, a.uin, c0, F);
    st_cell((DIR == 0 ? a.fx : a.fy) + 4 * c0, Cell{F[0], F[1], F[2], F[3]});
}

template <int NGP>
__global__ void __launch_bounds__(128) k_mood_faces(StageArgs a, const __grid_constant__ GpWeights w, int cur) {
    const int nt = a.sc->ntrb[cur];
    // 4 faces per troubled cell: x faces (l-1,n), (l,n), y faces (l,n-1), (l,n).
    // Even work items are x faces, odd ones y faces, so warps stay mostly uniform.
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * nt; i += gridDim.x * blockDim.x) {
        const size_t c = (size_t)a.tlist[cur][i >> 2];
        const int f = i & 3;
        if ((f & 1) == 0) face_any_order<0, NGP>(a, w, f == 0 ? c - 1 : c);
        else face_any_order<1, NGP>(a, w, f == 1 ? c - a.g.nx : c);
    }
}

__global__ void __launch_bounds__(256) k_mood_cells(StageArgs a, const __grid_constant__ GpWeights w, int cur,
                                                    unsigned pass_id) {
    const GridGeom& g = a.g;
    const int nt = a.sc->ntrb[cur];
    const double qx = a.sc->qx, qy = a.sc->qy;
    const int nxt = cur ^ 1;
    const int total = 5 * nt;
    const int stride = gridDim.x * blockDim.x;
    // Round the trip count up to a multiple of the stride so whole warps reach
    // list_append together.
    const int lim = ((total + stride - 1) / stride) * stride;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < lim; i += stride) {
        bool trb = false;
        int cval = 0;
        if (i < total) {
            const size_t t = (size_t)a.tlist[cur][i / 5];
            const int k = i % 5;
            const size_t c = k == 0 ? t - g.nx : k == 1 ? t - 1 : k == 2 ? t : k == 3 ? t + 1 : t + g.nx;
            const int l = (int)(c % (size_t)g.nx) - 3, n = (int)(c / (size_t)g.nx) - 3;
            const bool interior = l >= 1 && l <= g.lf && n >= 1 && n <= g.nf;
            if (interior && atomicExch(&a.stamp[c], pass_id) != pass_id) {
                const Cell uo = cell_update(g, a.uin, a.fx, a.fy, c, qx, qy);
                st_cell(a.uout + 4 * c, uo);
                if (a.order[c] > 1) trb = mood_troubled(uo, a.uin + 4 * c, g.nx, g, w.d2x, w.d2y);
                cval = (int)c;
            }
        }
        list_append(trb, a.tlist[nxt], &a.sc->ntrb[nxt], cval);
    }
}

static int list_grid(int max_items, int threads) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int need = (max_items + threads - 1) / threads;
    const int cap = sms * LIST_CTAS_PER_SM;
    return need < 1 ? 1 : (need < cap ? need : cap);
}

void launch_mood_mark(const StageArgs& a, int cur, int max_trb, cudaStream_t s) {
    k_mood_mark<<<list_grid(max_trb, 256), 256, 0, s>>>(a, cur);
}

void launch_mood_faces(const StageArgs& a, const GpWeights& w, int cur, int max_trb, cudaStream_t s) {
    const int gr = list_grid(4 * max_trb, 128);
    switch (a.g.ngp) {
    case 1: k_mood_faces<1><<<gr, 128, 0, s>>>(a, w, cur); break;
    case 2: k_mood_faces<2><<<gr, 128, 0, s>>>(a, w, cur); break;
    case 3: k_mood_faces<3><<<gr, 128, 0, s>>>(a, w, cur); break;
    case 4: k_mood_faces<4><<<gr, 128, 0, s>>>(a, w, cur); break;
    default: k_mood_faces<5><<<gr, 128, 0, s>>>(a, w, cur); break;
    }
}

void launch_mood_cells(const StageArgs& a, const GpWeights& w, int cur, int max_trb, unsigned pass_id,
                       cudaStream_t s) {
    k_mood_cells<<<list_grid(5 * max_trb, 256), 256, 0, s>>>(a, w, cur, pass_id);
}

// ---------------------------------------------------------------------------
// Setdt (physics.f90:78-129): min over every cell, ghosts included, of
// 1/(1/(dx/(|u|+c)) + 1/(dy/(|v|+c))).  Reduced with fmin inside a CTA and an
// atomicMin on the bit pattern across CTAs (positive doubles order like their
// bits); NaN cells are ignored (IEEE minNum, as in the CPU restatement).

__device__ __forceinline__ double cell_dt(const Cell& u, double dx, double dy) {
    const double vx = u.mx / u.r;
    const double vy = u.my / u.r;
    const double p = pressure(u);
    const double c = sqrt(GPM_GAMMA * p / u.r);
    return 1.0 / (1.0 / (dx / (fabs(vx) + c)) + 1.0 / (dy / (fabs(vy) + c)));
}

__device__ __forceinline__ void dt_reduce(double v, DevScalars* sc) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ double wmin[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) wmin[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < (int)(blockDim.x >> 5) ? wmin[lane] : 1.0e30;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.0 && v < 1.0e30)  // NaN fails both tests
            atomicMin(&sc->dtmin_bits, (unsigned long long)__double_as_longlong(v));
    }
}

__global__ void __launch_bounds__(256) k_cfl(GridGeom g, const double* __restrict__ u, DevScalars* sc) {
    const size_t ncell = (size_t)g.nx * g.ny;
    double v = 1.0e30;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x)
        v = fmin(v, cell_dt(ld_cell(u + 4 * c), g.dx, g.dy));
    dt_reduce(v, sc);
}

void launch_cfl(const GridGeom& g, const double* u, DevScalars* sc, cudaStream_t s) {
    k_cfl<<<list_grid(g.nx * g.ny, 256), 256, 0, s>>>(g, u, sc);
}

// SSP-RK3 combination y = a*x + b*y over every cell (ghosts included, as the
// reference's whole-array expressions); optionally the Setdt reduction of y.
__global__ void __launch_bounds__(256) k_combine(GridGeom g, const double* __restrict__ x, double* __restrict__ y,
                                                 double ca, double cb, int with_cfl, DevScalars* sc) {
    const size_t ncell = (size_t)g.nx * g.ny;
    double v = 1.0e30;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const Cell a = ld_cell(x + 4 * c);
        const Cell b = ld_cell_cg(y + 4 * c);
        Cell o;
        o.r = ca * a.r + cb * b.r;
        o.mx = ca * a.mx + cb * b.mx;
        o.my = ca * a.my + cb * b.my;
        o.e = ca * a.e + cb * b.e;
        st_cell(y + 4 * c, o);
        if (with_cfl) v = fmin(v, cell_dt(o, g.dx, g.dy));
    }
    if (with_cfl) dt_reduce(v, sc);
}

void launch_combine(const GridGeom& g, const double* x, double* y, double a, double b, int with_cfl, DevScalars* sc,
                    cudaStream_t s) {
    k_combine<<<list_grid(g.nx * g.ny, 256), 256, 0, s>>>(g, x, y, a, b, with_cfl, sc);
}

// dt = CFL * min, clipped to dtfinal (physics.f90:292-296); qx = dt/dx.
// dtfinal < 0 selects tmax - t (main.f90:149).
__global__ void k_dt_finalize(GridGeom g, DevScalars* sc, double dtfinal_in) {
    double dt = __longlong_as_double((long long)sc->dtmin_bits);
    dt = dt * sc->cfl;
    const double dtfinal = dtfinal_in < 0.0 ? sc->tmax - sc->t : dtfinal_in;
    if (dt > dtfinal) dt = dtfinal;
    sc->dt = dt;
    sc->qx = dt / g.dx;
    sc->qy = dt / g.dy;
    sc->dtmin_bits = (unsigned long long)__double_as_longlong(1.0e30);
    if (!(dt > 0.0) || is_nan(dt) || dt == __longlong_as_double(0x7ff0000000000000LL)) sc->status |= GPM_STATUS_DT;
    sc->detected_step = 0;
}

void launch_dt_finalize(const GridGeom& g, DevScalars* sc, double dtfinal, cudaStream_t s) {
    k_dt_finalize<<<1, 1, 0, s>>>(g, sc, dtfinal);
}

__global__ void k_advance_t(DevScalars* sc) { sc->t = sc->t + sc->dt; }  // main.f90:160
void launch_advance_t(DevScalars* sc, cudaStream_t s) { k_advance_t<<<1, 1, 0, s>>>(sc); }

const KernelTable table = {launch_bc,        launch_flux_all,  launch_update_detect, launch_mood_mark,
                           launch_mood_faces, launch_mood_cells, launch_combine,      launch_cfl,
                           launch_dt_finalize, launch_advance_t};

}  // namespace GPM_NS
