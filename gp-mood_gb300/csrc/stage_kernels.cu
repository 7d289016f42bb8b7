// stage_kernels.cu -- the kernels of one GP-MOOD Runge-Kutta stage.
//
// Compiled twice into libgpmood.so:
//   -DGPM_EXACT=1 --fmad=false  -> namespace gpm_exact (bit-identical to the
//                                  reference's operation order)
//   -DGPM_EXACT=0 --fmad=true   -> namespace gpm_fast
//
// One stage (Forward_Euler, gp-mood-code/mod_FE.f90:20-190) runs as:
//   k_bc_x / k_bc_y       Boundary_C(Uin)                      BC.f90:10-421
//   k_flux_xy_tma         every face: GP recon + HLLC + quadrature, stored
//   (k_flux_tile<x|y>)    (the first MOOD pass, mod_FE.f90:73-145); fast mode
//                         both directions per tile, exact mode one per launch
//   k_update_detect       Uout = Uin + flux differences, DETECTION on every
//                         cell, troubled cells (order already lowered 5->3->1)
//                         compacted into a list
//   k_mood_loop           while the list is not empty (the MOOD loop,
//                         mod_FE.f90:69-174), in one cooperative launch:
//                         recompute the 4 faces of each troubled cell, then
//                         Uout of its 5-point cross with DETECTION there ->
//                         next list
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

#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

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
    } else if (g.bc_type == 19) {  // Dirichlet: the right states come from the host (sin), BC.f90:61-75
        if (right) {
            for (int v = 0; v < 4; v++) dst[v] = sc->bcd[j][v];
        } else {
            p2c(3.857143, 2.629369, 0., 10.33333, dst);
        }
    } else if (g.bc_type == 201 || g.bc_type == 301) {  // Mach800 jets: outflow in x, BC.f90:137-152
        const double* src = u + 4 * cidx(g, right ? g.lf : 1, n);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    } else if (g.bc_type == 401) {  // RMI: inflow left, outflow right, BC.f90:243-256
        if (right) {
            const double* src = u + 4 * cidx(g, g.lf, n);
            for (int v = 0; v < 4; v++) dst[v] = src[v];
        } else {
            p2c(2.666666666666667, 2. * sqrt(1.4), 0., 4.5, dst);
        }
    } else if (g.bc_type == 402) {  // RT: reflective in x, BC.f90:344-362
        const int ls = right ? g.lf - j : 1 + j;
        const double* src = u + 4 * cidx(g, ls, n);
        dst[0] = src[0]; dst[1] = -src[1]; dst[2] = src[2]; dst[3] = src[3];
    } else if (g.bc_type == 403) {  // KH: periodic in x, BC.f90:394-400
        const int ls = right ? 1 + j : g.lf - j;
        const double* src = u + 4 * cidx(g, ls, n);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    }
}

__global__ void k_bc_y(GridGeom g, double* __restrict__ u, const DevScalars* __restrict__ sc, int stage) {
    const int l = (int)(blockIdx.x * blockDim.y + threadIdx.y) - 3;  // every column incl. ghosts
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
    } else if (g.bc_type == 19 || g.bc_type == 403) {  // Neumann in y (BC.f90:77-87, :402-413)
        const double* src = u + 4 * cidx(g, l, top ? g.nf : 1);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    } else if (g.bc_type == 201 || g.bc_type == 301) {  // outflow, then the jets (BC.f90:154-178, :199-236)
        const double* src = u + 4 * cidx(g, l, top ? g.nf : 1);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
        if (fabs((l * g.dx - g.dx / 2) - 0.75) <= 0.05) {
            if (!top) p2c(1.4, 0.0, 800.0, 1.0, dst);
            else if (g.bc_type == 301) p2c(1.4, 0.0, -800.0, 1.0, dst);
        }
    } else if (g.bc_type == 401) {  // RMI: reflective in y, BC.f90:258-280
        const int ns = top ? g.nf - j : 1 + j;
        const double* src = u + 4 * cidx(g, l, ns);
        dst[0] = src[0]; dst[1] = src[1]; dst[2] = -src[2]; dst[3] = src[3];
    } else if (g.bc_type == 402) {  // RT: hydrostatic ghosts, g = real(0.1, 4), BC.f90:364-389
        const double* q = u + 4 * cidx(g, l, top ? g.nf - j : 1 + j);
        const double grav = (double)0.1f;
        const double pr = (GPM_GAMMA - 1.) * (q[3] - (0.5 * (q[1] * q[1] + q[2] * q[2]) / q[0]));
        const double dp = 2 * j * g.dy * grav * q[0];
        p2c(q[0], q[1] / q[0], -(q[2] / q[0]), top ? pr - dp : pr + dp, dst);
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

// Gauss-point states of face `face` of one cell at order index o: the fast
// kernels use the mirror-symmetric split for ngp = 3 above first order.
template <int DIR, int NP, int NGP>
__device__ __forceinline__ void recon_face(const GpWeights& w, int o, int face, const Cell* q, double (*u)[4]) {
#if !GPM_EXACT
    if constexpr (NGP == 3 && NP > 1) {
        gp_recon_sym3<DIR, NP>(w.sym[o][face], q, u);
        return;
    }
#endif
    gp_recon<NP, NGP>(&w.zt[o][face][0][0], q, u);
}

// NN_GP_MOOD_CC_ (mod_NN_GP_MOOD_CC.f90:63-70): with the reference network
// on, a face state of cell (l, n) at order 1 is the cell value itself and at
// order 3 the blend v1*U(l,n) + v2*Uh with (v1, v2) = values_NN(l, n) taken
// to double.  values_NN is (0, 1) except in column g.cc_col of rows 1..nf:
// the reference's network loop writes its outputs to values_NN(L, n, :)
// (mod_NN.f90:41,44; Fortran reads `l` there as the input count L), so the
// row's last cell leaves its softmax there.  A (0, 1) blend is applied like
// any other, as the reference does.
__device__ __forceinline__ void cc_weights(const GridGeom& g, const float* ccw, int l, int n, double* v1,
                                           double* v2) {
    *v1 = 0.0;
    *v2 = 1.0;
    if (l == g.cc_col && n >= 1 && n <= g.nf) {
        *v1 = (double)ccw[2 * n];
        *v2 = (double)ccw[2 * n + 1];
    }
}

template <int NP>
__device__ __forceinline__ void cc_blend(double v1, double v2, const Cell& c, double* u) {
    const double cv[4] = {c.r, c.mx, c.my, c.e};
#pragma unroll
    for (int k = 0; k < 4; k++) u[k] = NP == 1 ? cv[k] : v1 * cv[k] + v2 * u[k];
}

// ccw != NULL (NN_GP_MOOD_CC): (l, n) is the low cell of the face.
template <int DIR, int NP, int NGP>
__device__ __forceinline__ void face_from_tile(const GpWeights& w, int o, const Cell (*tile)[HX], int tx, int ty,
                                               double* F, int nflux, const float* ccw = nullptr,
                                               const GridGeom* g = nullptr, int l = 0, int n = 0) {
    constexpr int FL = DIR == 0 ? 2 : 1;  // iR (x) / iT (y) face of the low cell
    constexpr int FH = DIR == 0 ? 0 : 3;  // iL (x) / iB (y) face of the high cell
    constexpr int hx = DIR == 0 ? 1 : 0, hy = DIR == 0 ? 0 : 1;
    double uL[NGP][4], uR[NGP][4];
    {
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = tile[ty + st_oy(m)][tx + st_ox(m)];
        recon_face<DIR, NP, NGP>(w, o, FL, q, uL);
        if (ccw) {
            double v1, v2;
            cc_weights(*g, ccw, l, n, &v1, &v2);
#pragma unroll
            for (int j = 0; j < NGP; j++) cc_blend<NP>(v1, v2, q[0], uL[j]);
        }
    }
    {
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = tile[ty + hy + st_oy(m)][tx + hx + st_ox(m)];
        recon_face<DIR, NP, NGP>(w, o, FH, q, uR);
        if (ccw) {
            double v1, v2;
            cc_weights(*g, ccw, l + hx, n + hy, &v1, &v2);
#pragma unroll
            for (int j = 0; j < NGP; j++) cc_blend<NP>(v1, v2, q[0], uR[j]);
        }
    }
    quad_flux<DIR, NGP>(uL, uR, w.gw, F, nflux);
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
        face_from_tile<DIR, np_of(UORD == 0 ? 1 : UORD), NGP>(w, UORD / 2, tile, tx, ty, F, g.num_flux);
    } else {
        const size_t c0 = cidx(g, l, n), c1 = DIR == 0 ? c0 + 1 : c0 + g.nx;
        const int o = min((int)a.order[c0], (int)a.order[c1]);
        if (o >= 5) face_from_tile<DIR, 13, NGP>(w, 2, tile, tx, ty, F, g.num_flux);
        else if (o >= 3) face_from_tile<DIR, 5, NGP>(w, 1, tile, tx, ty, F, g.num_flux, a.ccw, &g, l, n);
        else face_from_tile<DIR, 1, NGP>(w, 0, tile, tx, ty, F, g.num_flux, a.ccw, &g, l, n);
    }
    double* out = (DIR == 0 ? a.fx : a.fy) + 4 * cidx(g, l, n);
    st_cell(out, Cell{F[0], F[1], F[2], F[3]});
}

template <int DIR, int NP, int NGP>
__device__ __forceinline__ void face_global(const GridGeom& g, const GpWeights& w, int o, const double* __restrict__ uin,
                                            size_t c0, double* F);

#if !GPM_EXACT
// ---------------------------------------------------------------------------
// Fast first pass at uniform order 5 with ngp = 3: both face directions of a
// tile of cells in one CTA.  Every cell's 12 face states (left/right/bottom/
// top faces at 3 Gauss points) come from the mirror-symmetry components of its
// 13-point stencil (GpOrbit): 16 operations form the components, 32 give the
// six x-face states and 32 the six y-face states, per variable -- 80 FP64
// operations for 12 states, against 128 when each face gathers its two states
// on its own.  A cell passes its left and bottom states to its neighbours
// through shared memory, keeps its right states in registers and parks its
// top states in shared memory too (registers for the three Gauss points'
// Riemann solves, which run together); then every thread solves the x face
// and the y face of which its cell is the low side.  Tiles own the interior cells (l0..l0+XT-1, n0..n0+XY-1), l0, n0 >= 1;
// one extra column (left states) and row (bottom states) is computed by two
// warps.  The faces whose low cell is a ghost -- x faces (0,n), y faces (l,0)
// -- are 32-face edge items computed face by face (edge_faces).
constexpr int XT = 32, XY = 8;          // cells per tile
constexpr int XS = 13;                  // doubles per published state set (12 used, padded)

struct XyOut {
    double lo[3][4];  // left (x) or bottom (y) face states
    double hi[3][4];  // right (x) or top (y) face states
};

__device__ __forceinline__ double tile_var(const Cell* t, int k) { return cell_var(*t, k); }

// Components of the stencil values of variable k around tile position (cx, cy).
struct Comp {
    double v[13];  // [Q0 Q1p Q2p Q3p Q4p Q5pp Q1m Q2m Q5mp Q3m Q4m Q5pm Q5mm]
};

__device__ __forceinline__ void components(const Cell (*tile)[XT + 5], int cx, int cy, int k, Comp& c) {
    auto q = [&](int ox, int oy) { return cell_var(tile[cy + oy][cx + ox], k); };
    const double qm1 = q(-1, 0), qp1 = q(1, 0), qm2 = q(-2, 0), qp2 = q(2, 0);
    const double qb1 = q(0, -1), qt1 = q(0, 1), qb2 = q(0, -2), qt2 = q(0, 2);
    const double a = q(-1, -1), b = q(1, -1), cc = q(-1, 1), d = q(1, 1);
    c.v[0] = q(0, 0);
    c.v[1] = qm1 + qp1;
    c.v[2] = qm2 + qp2;
    c.v[3] = qb1 + qt1;
    c.v[4] = qb2 + qt2;
    const double s1 = a + b, s2 = cc + d, d1 = a - b, d2 = cc - d;
    c.v[5] = s1 + s2;
    c.v[6] = qm1 - qp1;
    c.v[7] = qm2 - qp2;
    c.v[8] = d1 + d2;
    c.v[9] = qb1 - qt1;
    c.v[10] = qb2 - qt2;
    c.v[11] = s1 - s2;
    c.v[12] = d1 - d2;
}

// x family: left (lo) and right (hi) face states at Gauss points 0, 1, 2.
__device__ __forceinline__ void x_family(const GpOrbit& o, const Comp& c, int k, XyOut& r) {
    const double Ppp = o.x0[0] * c.v[0] + o.x0[1] * c.v[1] + o.x0[2] * c.v[2] + o.x0[3] * c.v[3] +
                       o.x0[4] * c.v[4] + o.x0[5] * c.v[5];
    const double Pmp = o.x0[6] * c.v[6] + o.x0[7] * c.v[7] + o.x0[8] * c.v[8];
    const double Ppm = o.x0[9] * c.v[9] + o.x0[10] * c.v[10] + o.x0[11] * c.v[11];
    const double Pmm = o.x0[12] * c.v[12];
    const double A = Ppp + Ppm, B = Pmp + Pmm, C = Ppp - Ppm, D = Pmp - Pmm;
    r.lo[0][k] = A + B;
    r.hi[0][k] = A - B;
    r.lo[2][k] = C + D;
    r.hi[2][k] = C - D;
    const double P1pp = o.x1[0] * c.v[0] + o.x1[1] * c.v[1] + o.x1[2] * c.v[2] + o.x1[3] * c.v[3] +
                        o.x1[4] * c.v[4] + o.x1[5] * c.v[5];
    const double P1mp = o.x1[6] * c.v[6] + o.x1[7] * c.v[7] + o.x1[8] * c.v[8];
    r.lo[1][k] = P1pp + P1mp;
    r.hi[1][k] = P1pp - P1mp;
}

// y family: bottom (lo) and top (hi) face states at Gauss points 0, 1, 2.
__device__ __forceinline__ void y_family(const GpOrbit& o, const Comp& c, int k, XyOut& r) {
    const double Ppp = o.y0[0] * c.v[0] + o.y0[1] * c.v[1] + o.y0[2] * c.v[2] + o.y0[3] * c.v[3] +
                       o.y0[4] * c.v[4] + o.y0[5] * c.v[5];
    const double Pmp = o.y0[6] * c.v[6] + o.y0[7] * c.v[7] + o.y0[8] * c.v[8];
    const double Ppm = o.y0[9] * c.v[9] + o.y0[10] * c.v[10] + o.y0[11] * c.v[11];
    const double Pmm = o.y0[12] * c.v[12];
    const double A = Ppp + Ppm, B = Pmp + Pmm, C = Ppp - Ppm, D = Pmp - Pmm;
    r.lo[0][k] = A + B;
    r.lo[2][k] = A - B;
    r.hi[0][k] = C + D;
    r.hi[2][k] = C - D;
    const double P1pp = o.y1[0] * c.v[0] + o.y1[1] * c.v[1] + o.y1[2] * c.v[2] + o.y1[3] * c.v[3] +
                        o.y1[4] * c.v[4] + o.y1[5] * c.v[5];
    const double P1pm = o.y1[6] * c.v[9] + o.y1[7] * c.v[10] + o.y1[8] * c.v[11];
    r.lo[1][k] = P1pp + P1pm;
    r.hi[1][k] = P1pp - P1pm;
}

__device__ __forceinline__ void publish(double* dst, const double (*st)[4]) {
#pragma unroll
    for (int g = 0; g < 3; g++)
#pragma unroll
        for (int k = 0; k < 4; k++) dst[4 * g + k] = st[g][k];
}

struct XySmem {
    Cell tile[XY + 5][XT + 5];
    double left[XY][XT][XS];    // left-face states of cells l0+1 .. l0+XT
    double bottom[XY][XT][XS];  // bottom-face states of rows n0+1 .. n0+XY
    double top[XY][XT][XS];     // each cell's own top-face states, parked during its x-face solve
};

// staged: the halo tile is already in sm.tile (TMA); otherwise load it here.
__device__ __forceinline__ void xy_tile(const GridGeom& g, const GpWeights& w, const double* __restrict__ uin,
                                        double* __restrict__ fx, double* __restrict__ fy, int l0, int n0,
                                        XySmem& sm, bool staged) {
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * XT + tx;
    if (!staged)
        for (int i = tid; i < (XT + 5) * (XY + 5); i += XT * XY) {
            const int cy = i / (XT + 5), cx = i - cy * (XT + 5);
            const int l = l0 - 2 + cx, n = n0 - 2 + cy;
            if (l >= -3 && l <= g.lf + 4 && n >= -3 && n <= g.nf + 4)
                sm.tile[cy][cx] = ld_cell(uin + 4 * cidx(g, l, n));
        }
    __syncthreads();
    const int l = l0 + tx, n = n0 + ty;
    // a cell up to (lf+1, nf+1) provides states: its stencil stays inside the padded grid
    const bool live = l <= g.lf + 1 && n <= g.nf + 1;
    XyOut xs, ys;
    if (live) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            Comp c;
            components(sm.tile, tx + 2, ty + 2, k, c);
            x_family(w.orb, c, k, xs);
            y_family(w.orb, c, k, ys);
        }
        if (tx > 0) publish(sm.left[ty][tx - 1], xs.lo);
        if (ty > 0) publish(sm.bottom[ty - 1][tx], ys.lo);
        publish(sm.top[ty][tx], ys.hi);
    }
    // the extra column (left states of cells l0+XT) and row (bottom states of n0+XY)
    if (ty == XY - 1 && l <= g.lf + 1 && n0 + XY <= g.nf + 1) {
        XyOut e;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            Comp c;
            components(sm.tile, tx + 2, XY + 2, k, c);
            y_family(w.orb, c, k, e);
        }
        publish(sm.bottom[XY - 1][tx], e.lo);
    }
    if (ty == XY - 2 && tx < XY && l0 + XT <= g.lf + 1 && n0 + tx <= g.nf + 1) {
        XyOut e;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            Comp c;
            components(sm.tile, XT + 2, tx + 2, k, c);
            x_family(w.orb, c, k, e);
        }
        publish(sm.left[tx][XT - 1], e.lo);
    }
    __syncthreads();
    if (l <= g.lf && n <= g.nf) {  // x face between (l,n) and (l+1,n)
        double uR[3][4], F[4];
        const double* src = sm.left[ty][tx];
#pragma unroll
        for (int gp = 0; gp < 3; gp++)
#pragma unroll
            for (int k = 0; k < 4; k++) uR[gp][k] = src[4 * gp + k];
        quad_flux<0, 3>(xs.hi, uR, w.gw, F);
        st_cell(fx + 4 * cidx(g, l, n), Cell{F[0], F[1], F[2], F[3]});
    }
    if (l <= g.lf && n <= g.nf) {  // y face between (l,n) and (l,n+1)
        double uL[3][4], uR[3][4], F[4];
        const double* src = sm.bottom[ty][tx];
        const double* own = sm.top[ty][tx];
#pragma unroll
        for (int gp = 0; gp < 3; gp++)
#pragma unroll
            for (int k = 0; k < 4; k++) {
                uL[gp][k] = own[4 * gp + k];
                uR[gp][k] = src[4 * gp + k];
            }
        quad_flux<1, 3>(uL, uR, w.gw, F);
        st_cell(fy + 4 * cidx(g, l, n), Cell{F[0], F[1], F[2], F[3]});
    }
}

// Edge item: faces k0 .. k0+EDGE_T-1 of the list [x faces (0,1..nf), y faces
// (1..lf,0)], one warp per item so that the few edge faces spread over many SMs.
constexpr int EDGE_T = 32;
__device__ __forceinline__ void edge_faces(const GridGeom& g, const GpWeights& w, const double* __restrict__ uin,
                                           double* __restrict__ fx, double* __restrict__ fy, int k0) {
    const int k = k0 + (int)threadIdx.x;
    double F[4];
    if (k < g.nf) {
        const size_t c0 = cidx(g, 0, k + 1);
        face_global<0, 13, 3>(g, w, 2, uin, c0, F);
        st_cell(fx + 4 * c0, Cell{F[0], F[1], F[2], F[3]});
    } else if (k < g.nf + g.lf) {
        const size_t c0 = cidx(g, k - g.nf + 1, 0);
        face_global<1, 13, 3>(g, w, 2, uin, c0, F);
        st_cell(fy + 4 * c0, Cell{F[0], F[1], F[2], F[3]});
    }
}

// One cell tile per block (x fastest).
__global__ void __launch_bounds__(XT * XY, 2) k_flux_xy(StageArgs a, const __grid_constant__ GpWeights w, int tiles_x) {
    extern __shared__ __align__(16) unsigned char xy_raw[];
    XySmem& sm = *reinterpret_cast<XySmem*>(xy_raw);
    const int by = blockIdx.x / tiles_x, bx = blockIdx.x - by * tiles_x;
    xy_tile(a.g, w, a.uin, a.fx, a.fy, 1 + bx * XT, 1 + by * XY, sm, false);
}

// ---- the same kernel with the halo tile staged by the Tensor Memory Accelerator
// The padded state is a 2-D tensor of ny rows by 4*nx doubles; one
// cp.async.bulk.tensor copies the tile's (XY+5) rows of 4*(XT+5) doubles --
// exactly the row-major layout of XySmem::tile -- into this CTA's own shared
// memory and completes on an mbarrier.  The innermost start coordinate is
// 4*(l0+1) doubles, a multiple of 32 bytes; boxes that reach past the padded
// grid on the right or top are zero-filled, and those cells feed no live
// cell's stencil.
constexpr unsigned XY_TILE_BYTES = (unsigned)sizeof(Cell) * (XT + 5) * (XY + 5);
static_assert(sizeof(XySmem::tile) == XY_TILE_BYTES, "TMA box = staged tile");
static_assert(sizeof(XySmem) % 8 == 0, "mbarrier after the tile data");

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Bounded wait for phase `parity` of an mbarrier (~1 s at most).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity) {
    for (int it = 0; it < (1 << 20); it++) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__global__ void __launch_bounds__(XT * XY, 2) k_flux_xy_tma(StageArgs a, const __grid_constant__ GpWeights w,
                                                         const __grid_constant__ CUtensorMap tm, int tiles_x) {
    extern __shared__ __align__(1024) unsigned char xy_raw[];
    XySmem& sm = *reinterpret_cast<XySmem*>(xy_raw);
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(xy_raw + sizeof(XySmem));
    const int by = blockIdx.x / tiles_x, bx = blockIdx.x - by * tiles_x;
    const int l0 = 1 + bx * XT, n0 = 1 + by * XY;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                     "r"(XY_TILE_BYTES)
                     : "memory");
        // padded cell (l0-2, n0-2) is column l0+1, row n0+1 of the padded grid
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
            "[%4];" ::"r"(smem_addr(&sm.tile[0][0])),
            "l"(reinterpret_cast<uint64_t>(&tm)), "r"(4 * (l0 + 1)), "r"(n0 + 1), "r"(smem_addr(bar))
            : "memory");
    }
    __syncthreads();  // the barrier is initialised before anyone waits on it
    const bool ok = mbar_wait(bar, 0);
    if (!__syncthreads_and(ok)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            atomicOr(&a.sc->status, GPM_STATUS_TMA);
            mbar_wait(bar, 0);  // once more, bounded, for the copy in flight before the CTA leaves
        }
        return;
    }
    xy_tile(a.g, w, a.uin, a.fx, a.fy, l0, n0, sm, true);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no -lcuda).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    return fn;
}

// The tile map of a padded state: ny rows of 4*nx doubles, boxes of XY+5 rows
// by 4*(XT+5) doubles.  False if the CUDA driver refuses it or the state is not
// 16-byte aligned (TMA's rule for the global address).
static bool encode_tile_map(CUtensorMap* m, const double* u, const GridGeom& g) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || (reinterpret_cast<uintptr_t>(u) & 15)) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)4 * g.nx, (cuuint64_t)g.ny};
    const cuuint64_t strides[1] = {(cuuint64_t)4 * g.nx * sizeof(double)};
    const cuuint32_t box[2] = {4 * (XT + 5), XY + 5};
    const cuuint32_t estr[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<double*>(u), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The faces whose low cell is a ghost, EDGE_T per block.
__global__ void __launch_bounds__(EDGE_T) k_flux_edge(StageArgs a, const __grid_constant__ GpWeights w) {
    edge_faces(a.g, w, a.uin, a.fx, a.fy, blockIdx.x * EDGE_T);
}

bool launch_flux_xy(const StageArgs& a, const GpWeights& w, cudaStream_t s) {
    static std::atomic<bool> attr[GPM_MAX_DEVICES];
    const int dev = gpm_device();
    constexpr int tma_smem = (int)sizeof(XySmem) + 8;  // + the mbarrier
    if (!attr[dev].load(std::memory_order_relaxed)) {
        cudaFuncSetAttribute(k_flux_xy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(XySmem));
        cudaFuncSetAttribute(k_flux_xy_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, tma_smem);
        attr[dev].store(true, std::memory_order_relaxed);
    }
    const int tx = (a.g.lf + XT - 1) / XT, ty = (a.g.nf + XY - 1) / XY;
    const int edges = (a.g.lf + a.g.nf + EDGE_T - 1) / EDGE_T;
    CUtensorMap tm;
    if (a.g.flux_tma && encode_tile_map(&tm, a.uin, a.g))
        k_flux_xy_tma<<<tx * ty, dim3(XT, XY), tma_smem, s>>>(a, w, tm, tx);
    else
        k_flux_xy<<<tx * ty, dim3(XT, XY), sizeof(XySmem), s>>>(a, w, tx);
    k_flux_edge<<<edges, EDGE_T, 0, s>>>(a, w);
    return true;
}
#endif

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

int launch_flux_all(const StageArgs& a, const GpWeights& w, cudaStream_t s) {
#if !GPM_EXACT
    if (a.uniform_order && a.g.mord == 5 && a.g.ngp == 3 && a.g.num_flux == 100 && launch_flux_xy(a, w, s))
        return 2;
#endif
    switch (a.g.ngp) {
    case 1: launch_flux_ngp<1>(a, w, s); break;
    case 2: launch_flux_ngp<2>(a, w, s); break;
    case 3: launch_flux_ngp<3>(a, w, s); break;
    case 4: launch_flux_ngp<4>(a, w, s); break;
    default: launch_flux_ngp<5>(a, w, s); break;
    }
    return 2;
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

// Position of the calling thread in an order that fills whole warps with
// consecutive work items and deals the warps round-robin over the CTAs (one
// or a few per SM).  An FP64 instruction costs the SM the same time whether
// 1 or 32 lanes of the warp are active, so a short list must pack its items
// into as few warps as possible, and spread those warps over the SMs.
__device__ __forceinline__ int pack_tid() {
    return (((threadIdx.x >> 5) * gridDim.x + blockIdx.x) << 5) + (threadIdx.x & 31);
}

// Face item i of the 4*nt faces of nt troubled cells: the x faces come first
// (item 2j: left face of cell j, 2j+1: its right face), then the y faces
// (below, above), so the lanes of a warp share one direction.
__device__ __forceinline__ int face_item(int i, int nt, int* dir, int* side) {
    const int x = i < 2 * nt ? 1 : 0;
    const int j = x ? i : i - 2 * nt;
    *dir = x ? 0 : 1;
    *side = j & 1;
    return j >> 1;
}

// The order cascade of a troubled cell, mod_subroutine_MOOD.f90:159-163
// (5 -> 3, 3 -> 1).  It is applied by the thread that finds the cell troubled,
// when it lists the cell: no other thread reads that cell's order before the
// next pass's faces, which come after a grid barrier or a kernel boundary.
__device__ __forceinline__ void cascade_order(int8_t* o) {
    const int v = *o;
    *o = (int8_t)(v == 3 ? 1 : (v > 3 ? 3 : v));
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
        else if (inadmissible(uo)) atomicOr(&a.sc->status, GPM_STATUS_NAN);
    }
    if (trb) cascade_order(&a.order[c]);
    list_append(trb, a.tlist[cur], &a.sc->ntrb[cur], (int)c);
}

void launch_update_detect(const StageArgs& a, const GpWeights& w, int cur, cudaStream_t s) {
    const dim3 grid((a.g.lf + 31) / 32, (a.g.nf + 7) / 8), blk(32, 8);
    k_update_detect<<<grid, blk, 0, s>>>(a, w, cur);
}

// ---------------------------------------------------------------------------
// MOOD passes 2, 3, ... on the troubled list only.

constexpr int LIST_CTAS_PER_SM = 4;

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
        recon_face<DIR, NP, NGP>(w, o, FL, q, uL);
    }
    {
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = ld_cell(uin + 4 * (c1 + st_ox(m) + row * st_oy(m)));
        recon_face<DIR, NP, NGP>(w, o, FH, q, uR);
    }
    quad_flux<DIR, NGP>(uL, uR, w.gw, F, g.num_flux);
}

// The MOOD face phase, split by Gauss point.  A pass's face list is short
// (the faces of the cells lowered in the previous pass), so the SMs hold one
// or two warps each and a pass waits on one warp's chain of dependent FP64
// instructions.  NGP consecutive lanes share a face: each reconstructs both
// sides at its own Gauss point (gp_recon_at, the per-point sum of
// mod_GP_MOOD.f90:61) and solves that point's Riemann problem; the face's
// lanes gather the NGP fluxes by shuffles and sum them in Gauss-point order
// with quad_flux's expression, and the first lane stores the face.  The chain
// is one Gauss point's work instead of the face's.  A listed cell was lowered
// when it was listed, so its faces are at order <= 3; the 13-point branch only
// keeps the function total.
struct FaceGp {
    double F[4];        // this lane's Gauss-point flux
    double* out;        // the face's stored flux
    const double* gw;   // Gauss weights
};

// The two face states of one Gauss point at order NP (stencil straight from
// global memory).
template <int DIR, int NP>
__device__ __forceinline__ void face_gp_states(const GridGeom& g, const GpWeights& w, int o,
                                               const double* __restrict__ uin, size_t c0, int gp, double* uL,
                                               double* uR, const float* ccw) {
    constexpr int FL = DIR == 0 ? 2 : 1;
    constexpr int FH = DIR == 0 ? 0 : 3;
    constexpr int hx = DIR == 0 ? 1 : 0, hy = DIR == 0 ? 0 : 1;
    const ptrdiff_t row = g.nx;
    const size_t c1 = DIR == 0 ? c0 + 1 : c0 + g.nx;
    const int l0 = (int)(c0 % (size_t)g.nx) - 3, n0 = (int)(c0 / (size_t)g.nx) - 3;  // low cell (l, n)
    {
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = ld_cell(uin + 4 * (c0 + st_ox(m) + row * st_oy(m)));
        gp_recon_at<NP>(&w.zt[o][FL][gp][0], q, uL);
        if (ccw) {
            double v1, v2;
            cc_weights(g, ccw, l0, n0, &v1, &v2);
            cc_blend<NP>(v1, v2, q[0], uL);
        }
    }
    {
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = ld_cell(uin + 4 * (c1 + st_ox(m) + row * st_oy(m)));
        gp_recon_at<NP>(&w.zt[o][FH][gp][0], q, uR);
        if (ccw) {
            double v1, v2;
            cc_weights(g, ccw, l0 + hx, n0 + hy, &v1, &v2);
            cc_blend<NP>(v1, v2, q[0], uR);
        }
    }
}

// Lanes of one warp may hold faces of different orders: only the
// reconstruction branches on the order, and the Riemann solve runs once for
// the whole warp after the branches rejoin (an FP64 warp instruction costs
// its SM partition ~64 cycles however many lanes are active, so a solve in
// each branch would double the pass's critical path).
template <int DIR>
__device__ __forceinline__ void face_gp_any(const StageArgs& a, const GpWeights& w, size_t c0, int gp, FaceGp& f) {
    const GridGeom& g = a.g;
    const size_t c1 = DIR == 0 ? c0 + 1 : c0 + g.nx;
    const int o = min((int)a.order[c0], (int)a.order[c1]);
    double uL[4], uR[4];
    if (o >= 5) face_gp_states<DIR, 13>(g, w, 2, a.uin, c0, gp, uL, uR, nullptr);
    else if (o >= 3) face_gp_states<DIR, 5>(g, w, 1, a.uin, c0, gp, uL, uR, a.ccw);
    else face_gp_states<DIR, 1>(g, w, 0, a.uin, c0, gp, uL, uR, a.ccw);
    riemann<DIR>(g.num_flux, uL, uR, f.F);
    f.out = (DIR == 0 ? a.fx : a.fy) + 4 * c0;
    f.gw = w.gw;
}

// The same face item with the direction a runtime value (0: x face between
// c0 and c0+1, 1: y face between c0 and c0+nx): the reconstruction reads the
// weights of the face's sides by index and HLLC runs as hllc_dyn, so a warp
// may hold x and y faces at once; in the exact mode the bits are
// face_gp_any's.  Other Riemann solvers branch on the direction.
__device__ __forceinline__ void face_gp_dyn(const StageArgs& a, const GpWeights& w, size_t c0, int dir, int gp,
                                            FaceGp& f) {
    const GridGeom& g = a.g;
    const size_t c1 = c0 + (dir == 0 ? (size_t)1 : (size_t)g.nx);
    const int o = min((int)a.order[c0], (int)a.order[c1]);
    const int FL = dir == 0 ? 2 : 1, FH = dir == 0 ? 0 : 3;
    const ptrdiff_t row = g.nx;
    double uL[4], uR[4];
    if (o >= 5) {
        Cell q[13];
#pragma unroll
        for (int m = 0; m < 13; m++) q[m] = ld_cell(a.uin + 4 * (c0 + st_ox(m) + row * st_oy(m)));
        gp_recon_at<13>(&w.zt[2][FL][gp][0], q, uL);
#pragma unroll
        for (int m = 0; m < 13; m++) q[m] = ld_cell(a.uin + 4 * (c1 + st_ox(m) + row * st_oy(m)));
        gp_recon_at<13>(&w.zt[2][FH][gp][0], q, uR);
    } else {
        const int NPo = o >= 3 ? 1 : 0;  // weight set: order 3 or 1
        Cell q[5];
#pragma unroll
        for (int m = 0; m < 5; m++) q[m] = ld_cell(a.uin + 4 * (c0 + st_ox(m) + row * st_oy(m)));
        if (o >= 3) gp_recon_at<5>(&w.zt[NPo][FL][gp][0], q, uL);
        else gp_recon_at<1>(&w.zt[0][FL][gp][0], q, uL);
        if (a.ccw) {
            const int l0 = (int)(c0 % (size_t)g.nx) - 3, n0 = (int)(c0 / (size_t)g.nx) - 3;
            double v1, v2;
            cc_weights(g, a.ccw, l0, n0, &v1, &v2);
            if (o >= 3) cc_blend<5>(v1, v2, q[0], uL);
            else cc_blend<1>(v1, v2, q[0], uL);
        }
#pragma unroll
        for (int m = 0; m < 5; m++) q[m] = ld_cell(a.uin + 4 * (c1 + st_ox(m) + row * st_oy(m)));
        if (o >= 3) gp_recon_at<5>(&w.zt[NPo][FH][gp][0], q, uR);
        else gp_recon_at<1>(&w.zt[0][FH][gp][0], q, uR);
        if (a.ccw) {
            const int l0 = (int)(c0 % (size_t)g.nx) - 3, n0 = (int)(c0 / (size_t)g.nx) - 3;
            double v1, v2;
            cc_weights(g, a.ccw, l0 + (dir == 0), n0 + (dir == 1), &v1, &v2);
            if (o >= 3) cc_blend<5>(v1, v2, q[0], uR);
            else cc_blend<1>(v1, v2, q[0], uR);
        }
    }
    if (g.num_flux == 100) hllc_dyn(uL, uR, dir, f.F);
    else if (dir == 0) riemann<0>(g.num_flux, uL, uR, f.F);
    else riemann<1>(g.num_flux, uL, uR, f.F);
    f.out = (dir == 0 ? a.fx : a.fy) + 4 * c0;
    f.gw = w.gw;
}

// Faces 0 .. nf-1 dealt to whole warps (stid: pack_tid, gstride: threads of
// the grid); item(i, gp, f) fills face i's Gauss point gp.  Faces 0 .. n0-1
// (the x faces) and n0 .. nf-1 (the y faces) start on warp boundaries, so no
// warp runs both directions' code.  Every lane of a warp runs the same trip
// count, so the shuffles see full warps.
template <int NGP, class Item>
__device__ __forceinline__ void face_phase_gp(int nf, int n0, int stid, int gstride, Item item) {
    constexpr int FPW = 32 / NGP;  // faces per warp
    const int lane = threadIdx.x & 31, fl = lane / NGP, gp = lane - fl * NGP, lead = lane - gp;
    const int w0 = (n0 + FPW - 1) / FPW, nw = w0 + (nf - n0 + FPW - 1) / FPW;
    for (int wi = stid >> 5; wi < nw; wi += gstride >> 5) {
        const int i = wi < w0 ? wi * FPW + fl : n0 + (wi - w0) * FPW + fl;
        const bool act = fl < FPW && i < (wi < w0 ? n0 : nf);
        FaceGp f;
        f.F[0] = f.F[1] = f.F[2] = f.F[3] = 0.0;
        f.out = nullptr;
        f.gw = nullptr;
        if (act) item(i, gp, f);
        double acc[4];
#pragma unroll
        for (int j = 0; j < NGP; j++) {
            const int src = min(lead + j, 31);
            const double wj = act ? f.gw[j] : 0.0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const double v = __shfl_sync(0xffffffffu, f.F[k], src);
                acc[k] = (j == 0) ? v * wj : acc[k] + v * wj;
            }
        }
        if (act && gp == 0) {
#if GPM_EXACT
#pragma unroll
            for (int k = 0; k < 4; k++) acc[k] = plus_zero(acc[k]);
#endif
            st_cell(f.out, Cell{acc[0], acc[1], acc[2], acc[3]});
        }
    }
}

template <int NGP>
__global__ void __launch_bounds__(128) k_mood_faces(StageArgs a, const __grid_constant__ GpWeights w, int cur) {
    const int nt = a.sc->ntrb[cur];
    // 4 faces per troubled cell: x faces (l-1,n), (l,n), y faces (l,n-1), (l,n)
    face_phase_gp<NGP>(4 * nt, 2 * nt, pack_tid(), gridDim.x * blockDim.x, [&](int i, int gp, FaceGp& f) {
        int dir, side;
        const size_t c = (size_t)a.tlist[cur][face_item(i, nt, &dir, &side)];
        if (dir == 0) face_gp_any<0>(a, w, side == 0 ? c - 1 : c, gp, f);
        else face_gp_any<1>(a, w, side == 0 ? c - a.g.nx : c, gp, f);
    });
}

// ---------------------------------------------------------------------------
// The whole MOOD loop on the device: one cooperative launch runs passes 2, 3,
// ... until the troubled list is empty, with a grid barrier after each of the
// two phases of a pass (faces, crosses; the cascade is applied when a cell is
// listed).  Every CTA is co-resident
// (cooperative launch), so the barrier cannot wait on an unscheduled CTA; its
// spin is still bounded, and a timeout records GPM_STATUS_BARRIER and makes
// every CTA leave.

// Threads per CTA of the cooperative MOOD loops: one 16-warp CTA per SM
// keeps the barrier's arrival count at the SM count.
constexpr int MOOD_THREADS = 512;

__device__ __forceinline__ bool grid_sync(GridBar* b) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &b->gen;
        const unsigned g = *vgen;
        const int lim = *(volatile int*)&b->limit;
        const long long max_it = lim > 0 ? lim : (1LL << 24);  // ~1 s: far beyond any pass
        __threadfence();
        if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
            atomicExch(&b->count, 0u);
            __threadfence();
            atomicAdd(&b->gen, 1u);
        } else {
            long long it = 0;
            while (*vgen == g) {
                if (++it > max_it) {
                    atomicExch(&b->err, 1);
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)&b->err == 0;
}

// Passes whose troubled list holds at most GridGeom::mood_solo cells run in CTA 0
// alone, with CTA barriers: such a pass is a few dependent chains of FP64
// work, and two grid barriers cost more than its work.  Every CTA reads the
// same count after a grid barrier, so all take the switch at the same pass;
// the others leave and CTA 0 runs the loop to its end (a list that grows
// again is still done, by one CTA's threads).  Runs whose cascade crawls
// cell by cell need hundreds of such passes per stage.
__device__ __forceinline__ bool mood_sync(GridBar* b, bool solo) {
    if (solo) {
        __syncthreads();
        return true;
    }
    return grid_sync(b);
}

// The cross phase of a pass run by one CTA (solo).  A lone warp pays ~64
// cycles for every FP64 instruction, so one cross cell's DETECTION chain
// (update, positivity, DMP bounds, shock detector, U2 in x and in y) is what
// a short pass waits on.  Its parts are split over five warp roles that run
// at once on every cross cell of a chunk: role 0 updates Uout and runs the
// Uout tests (mood_uout_part), roles 1-4 the Uin-only tests -- the shock
// detector's flow half, the two U2 tests and the shock detector's
// pressure-jump half; after a CTA barrier role 0 combines them, lowers the
// order of a troubled cell and lists it.  The decision is mood_troubled's.
// Warp w takes role w % 5; 16 warps give every role at least 3 warps.
constexpr int SOLO_ROLES = 5;
constexpr int SOLO_CHUNK = (MOOD_THREADS / 32 / SOLO_ROLES) * 32;  // cross cells per chunk (96)
// One-CTA passes keep the troubled lists in shared memory (every entry is also
// written to the global list, which a list longer than this is read from):
// reading a list entry and appending one then costs the SM's shared-memory
// latency instead of an L2 round trip or a global atomic.
constexpr int SOLO_LIST_CAP = 2048;

struct SoloCross {
    int cell[SOLO_CHUNK];
    int8_t part[SOLO_CHUNK];      // mood_uout_part; -1: ghost cell or already updated in this pass
    int8_t ord[SOLO_CHUNK];       // the cell's order when it was checked
    bool flag[4][SOLO_CHUNK];     // shock flow half, U2 smooth in x, U2 smooth in y, shock pressure-jump half
};

struct SoloLists {
    int list[2][SOLO_LIST_CAP];
    int count[2];
};

// lst: the current troubled list (shared or global), nt entries.  A cross
// cell that several listed cells share is updated once: in a pass that fits
// one chunk by the first listed cell whose cross holds it (a scan of the
// shared list), otherwise by whoever stamps it first (global atomics).
__device__ __forceinline__ void solo_cross(const StageArgs& a, const GpWeights& w, int cur, int nt, unsigned pid,
                                           const int* lst, SoloCross& sm, SoloLists& sl) {
    const GridGeom& g = a.g;
    const double qx = a.sc->qx, qy = a.sc->qy;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int role = warp % SOLO_ROLES, j = (warp / SOLO_ROLES) * 32 + lane;  // item of the chunk
    const bool slot = j < SOLO_CHUNK;  // a role's fourth warp (warp 15) has no items
    const int nxt = cur ^ 1, total = 5 * nt;
    const bool scan = total <= SOLO_CHUNK && nt <= SOLO_LIST_CAP;  // one chunk, list in shared memory
    const int nx = g.nx;
    for (int base = 0; base < total; base += SOLO_CHUNK) {
        const int i = base + j;
        if (slot && i < total) {
            const int q = i / 5;
            const size_t t = (size_t)lst[q];
            const int k = i % 5;
            const size_t c = k == 0 ? t - nx : k == 1 ? t - 1 : k == 2 ? t : k == 3 ? t + 1 : t + nx;
            const int l = (int)(c % (size_t)nx) - 3, n = (int)(c / (size_t)nx) - 3;
            const bool interior = l >= 1 && l <= g.lf && n >= 1 && n <= g.nf;
            const double* uin = a.uin + 4 * c;
            if (role == 0) {
                bool own = interior;
                if (own && scan) {
                    for (int q2 = 0; q2 < q; q2++) {
                        const long long d = (long long)c - (long long)lst[q2];
                        if (d == 0 || d == 1 || d == -1 || d == nx || d == -nx) own = false;
                    }
                } else if (own) {
                    own = atomicExch(&a.stamp[c], pid) != pid;
                }
                int r = -1, o = 0;
                if (own) {
                    const Cell uo = cell_update(g, a.uin, a.fx, a.fy, c, qx, qy);
                    st_cell(a.uout + 4 * c, uo);
                    o = a.order[c];
                    if (o > 1) {
                        r = mood_uout_part(uo, uin, nx, g);
                    } else {
                        if (inadmissible(uo)) atomicOr(&a.sc->status, GPM_STATUS_NAN);
                        r = 0;
                    }
                }
                sm.cell[j] = (int)c;
                sm.part[j] = (int8_t)r;
                sm.ord[j] = (int8_t)o;
            } else if (interior) {
                sm.flag[role - 1][j] = role == 1   ? mood_shock_flow_part(uin, nx, g)
                                       : role == 2 ? mood_u2_smooth<0>(uin, nx, g, w.d2x)
                                       : role == 3 ? mood_u2_smooth<1>(uin, nx, g, w.d2y)
                                                   : mood_shock_grad_part(uin, nx, g);
            }
        }
        __syncthreads();
        if (role == 0) {
            bool trb = false;
            int cval = 0;
            if (slot && i < total && sm.part[j] >= 0) {
                const int r = sm.part[j];
                cval = sm.cell[j];
                const bool shock = sm.flag[0][j] && sm.flag[3][j];
                trb = r == 1 || (r == 2 && shock && !(g.u2 && (sm.flag[1][j] || sm.flag[2][j])));
            }
            if (trb) {  // the cascade of cascade_order, on the order read above
                const int v = sm.ord[j];
                a.order[cval] = (int8_t)(v == 3 ? 1 : (v > 3 ? 3 : v));
            }
            // warp-aggregated append to the next list, shared and global
            const unsigned m = __ballot_sync(0xffffffffu, trb);
            if (m) {
                int b0 = 0;
                if (lane == 0) b0 = atomicAdd(&sl.count[nxt], __popc(m));
                b0 = __shfl_sync(0xffffffffu, b0, 0);
                if (trb) {
                    const int idx = b0 + __popc(m & ((1u << lane) - 1));
                    a.tlist[nxt][idx] = cval;
                    if (idx < SOLO_LIST_CAP) sl.list[nxt][idx] = cval;
                }
            }
        }
        __syncthreads();
    }
}

template <int NGP>
__global__ void __launch_bounds__(MOOD_THREADS, 1) k_mood_loop(StageArgs a, const __grid_constant__ GpWeights w, GridBar* bar,
                                                      int max_pass, int stage) {
    __shared__ SoloCross solo_sm;
    __shared__ SoloLists solo_ls;
    const GridGeom& g = a.g;
    const double qx = a.sc->qx, qy = a.sc->qy;
    const unsigned epoch = a.sc->stamp_epoch;  // stamps epoch+2, epoch+3, ... are new
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
    int stid = pack_tid(), wstride = gstride;  // whole warps of work items, dealt over all SMs
    bool solo = false, shared_lists = false;  // shared_lists: a one-CTA loop with role-split DETECTION
    int cur = 0, pass = 1;  // pass 1 (all faces) ran before this kernel
    for (;;) {
        const int nt = shared_lists ? solo_ls.count[cur] : *(volatile int*)&a.sc->ntrb[cur];
        if (nt == 0) break;
        if (pass >= max_pass) {
            if (gtid == 0) a.sc->status |= GPM_STATUS_MOODCAP;
            break;
        }
        if (!solo && nt <= g.mood_solo) {
            if (blockIdx.x != 0) return;
            solo = true;
            stid = threadIdx.x;
            wstride = blockDim.x;
            if (g.solo_split) {  // from here on the lists also live in shared memory
                shared_lists = true;
                for (int i = threadIdx.x; i < nt && i < SOLO_LIST_CAP; i += blockDim.x)
                    solo_ls.list[cur][i] = a.tlist[cur][i];
                if (threadIdx.x == 0) solo_ls.count[cur] = nt;
                __syncthreads();
            }
        }
        pass++;
        // the listed cells' orders were lowered when they were listed
        if (gtid == 0) {
            a.sc->ntrb[cur ^ 1] = 0;  // nobody appends to it before the next barrier
            a.sc->detected_step += (unsigned long long)nt;
            if (shared_lists) solo_ls.count[cur ^ 1] = 0;
        }
        const int* lst = shared_lists && nt <= SOLO_LIST_CAP ? solo_ls.list[cur] : a.tlist[cur];
        // the four faces of every troubled cell at the new orders
        // x and y faces share warps (face_gp_dyn): 4*nt items packed densely
        face_phase_gp<NGP>(4 * nt, 4 * nt, stid, wstride, [&](int i, int gp, FaceGp& f) {
            int dir, side;
            const size_t c = (size_t)lst[face_item(i, nt, &dir, &side)];
            face_gp_dyn(a, w, side == 0 ? (dir == 0 ? c - 1 : c - g.nx) : c, dir, gp, f);
        });
        if (!mood_sync(bar, solo)) return;
        // the 5-point crosses: Uout from Uin and the current fluxes, DETECTION
        const unsigned pid = epoch + (unsigned)pass;
        if (shared_lists) {
            solo_cross(a, w, cur, nt, pid, lst, solo_sm, solo_ls);
            cur ^= 1;
            continue;
        }
        const int nxt = cur ^ 1, total = 5 * nt;
        const int lim = ((total + wstride - 1) / wstride) * wstride;
        for (int base = 0; base < lim; base += wstride) {
            const int i = base + stid;
            bool trb = false;
            int cval = 0;
            if (i < total) {
                const size_t t = (size_t)a.tlist[cur][i / 5];
                const int k = i % 5;
                const size_t c = k == 0 ? t - g.nx : k == 1 ? t - 1 : k == 2 ? t : k == 3 ? t + 1 : t + g.nx;
                const int l = (int)(c % (size_t)g.nx) - 3, n = (int)(c / (size_t)g.nx) - 3;
                if (l >= 1 && l <= g.lf && n >= 1 && n <= g.nf && atomicExch(&a.stamp[c], pid) != pid) {
                    const Cell uo = cell_update(g, a.uin, a.fx, a.fy, c, qx, qy);
                    st_cell(a.uout + 4 * c, uo);
                    if (a.order[c] > 1) trb = mood_troubled(uo, a.uin + 4 * c, g.nx, g, w.d2x, w.d2y);
                    else if (inadmissible(uo)) atomicOr(&a.sc->status, GPM_STATUS_NAN);
                    cval = (int)c;
                }
            }
            if (trb) cascade_order(&a.order[cval]);
            list_append(trb, a.tlist[nxt], &a.sc->ntrb[nxt], cval);
        }
        if (!mood_sync(bar, solo)) return;
        cur ^= 1;
    }
    if (gtid == 0) {  // every CTA read the epoch before the first barrier
        a.sc->passes_stage[stage] = pass;
        a.sc->stamp_epoch = epoch + (unsigned)pass + 1u;
        if (shared_lists) a.sc->ntrb[cur] = solo_ls.count[cur];
    }
}

template <int NGP>
static int launch_mood_loop_n(const StageArgs& a, const GpWeights& w, GridBar* bar, int max_pass, int stage,
                              cudaStream_t s) {
    static std::atomic<int> grids[GPM_MAX_DEVICES];
    const int dev = gpm_device();
    int grid = grids[dev].load(std::memory_order_relaxed);
    if (!grid) {
        int sms = 0, occ = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mood_loop<NGP>, MOOD_THREADS, 0);
        grid = sms * (occ > 0 ? occ : 1);
        grids[dev].store(grid, std::memory_order_relaxed);
    }
    StageArgs aa = a;
    GpWeights ww = w;
    void* args[] = {&aa, &ww, &bar, &max_pass, &stage};
    return cudaLaunchCooperativeKernel((const void*)k_mood_loop<NGP>, dim3(grid), dim3(MOOD_THREADS), args, 0, s) == cudaSuccess
               ? 0
               : -1;
}

int launch_mood_loop(const StageArgs& a, const GpWeights& w, GridBar* bar, int max_pass, int stage,
                     cudaStream_t s) {
    switch (a.g.ngp) {
    case 1: return launch_mood_loop_n<1>(a, w, bar, max_pass, stage, s);
    case 2: return launch_mood_loop_n<2>(a, w, bar, max_pass, stage, s);
    case 3: return launch_mood_loop_n<3>(a, w, bar, max_pass, stage, s);
    case 4: return launch_mood_loop_n<4>(a, w, bar, max_pass, stage, s);
    default: return launch_mood_loop_n<5>(a, w, bar, max_pass, stage, s);
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


// The gate's extras repair (optional): a gated cell whose update from the
// uniform first pass (every face at mord, already stored) passes DETECTION is
// given mord back before the gated cells' faces are recomputed, so that only
// cells plain MOOD would also flag in its first pass start lowered.  The
// a-priori count drops by the cells given back.
__global__ void __launch_bounds__(256) k_gate_repair(StageArgs a, const __grid_constant__ GpWeights w) {
    const GridGeom& g = a.g;
    const int n = a.sc->ntrb[1];
    const double qx = a.sc->qx, qy = a.sc->qy;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const size_t c = (size_t)a.tlist[1][i];
        const Cell uo = cell_update(g, a.uin, a.fx, a.fy, c, qx, qy);
        if (!mood_troubled(uo, a.uin + 4 * c, g.nx, g, w.d2x, w.d2y)) {
            a.order[c] = (int8_t)g.mord;
            atomicAdd(&a.sc->apriori_step, ~0ull);  // minus one
        }
    }
}

void launch_gate_repair(const StageArgs& a, const GpWeights& w, int max_items, cudaStream_t s) {
    k_gate_repair<<<list_grid(max_items, 256), 256, 0, s>>>(a, w);
}

// ---------------------------------------------------------------------------
// Setdt (physics.f90:78-129): min over every cell, ghosts included, of
// 1/(1/(dx/(|u|+c)) + 1/(dy/(|v|+c))).  Reduced with fmin inside a CTA and an
// atomicMin on the bit pattern across CTAs (positive doubles order like their
// bits); NaN cells are ignored (IEEE minNum, as in the CPU restatement).

#if GPM_EXACT
__device__ __forceinline__ double cell_dt(const Cell& u, double dx, double dy) {
    const double vx = u.mx / u.r;
    const double vy = u.my / u.r;
    const double p = pressure(u);
    const double c = sqrt(GPM_GAMMA * p / u.r);
    return 1.0 / (1.0 / (dx / (fabs(vx) + c)) + 1.0 / (dy / (fabs(vy) + c)));
}
#else
// Fast mode: dx*dy / ((|u|+c)*dy + (|v|+c)*dx) with Newton reciprocals and
// the fast square root, equal to the form above up to rounding (a NaN or
// non-positive cell still gives NaN or a non-positive value, which the
// reduction skips).
__device__ __forceinline__ double cell_dt(const Cell& u, double dx, double dy) {
    const double ir = gpm_fast_rcp(u.r);
    const double vx = u.mx * ir, vy = u.my * ir;
    const double c = gpm_fast_sqrt(GPM_GAMMA * pressure_ir(u, ir) * ir);
    return dx * dy * gpm_fast_rcp((fabs(vx) + c) * dy + (fabs(vy) + c) * dx);
}
#endif

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

// y = c[0]*x[0] + c[1]*x[1] + ... (n terms, summed left to right as the
// reference's whole-array expressions of mod_SSP_RK4.f90:25-36 and
// mod_FE.f90:188), over every cell; y may be one of the x.
struct LinComb {
    const double* x[5];
    double c[5];
    int n;
};

__global__ void __launch_bounds__(256) k_lincomb(GridGeom g, double* y, LinComb lc, int with_cfl, DevScalars* sc) {
    const size_t ncell = (size_t)g.nx * g.ny;
    double v = 1.0e30;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const Cell a = ld_cell_cg(lc.x[0] + 4 * c);
        Cell o{lc.c[0] * a.r, lc.c[0] * a.mx, lc.c[0] * a.my, lc.c[0] * a.e};
        for (int i = 1; i < lc.n; i++) {
            const Cell b = ld_cell_cg(lc.x[i] + 4 * c);
            o.r = o.r + lc.c[i] * b.r;
            o.mx = o.mx + lc.c[i] * b.mx;
            o.my = o.my + lc.c[i] * b.my;
            o.e = o.e + lc.c[i] * b.e;
        }
        st_cell(y + 4 * c, o);
        if (with_cfl) v = fmin(v, cell_dt(o, g.dx, g.dy));
    }
    if (with_cfl) dt_reduce(v, sc);
}

void launch_lincomb(const GridGeom& g, double* y, int n, const double* const* x, const double* c, int with_cfl,
                    DevScalars* sc, cudaStream_t s) {
    LinComb lc{};
    lc.n = n;
    for (int i = 0; i < n; i++) {
        lc.x[i] = x[i];
        lc.c[i] = c[i];
    }
    k_lincomb<<<list_grid(g.nx * g.ny, 256), 256, 0, s>>>(g, y, lc, with_cfl, sc);
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

const KernelTable table = {launch_bc,          launch_flux_all,  launch_update_detect, launch_mood_faces,
                           launch_combine,     launch_cfl,       launch_dt_finalize,   launch_advance_t,
                           launch_mood_loop,   launch_lincomb,   launch_gate_repair};

}  // namespace GPM_NS

// ===========================================================================
// Batched stepping: many independent problems of uneven size (batch_common.h).
// Every phase of an RK stage is one persistent launch over all problems'
// work items, so a whole step has a fixed launch sequence that is captured
// once as a CUDA graph.  Per-problem arithmetic is the single-problem path's.
#include "batch_common.h"

namespace GPM_NS {

__device__ __forceinline__ GridGeom bgeom(const BatchArgs& a, const BProb& p) {
    GridGeom g;
    g.lf = p.lf; g.nf = p.nf; g.nx = p.nx; g.ny = p.ny;
    g.dx = p.dx; g.dy = p.dy;
    g.bc_type = a.bc_type; g.ngp = a.ngp; g.mord = a.mord; g.method = a.method;
    g.dmp = a.dmp; g.u2 = a.u2; g.u2_tol = a.u2_tol; g.u2_fd = 0; g.num_flux = a.num_flux;
    g.mood_solo = a.mood_solo;
    g.flux_tma = 0;
    g.solo_split = 0;
    g.cc_col = -1;
    return g;
}

// Boundary_C of every problem: blockIdx.y is the problem.
__global__ void kb_bc_x(BatchArgs a, double* __restrict__ u) {
    const BProb P = a.prob[blockIdx.y];
    const GridGeom g = bgeom(a, P);
    const int n = 1 + blockIdx.x * blockDim.y + threadIdx.y, k = threadIdx.x;
    if (n > g.nf || k >= 2 * GPM_NGC) return;
    double* ub = u + 4 * P.off;
    const bool right = k >= GPM_NGC;
    const int j = right ? k - GPM_NGC : k;
    const int l = right ? g.lf + 1 + j : -j;
    double* dst = ub + 4 * cidx(g, l, n);
    if (g.bc_type == 17) {
        const double* src = ub + 4 * cidx(g, right ? g.lf : 1, n);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    } else if (g.bc_type == 18) {
        const double* src = ub + 4 * cidx(g, right ? 1 + j : g.lf - j, n);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    } else if (g.bc_type == 20) {
        const double* src = ub + 4 * cidx(g, right ? g.lf - j : 1 + j, n);
        dst[0] = src[0]; dst[1] = -src[1]; dst[2] = src[2]; dst[3] = src[3];
    }
}

__global__ void kb_bc_y(BatchArgs a, double* __restrict__ u) {
    const BProb P = a.prob[blockIdx.y];
    const GridGeom g = bgeom(a, P);
    const int l = (int)(blockIdx.x * blockDim.y + threadIdx.y) - 3, k = threadIdx.x;
    if (l > g.lf + GPM_NGC || k >= 2 * GPM_NGC) return;
    double* ub = u + 4 * P.off;
    const bool top = k >= GPM_NGC;
    const int j = top ? k - GPM_NGC : k;
    const int n = top ? g.nf + 1 + j : -j;
    double* dst = ub + 4 * cidx(g, l, n);
    if (g.bc_type == 17) {
        const double* src = ub + 4 * cidx(g, l, top ? g.nf : 1);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    } else if (g.bc_type == 18) {
        const double* src = ub + 4 * cidx(g, l, top ? 1 + j : g.nf - j);
        for (int v = 0; v < 4; v++) dst[v] = src[v];
    } else if (g.bc_type == 20) {
        const double* src = ub + 4 * cidx(g, l, top ? g.nf - j : 1 + j);
        dst[0] = src[0]; dst[1] = src[1]; dst[2] = -src[2]; dst[3] = src[3];
    }
}

static int g_max_nx = 0;  // set by the batch host code before launches (largest nx/ny of the batch)

void blaunch_bc(const BatchArgs& a, double* u, cudaStream_t s) {
    const dim3 blk(8, 32);
    kb_bc_x<<<dim3((g_max_nx + 31) / 32, a.nprob), blk, 0, s>>>(a, u);
    kb_bc_y<<<dim3((g_max_nx + 31) / 32, a.nprob), blk, 0, s>>>(a, u);
}

// Face tiles of every problem: a persistent CTA walks the tile list.  Tile
// shape TXB x TYB is a template parameter chosen by the autotuner.
template <int DIR, int NP, int NGP, int HXB>
__device__ __forceinline__ void face_tile_b(const GpWeights& w, int o, const Cell* tile, int tx, int ty, double* F,
                                            int nflux) {
    constexpr int FL = DIR == 0 ? 2 : 1;
    constexpr int FH = DIR == 0 ? 0 : 3;
    double uL[NGP][4], uR[NGP][4];
    {
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = tile[(ty + st_oy(m)) * HXB + tx + st_ox(m)];
        recon_face<DIR, NP, NGP>(w, o, FL, q, uL);
    }
    {
        constexpr int hx = DIR == 0 ? 1 : 0, hy = DIR == 0 ? 0 : 1;
        Cell q[NP];
#pragma unroll
        for (int m = 0; m < NP; m++) q[m] = tile[(ty + hy + st_oy(m)) * HXB + tx + hx + st_ox(m)];
        recon_face<DIR, NP, NGP>(w, o, FH, q, uR);
    }
    quad_flux<DIR, NGP>(uL, uR, w.gw, F, nflux);
}

template <int TXB, int TYB, int NGP, int ORD>
__global__ void __launch_bounds__(TXB* TYB) kb_flux(BatchArgs a) {
    constexpr int HXB = TXB + 5, HYB = TYB + 5;
    __shared__ Cell tile[HXB * HYB];
    const int tid = threadIdx.y * TXB + threadIdx.x;
    for (int item = blockIdx.x; item < a.nftiles; item += gridDim.x) {
        const int4 it = a.ftiles[item];
        const BProb P = a.prob[it.x];
        const GridGeom g = bgeom(a, P);
        const GpWeights& w = a.wtab[P.wc];
        const double* ub = a.uin + 4 * P.off;
        __syncthreads();  // the previous tile's faces are done with the buffer
        for (int i = tid; i < HXB * HYB; i += TXB * TYB) {
            const int cy = i / HXB, cx = i - cy * HXB;
            const int l = it.z - 2 + cx, n = it.w - 2 + cy;
            if (l >= -3 && l <= g.lf + 4 && n >= -3 && n <= g.nf + 4) tile[i] = ld_cell(ub + 4 * cidx(g, l, n));
        }
        __syncthreads();
        const int l = it.z + threadIdx.x, n = it.w + threadIdx.y;
        if (l > g.lf || n > g.nf) continue;
        double F[4];
        if (it.y == 0)
            face_tile_b<0, np_of(ORD), NGP, HXB>(w, ORD / 2, tile, threadIdx.x + 2, threadIdx.y + 2, F, g.num_flux);
        else face_tile_b<1, np_of(ORD), NGP, HXB>(w, ORD / 2, tile, threadIdx.x + 2, threadIdx.y + 2, F, g.num_flux);
        st_cell((it.y == 0 ? a.fx : a.fy) + 4 * (P.off + (long long)cidx(g, l, n)), Cell{F[0], F[1], F[2], F[3]});
    }
}

#if !GPM_EXACT
// The two-direction cell tiles of every problem (xy_tile), persistent CTAs.
__global__ void __launch_bounds__(XT * XY, 2) kb_flux_xy(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char xy_raw[];
    XySmem& sm = *reinterpret_cast<XySmem*>(xy_raw);
    for (int item = blockIdx.x; item < a.nftiles; item += gridDim.x) {
        const int4 it = a.ftiles[item];
        const BProb P = a.prob[it.x];
        __syncthreads();  // the previous tile is done with the shared buffers
        xy_tile(bgeom(a, P), a.wtab[P.wc], a.uin + 4 * P.off, a.fx + 4 * P.off, a.fy + 4 * P.off, it.z, it.w, sm, false);
    }
}

// The edge items (problem, 3, k0, 0) of every problem.
__global__ void __launch_bounds__(EDGE_T) kb_flux_edge(BatchArgs a) {
    for (int item = blockIdx.x; item < a.netiles; item += gridDim.x) {
        const int4 it = a.etiles[item];
        const BProb P = a.prob[it.x];
        edge_faces(bgeom(a, P), a.wtab[P.wc], a.uin + 4 * P.off, a.fx + 4 * P.off, a.fy + 4 * P.off, it.z);
    }
}
#endif

static int sm_count() {
    static std::atomic<int> sms[GPM_MAX_DEVICES];
    const int dev = gpm_device();
    int n = sms[dev].load(std::memory_order_relaxed);
    if (!n) {
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
        sms[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

template <int TXB, int TYB, int NGP>
static void blaunch_flux_t(const BatchArgs& a, cudaStream_t s) {
    const int grid = a.nftiles < sm_count() * 4 ? a.nftiles : sm_count() * 4;
    const dim3 blk(TXB, TYB);
    if (a.mord == 5) kb_flux<TXB, TYB, NGP, 5><<<grid, blk, 0, s>>>(a);
    else if (a.mord == 3) kb_flux<TXB, TYB, NGP, 3><<<grid, blk, 0, s>>>(a);
    else kb_flux<TXB, TYB, NGP, 1><<<grid, blk, 0, s>>>(a);
}

template <int NGP>
static void blaunch_flux_n(const BatchArgs& a, cudaStream_t s) {
#if !GPM_EXACT
    if (a.tile == GPM_TILE_XY && NGP == 3 && a.mord == 5) {
        static std::atomic<bool> attr[GPM_MAX_DEVICES];
        const int dev = gpm_device();
        if (!attr[dev].load(std::memory_order_relaxed)) {
            cudaFuncSetAttribute(kb_flux_xy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(XySmem));
            attr[dev].store(true, std::memory_order_relaxed);
        }
        const int grid = a.nftiles < sm_count() * 2 ? a.nftiles : sm_count() * 2;
        kb_flux_xy<<<grid, dim3(XT, XY), sizeof(XySmem), s>>>(a);
        const int ge = a.netiles < sm_count() * 16 ? a.netiles : sm_count() * 16;
        if (ge > 0) kb_flux_edge<<<ge, EDGE_T, 0, s>>>(a);
        return;
    }
#endif
    switch (a.tile) {
    case 0: blaunch_flux_t<32, 8, NGP>(a, s); break;
    case 1: blaunch_flux_t<32, 4, NGP>(a, s); break;
    case 2: blaunch_flux_t<16, 16, NGP>(a, s); break;
    default: blaunch_flux_t<64, 4, NGP>(a, s); break;
    }
}

void blaunch_flux(const BatchArgs& a, cudaStream_t s) {
    switch (a.ngp) {
    case 1: blaunch_flux_n<1>(a, s); break;
    case 2: blaunch_flux_n<2>(a, s); break;
    case 3: blaunch_flux_n<3>(a, s); break;
    case 4: blaunch_flux_n<4>(a, s); break;
    default: blaunch_flux_n<5>(a, s); break;
    }
}

__device__ __forceinline__ void list_append2(bool flag, int2* __restrict__ list, int* __restrict__ count, int2 value) {
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

// First-pass update + DETECTION: persistent over blocks of 256 interior cells.
__global__ void __launch_bounds__(256) kb_update(BatchArgs a) {
    for (int item = blockIdx.x; item < a.ncblocks; item += gridDim.x) {
        const int2 it = a.cblocks[item];
        const BProb P = a.prob[it.x];
        const GridGeom g = bgeom(a, P);
        const int k = it.y + threadIdx.x;
        bool trb = false;
        int cl = 0;
        if (k < g.lf * g.nf) {
            const int l = 1 + k % g.lf, n = 1 + k / g.lf;
            const size_t c = cidx(g, l, n);
            const double* ub = a.uin + 4 * P.off;
            const Cell uo = cell_update(g, ub, a.fx + 4 * P.off, a.fy + 4 * P.off, c, a.sc[it.x].qx, a.sc[it.x].qy);
            st_cell(a.uout + 4 * (P.off + (long long)c), uo);
            if (a.method == 2 && g.mord > 1)
                trb = mood_troubled(uo, ub + 4 * c, g.nx, g, a.wtab[P.wc].d2x, a.wtab[P.wc].d2y);
            else if (a.method == 2 && inadmissible(uo))
                atomicOr(&a.ntrb[6], 1);
            cl = (int)c;
        }
        if (trb) cascade_order(a.order + P.off + cl);
        list_append2(trb, a.tlist[0], &a.ntrb[0], make_int2(it.x, cl));
    }
}

void blaunch_update(const BatchArgs& a, cudaStream_t s) {
    const int grid = a.ncblocks < sm_count() * 8 ? a.ncblocks : sm_count() * 8;
    kb_update<<<grid, 256, 0, s>>>(a);
}

// One MOOD pass over every problem's list: cascade, the troubled cells' faces,
// then their 5-point crosses.  Each kernel returns at once on an empty list,
// so a captured graph holds a fixed number of passes at almost no cost.
// Face i of the batch's face list at Gauss point gp (face_phase_gp item).
__device__ __forceinline__ void kb_face_gp(const BatchArgs& a, int cur, int nt, int i, int gp, FaceGp& f) {
    int dir, side;
    const int2 e = a.tlist[cur][face_item(i, nt, &dir, &side)];
    const BProb P = a.prob[e.x];
    StageArgs sa;
    sa.ccw = nullptr;
    sa.g = bgeom(a, P);
    sa.uin = a.uin + 4 * P.off;
    sa.fx = a.fx + 4 * P.off;
    sa.fy = a.fy + 4 * P.off;
    sa.order = a.order + P.off;
    const GpWeights& w = a.wtab[P.wc];
    const size_t c = (size_t)e.y;
    if (dir == 0) face_gp_any<0>(sa, w, side == 0 ? c - 1 : c, gp, f);
    else face_gp_any<1>(sa, w, side == 0 ? c - sa.g.nx : c, gp, f);
}

__global__ void kb_mood_mark(BatchArgs a, int cur) {  // the listed cells' orders are already lowered
    const int nt = a.ntrb[cur];
    if (nt == 0) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ntrb[cur ^ 1] = 0;
        a.ntrb[2] += 1;  // pass epoch for the de-duplication stamps
    }
}

template <int NGP>
__global__ void __launch_bounds__(128) kb_mood_faces(BatchArgs a, int cur) {
    const int nt = a.ntrb[cur];
    face_phase_gp<NGP>(4 * nt, 2 * nt, pack_tid(), gridDim.x * blockDim.x,
                       [&](int i, int gp, FaceGp& f) { kb_face_gp(a, cur, nt, i, gp, f); });
}

__global__ void __launch_bounds__(256) kb_mood_cells(BatchArgs a, int cur) {
    const int nt = a.ntrb[cur];
    if (nt == 0) return;
    const unsigned epoch = (unsigned)a.ntrb[2];
    const int nxt = cur ^ 1;
    const int total = 5 * nt;
    const int stride = gridDim.x * blockDim.x;
    const int lim = ((total + stride - 1) / stride) * stride;
    const int st = pack_tid();
    for (int base = 0; base < lim; base += stride) {
        const int i = base + st;
        bool trb = false;
        int2 val = make_int2(0, 0);
        if (i < total) {
            const int2 e = a.tlist[cur][i / 5];
            const BProb P = a.prob[e.x];
            const GridGeom g = bgeom(a, P);
            const size_t t = (size_t)e.y;
            const int k = i % 5;
            const size_t c = k == 0 ? t - g.nx : k == 1 ? t - 1 : k == 2 ? t : k == 3 ? t + 1 : t + g.nx;
            const int l = (int)(c % (size_t)g.nx) - 3, n = (int)(c / (size_t)g.nx) - 3;
            if (l >= 1 && l <= g.lf && n >= 1 && n <= g.nf &&
                atomicExch(&a.stamp[P.off + (long long)c], epoch) != epoch) {
                const double* ub = a.uin + 4 * P.off;
                const Cell uo = cell_update(g, ub, a.fx + 4 * P.off, a.fy + 4 * P.off, c, a.sc[e.x].qx, a.sc[e.x].qy);
                st_cell(a.uout + 4 * (P.off + (long long)c), uo);
                if (a.order[P.off + (long long)c] > 1)
                    trb = mood_troubled(uo, ub + 4 * c, g.nx, g, a.wtab[P.wc].d2x, a.wtab[P.wc].d2y);
                else if (inadmissible(uo))
                    atomicOr(&a.ntrb[6], 1);
                val = make_int2(e.x, (int)c);
            }
        }
        if (trb) cascade_order(a.order + a.prob[val.x].off + val.y);
        list_append2(trb, a.tlist[nxt], &a.ntrb[nxt], val);
    }
}

void blaunch_mood_pass(const BatchArgs& a, int cur, cudaStream_t s) {
    const int g = sm_count() * 4;
    kb_mood_mark<<<g, 256, 0, s>>>(a, cur);
    switch (a.ngp) {
    case 1: kb_mood_faces<1><<<g, 128, 0, s>>>(a, cur); break;
    case 2: kb_mood_faces<2><<<g, 128, 0, s>>>(a, cur); break;
    case 3: kb_mood_faces<3><<<g, 128, 0, s>>>(a, cur); break;
    case 4: kb_mood_faces<4><<<g, 128, 0, s>>>(a, cur); break;
    default: kb_mood_faces<5><<<g, 128, 0, s>>>(a, cur); break;
    }
    kb_mood_cells<<<g, 256, 0, s>>>(a, cur);
}

// The batch's whole MOOD loop in one cooperative launch (see k_mood_loop):
// passes run until every problem's list is empty.  ntrb[2] is the stamp epoch,
// ntrb[4] the detected-cell total, ntrb[5] the pass count of the last stage.
template <int NGP>
__global__ void __launch_bounds__(MOOD_THREADS, 1) kb_mood_loop(BatchArgs a, GridBar* bar, int max_pass) {
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
    int stid = pack_tid(), wstride = gstride;
    bool solo = false;
    int cur = 0, pass = 1;
    for (;;) {
        const int nt = *(volatile int*)&a.ntrb[cur];
        if (nt == 0) break;
        if (pass >= max_pass) {
            if (gtid == 0) a.ntrb[3] = 1;
            break;
        }
        if (!solo && nt <= a.mood_solo) {  // as in k_mood_loop
            if (blockIdx.x != 0) return;
            solo = true;
            stid = threadIdx.x;
            wstride = blockDim.x;
        }
        pass++;
        // the listed cells' orders were lowered when they were listed
        if (gtid == 0) {
            a.ntrb[cur ^ 1] = 0;  // nobody appends to it before the next barrier
            a.ntrb[2] += 1;       // stamp epoch, read after the next barrier
            a.ntrb[4] += nt;
        }
        face_phase_gp<NGP>(4 * nt, 2 * nt, stid, wstride,
                           [&](int i, int gp, FaceGp& f) { kb_face_gp(a, cur, nt, i, gp, f); });
        if (!mood_sync(bar, solo)) return;
        const unsigned epoch = (unsigned)*(volatile int*)&a.ntrb[2];
        const int nxt = cur ^ 1, total = 5 * nt;
        const int lim = ((total + wstride - 1) / wstride) * wstride;
        for (int base = 0; base < lim; base += wstride) {
            const int i = base + stid;
            bool trb = false;
            int2 val = make_int2(0, 0);
            if (i < total) {
                const int2 e = a.tlist[cur][i / 5];
                const BProb P = a.prob[e.x];
                const GridGeom g = bgeom(a, P);
                const size_t t = (size_t)e.y;
                const int k = i % 5;
                const size_t c = k == 0 ? t - g.nx : k == 1 ? t - 1 : k == 2 ? t : k == 3 ? t + 1 : t + g.nx;
                const int l = (int)(c % (size_t)g.nx) - 3, n = (int)(c / (size_t)g.nx) - 3;
                if (l >= 1 && l <= g.lf && n >= 1 && n <= g.nf &&
                    atomicExch(&a.stamp[P.off + (long long)c], epoch) != epoch) {
                    const double* ub = a.uin + 4 * P.off;
                    const Cell uo =
                        cell_update(g, ub, a.fx + 4 * P.off, a.fy + 4 * P.off, c, a.sc[e.x].qx, a.sc[e.x].qy);
                    st_cell(a.uout + 4 * (P.off + (long long)c), uo);
                    if (a.order[P.off + (long long)c] > 1)
                        trb = mood_troubled(uo, ub + 4 * c, g.nx, g, a.wtab[P.wc].d2x, a.wtab[P.wc].d2y);
                    else if (inadmissible(uo))
                        atomicOr(&a.ntrb[6], 1);
                    val = make_int2(e.x, (int)c);
                }
            }
            if (trb) cascade_order(a.order + a.prob[val.x].off + val.y);
            list_append2(trb, a.tlist[nxt], &a.ntrb[nxt], val);
        }
        if (!mood_sync(bar, solo)) return;
        cur ^= 1;
    }
    if (gtid == 0) a.ntrb[5] = pass;
}

template <int NGP>
static int blaunch_mood_loop_n(const BatchArgs& a, GridBar* bar, int max_pass, cudaStream_t s) {
    static std::atomic<int> grids[GPM_MAX_DEVICES];
    const int dev = gpm_device();
    int grid = grids[dev].load(std::memory_order_relaxed);
    if (!grid) {
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kb_mood_loop<NGP>, MOOD_THREADS, 0);
        grid = sm_count() * (occ > 0 ? occ : 1);
        grids[dev].store(grid, std::memory_order_relaxed);
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(MOOD_THREADS);
    cfg.stream = s;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeCooperative;
    attr.val.cooperative = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kb_mood_loop<NGP>, a, bar, max_pass) == cudaSuccess ? 0 : -1;
}

int blaunch_mood_loop(const BatchArgs& a, GridBar* bar, int max_pass, cudaStream_t s) {
    switch (a.ngp) {
    case 1: return blaunch_mood_loop_n<1>(a, bar, max_pass, s);
    case 2: return blaunch_mood_loop_n<2>(a, bar, max_pass, s);
    case 3: return blaunch_mood_loop_n<3>(a, bar, max_pass, s);
    case 4: return blaunch_mood_loop_n<4>(a, bar, max_pass, s);
    default: return blaunch_mood_loop_n<5>(a, bar, max_pass, s);
    }
}

// After the last captured pass: a non-empty list means the stage hit the cap.
__global__ void kb_leftover(BatchArgs a, int cur) {
    if (a.ntrb[cur] != 0) a.ntrb[3] = 1;
}
void blaunch_leftover(const BatchArgs& a, int cur, cudaStream_t s) { kb_leftover<<<1, 1, 0, s>>>(a, cur); }

// Per-problem CFL minimum: every block of padded cells belongs to one problem.
__device__ __forceinline__ void bdt_reduce(double v, BScal* sc) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ double wmin[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) wmin[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < (int)(blockDim.x >> 5) ? wmin[lane] : 1.0e30;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0 && v > 0.0 && v < 1.0e30) atomicMin(&sc->dtmin_bits, (unsigned long long)__double_as_longlong(v));
    }
}

__global__ void __launch_bounds__(256) kb_combine(BatchArgs a, const double* __restrict__ x, double* __restrict__ y,
                                                  double ca, double cb, int with_cfl, int only_cfl) {
    for (int item = blockIdx.x; item < a.npblocks; item += gridDim.x) {
        const int2 it = a.pblocks[item];
        const BProb P = a.prob[it.x];
        const int k = it.y + threadIdx.x;
        double v = 1.0e30;
        if (k < P.nx * P.ny) {
            const long long c = P.off + k;
            if (only_cfl) {
                v = cell_dt(ld_cell(x + 4 * c), P.dx, P.dy);
            } else {
                const Cell p = ld_cell(x + 4 * c);
                const Cell q = ld_cell_cg(y + 4 * c);
                Cell o;
                o.r = ca * p.r + cb * q.r;
                o.mx = ca * p.mx + cb * q.mx;
                o.my = ca * p.my + cb * q.my;
                o.e = ca * p.e + cb * q.e;
                st_cell(y + 4 * c, o);
                if (with_cfl) v = cell_dt(o, P.dx, P.dy);
            }
        }
        if (with_cfl || only_cfl) bdt_reduce(v, &a.sc[it.x]);
    }
}

void blaunch_combine(const BatchArgs& a, const double* x, double* y, double ca, double cb, int with_cfl, cudaStream_t s) {
    const int grid = a.npblocks < sm_count() * 8 ? a.npblocks : sm_count() * 8;
    kb_combine<<<grid, 256, 0, s>>>(a, x, y, ca, cb, with_cfl, 0);
}

void blaunch_cfl(const BatchArgs& a, const double* u, cudaStream_t s) {
    const int grid = a.npblocks < sm_count() * 8 ? a.npblocks : sm_count() * 8;
    kb_combine<<<grid, 256, 0, s>>>(a, u, nullptr, 0.0, 0.0, 1, 1);
}

__global__ void kb_dt_finalize(BatchArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nprob) return;
    BScal& sc = a.sc[i];
    double dt = __longlong_as_double((long long)sc.dtmin_bits);
    dt = dt * sc.cfl;
    const double dtfinal = sc.tmax - sc.t;
    if (dt > dtfinal) dt = dtfinal;
    sc.dt = dt;
    sc.qx = dt / a.prob[i].dx;
    sc.qy = dt / a.prob[i].dy;
    sc.dtmin_bits = (unsigned long long)__double_as_longlong(1.0e30);
    if (!(dt > 0.0) || is_nan(dt)) sc.status |= GPM_STATUS_DT;
}

__global__ void kb_advance_t(BatchArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.nprob) a.sc[i].t = a.sc[i].t + a.sc[i].dt;
}

void blaunch_dt_finalize(const BatchArgs& a, cudaStream_t s) { kb_dt_finalize<<<(a.nprob + 127) / 128, 128, 0, s>>>(a); }
void blaunch_advance_t(const BatchArgs& a, cudaStream_t s) { kb_advance_t<<<(a.nprob + 127) / 128, 128, 0, s>>>(a); }

void batch_set_max_nx(int nx) { g_max_nx = nx; }

const BatchTable batch_table = {blaunch_bc,      blaunch_flux,        blaunch_update,    blaunch_mood_pass,
                                blaunch_leftover, blaunch_combine,     blaunch_cfl,       blaunch_dt_finalize,
                                blaunch_advance_t, blaunch_mood_loop};

}  // namespace GPM_NS
