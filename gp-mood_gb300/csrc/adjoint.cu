// adjoint.cu -- hand-written adjoint (vector-Jacobian product) of one GP-MOOD
// RK stage with its MOOD order mask frozen.
//
// With the orders fixed, a stage is the smooth-almost-everywhere map
//   Uout = Uin + qy*Fy(c-y) + qx*Fx(c-x) - qx*Fx(c) - qy*Fy(c)   (interior c)
//   F    = sum_g w_g HLLC(uL_g, uR_g),  uL_g/uR_g = GP dot products of BC(Uin)
// (mod_FE.f90:75-145, mod_GP_MOOD.f90:58-65, mod_HLLC.f90:11-169).  Its VJP:
//   mu_F        = q * (lam(high cell) - lam(low cell))            per face
//   mu_uL_g     = w_g * J_L(g)^T mu_F,  mu_uR_g = w_g * J_R(g)^T mu_F
//   mu_U(c)    += z_m * mu_u  over every face state whose stencil holds c
//   lam_in      = lam_out + BC^T(mu_U)
// The 4x8 HLLC Jacobians come from forward-mode dual numbers carried through
// the same HLLC expressions (the branch is picked on the values, as in HLLC).
#define GPM_EXACT 1
#include "physics.cuh"
#include "adjoint.h"

namespace {

struct D8 {  // value and derivatives with respect to the 8 inputs (uL, uR)
    double v, d[8];
};
__device__ __forceinline__ D8 dconst(double v) {
    D8 r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < 8; i++) r.d[i] = 0.0;
    return r;
}
__device__ __forceinline__ D8 operator+(const D8& a, const D8& b) {
    D8 r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < 8; i++) r.d[i] = a.d[i] + b.d[i];
    return r;
}
__device__ __forceinline__ D8 operator-(const D8& a, const D8& b) {
    D8 r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < 8; i++) r.d[i] = a.d[i] - b.d[i];
    return r;
}
__device__ __forceinline__ D8 operator*(const D8& a, const D8& b) {
    D8 r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < 8; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
__device__ __forceinline__ D8 operator*(double s, const D8& a) {
    D8 r;
    r.v = s * a.v;
#pragma unroll
    for (int i = 0; i < 8; i++) r.d[i] = s * a.d[i];
    return r;
}
__device__ __forceinline__ D8 operator/(const D8& a, const D8& b) {
    D8 r;
    r.v = a.v / b.v;
    const double ib = 1.0 / b.v;
#pragma unroll
    for (int i = 0; i < 8; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    return r;
}
__device__ __forceinline__ D8 dsqrt(const D8& a) {
    D8 r;
    r.v = sqrt(a.v);
    const double h = 0.5 / r.v;
#pragma unroll
    for (int i = 0; i < 8; i++) r.d[i] = a.d[i] * h;
    return r;
}
__device__ __forceinline__ const D8& dmin(const D8& a, const D8& b) { return (b.v < a.v) ? b : a; }
__device__ __forceinline__ const D8& dmax(const D8& a, const D8& b) { return (b.v > a.v) ? b : a; }

struct DPrim {
    D8 vn, vt, vn2, p, c;
};

template <int DIR>
__device__ __forceinline__ DPrim dc2p(const D8* u) {
    DPrim s;
    const D8 vx = u[1] / u[0], vy = u[2] / u[0];
    s.p = (GPM_GAMMA - 1.) * (u[3] - (0.5 * (u[1] * u[1] + u[2] * u[2]) / u[0]));
    s.c = dsqrt(GPM_GAMMA * s.p / u[0]);
    s.vn = DIR == 0 ? vx : vy;
    s.vt = DIR == 0 ? vy : vx;
    s.vn2 = s.vn * s.vn;
    return s;
}

template <int DIR>
__device__ __forceinline__ void dflux(const D8* u, const DPrim& s, D8* r) {
    if (DIR == 0) {
        r[0] = u[1];
        r[1] = u[0] * s.vn2 + s.p;
        r[2] = u[2] * s.vn;
        r[3] = s.vn * (u[3] + s.p);
    } else {
        r[0] = u[2];
        r[1] = u[1] * s.vn;
        r[2] = u[0] * s.vn2 + s.p;
        r[3] = s.vn * (u[3] + s.p);
    }
}

// HLLC with derivatives, same branch structure as hllc<DIR> (admissible states).
template <int DIR>
__device__ void dhllc(const double* ul, const double* ur, double J[4][8]) {
    D8 L[4], R[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        L[k] = dconst(ul[k]);
        R[k] = dconst(ur[k]);
        L[k].d[k] = 1.0;
        R[k].d[4 + k] = 1.0;
    }
    const DPrim pl = dc2p<DIR>(L), pr = dc2p<DIR>(R);
    const D8 SL = dmin(pl.vn - pl.c, pr.vn - pr.c);
    const D8 SR = dmax(pl.vn + pl.c, pr.vn + pr.c);
    D8 F[4];
    if (SL.v >= 0.) {
        dflux<DIR>(L, pl, F);
    } else {
        const D8 numerL = SL - pl.vn, numerR = SR - pr.vn;
        D8 uStar = L[0] * pl.vn * numerL - R[0] * pr.vn * numerR;
        uStar = (pr.p - pl.p) + uStar;
        const D8 aL = L[0] * numerL, aR = R[0] * numerR;
        uStar = uStar / (aL - aR);
        const bool left = (SL.v < 0.) && (uStar.v >= 0.);
        const bool right = (uStar.v < 0.) && (SR.v >= 0.);
        if (!left && !right) {
            dflux<DIR>(R, pr, F);
        } else {
            const D8* u = left ? L : R;
            const DPrim& s = left ? pl : pr;
            const D8& S = left ? SL : SR;
            const D8& a = left ? aL : aR;
            D8 Fk[4];
            dflux<DIR>(u, s, Fk);
            const D8 dStar = a / (S - uStar);
            D8 st[4];
            st[0] = dconst(1.0);
            st[DIR == 0 ? 1 : 2] = uStar;
            st[DIR == 0 ? 2 : 1] = s.vt;
            st[3] = u[3] / u[0] + (uStar - s.vn) * (uStar + s.p / a);
#pragma unroll
            for (int k = 0; k < 4; k++) F[k] = Fk[k] + S * (st[k] * dStar - u[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int i = 0; i < 8; i++) J[k][i] = F[k].d[i];
}

__device__ __forceinline__ size_t aidx(int nx, int l, int n) { return (size_t)(n + 3) * nx + (size_t)(l + 3); }

// Per face: states at the frozen order, HLLC Jacobians, and the adjoints of
// the face states mu_uL[g][4], mu_uR[g][4] (stored per face).
template <int DIR, int NGP>
__global__ void __launch_bounds__(128) k_adj_faces(AdjArgs a, const __grid_constant__ GpWeights w) {
    const GridGeom& g = a.g;
    const int nl = DIR == 0 ? g.lf + 1 : g.lf, nn = DIR == 0 ? g.nf : g.nf + 1;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nl * nn) return;
    const int l = (DIR == 0 ? 0 : 1) + (int)(idx % nl), n = (DIR == 0 ? 1 : 0) + (int)(idx / nl);
    const size_t c0 = aidx(g.nx, l, n), c1 = DIR == 0 ? c0 + 1 : c0 + g.nx;
    const int o = min((int)a.order[c0], (int)a.order[c1]);
    const int oi = o >= 5 ? 2 : (o >= 3 ? 1 : 0), np = o >= 5 ? 13 : (o >= 3 ? 5 : 1);
    constexpr int FL = DIR == 0 ? 2 : 1, FH = DIR == 0 ? 0 : 3;
    double muF[4];
    const double q = DIR == 0 ? a.qx : a.qy;
    const bool lin = (l >= 1 && l <= g.lf && n >= 1 && n <= g.nf);
    const int lh = DIR == 0 ? l + 1 : l, nh = DIR == 0 ? n : n + 1;
    const bool hin = (lh >= 1 && lh <= g.lf && nh >= 1 && nh <= g.nf);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double lo = lin ? a.lam_out[4 * c0 + k] : 0.0, hi = hin ? a.lam_out[4 * c1 + k] : 0.0;
        muF[k] = q * (hi - lo);
    }
    double* out = a.face_adj + (DIR == 0 ? 0 : (size_t)g.nx * g.ny * 8 * GPM_MAXGP) + c0 * 8 * GPM_MAXGP;
#pragma unroll
    for (int gp = 0; gp < NGP; gp++) {
        double uL[4] = {0, 0, 0, 0}, uR[4] = {0, 0, 0, 0};
        for (int m = 0; m < np; m++) {
            const double zl = w.zt[oi][FL][gp][m], zh = w.zt[oi][FH][gp][m];
            const size_t sl = c0 + st_ox(m) + (ptrdiff_t)g.nx * st_oy(m);
            const size_t sh = c1 + st_ox(m) + (ptrdiff_t)g.nx * st_oy(m);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                uL[k] += zl * a.u_in[4 * sl + k];
                uR[k] += zh * a.u_in[4 * sh + k];
            }
        }
        double J[4][8];
        dhllc<DIR>(uL, uR, J);
        const double wg = w.gw[gp];
#pragma unroll
        for (int i = 0; i < 8; i++) {
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < 4; k++) s += J[k][i] * muF[k];
            out[gp * 8 + i] = wg * s;
        }
    }
}

// mu_U(c) for every padded cell within reach of a face: gather over the face
// states whose stencils hold c.
template <int NGP>
__global__ void __launch_bounds__(128) k_adj_gather(AdjArgs a, const __grid_constant__ GpWeights w) {
    const GridGeom& g = a.g;
    const long long ncell = (long long)g.nx * g.ny;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const int l = (int)(c % g.nx) - 3, n = (int)(c / g.nx) - 3;
    double mu[4] = {0, 0, 0, 0};
    for (int m = 0; m < 13; m++) {
        for (int dir = 0; dir < 2; dir++) {
            // as the low cell's stencil point m: face with low cell (l - ox, n - oy)
            // as the high cell's stencil point m: face with high cell (l - ox, n - oy)
            for (int side = 0; side < 2; side++) {
                const int cl = l - st_ox(m) - (side == 1 && dir == 0 ? 1 : 0);
                const int cn = n - st_oy(m) - (side == 1 && dir == 1 ? 1 : 0);
                const bool ok = dir == 0 ? (cl >= 0 && cl <= g.lf && cn >= 1 && cn <= g.nf)
                                         : (cl >= 1 && cl <= g.lf && cn >= 0 && cn <= g.nf);
                if (!ok) continue;
                const size_t f0 = aidx(g.nx, cl, cn), f1 = dir == 0 ? f0 + 1 : f0 + g.nx;
                const int o = min((int)a.order[f0], (int)a.order[f1]);
                const int np = o >= 5 ? 13 : (o >= 3 ? 5 : 1);
                if (m >= np) continue;
                const int oi = o >= 5 ? 2 : (o >= 3 ? 1 : 0);
                const int face = dir == 0 ? (side == 0 ? 2 : 0) : (side == 0 ? 1 : 3);
                const double* fa = a.face_adj + (dir == 0 ? 0 : (size_t)g.nx * g.ny * 8 * GPM_MAXGP) + f0 * 8 * GPM_MAXGP;
#pragma unroll
                for (int gp = 0; gp < NGP; gp++) {
                    const double z = w.zt[oi][face][gp][m];
#pragma unroll
                    for (int k = 0; k < 4; k++) mu[k] += z * fa[gp * 8 + side * 4 + k];
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) a.mu_pad[4 * c + k] = mu[k];
}

// Transpose of Boundary_C (BC.f90:10-421 as k_bc_x then k_bc_y): first the
// ghost rows are folded into the interior rows they copy (every column), then
// the ghost columns into the interior columns.  Reflective ghosts carry the
// sign flip of the normal momentum.
__device__ __forceinline__ int ghost_source(int bc, int i, int nint, int* sign) {
    // source index of ghost i (i <= 0 or i > nint) along one axis; sign -1 on a mirror
    *sign = 1;
    if (bc == 17) return i <= 0 ? 1 : nint;
    if (bc == 18) return i <= 0 ? i + nint : i - nint;
    *sign = -1;  // 20
    return i <= 0 ? 1 - i : 2 * nint + 1 - i;
}

__global__ void k_adj_fold_y(GridGeom g, double* __restrict__ mu) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.nx * g.nf) return;
    const int l = (int)(idx % g.nx) - 3, n = 1 + (int)(idx / g.nx);
    double s[4];
    const size_t c = aidx(g.nx, l, n);
#pragma unroll
    for (int k = 0; k < 4; k++) s[k] = mu[4 * c + k];
    for (int j = 0; j < GPM_NGC; j++) {
        for (int top = 0; top < 2; top++) {
            const int ng = top ? g.nf + 1 + j : -j;
            int sg;
            if (ghost_source(g.bc_type, ng, g.nf, &sg) != n) continue;
            const size_t cg = aidx(g.nx, l, ng);
            s[0] += mu[4 * cg + 0];
            s[1] += mu[4 * cg + 1];
            s[2] += sg * mu[4 * cg + 2];
            s[3] += mu[4 * cg + 3];
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) mu[4 * c + k] = s[k];
}

__global__ void k_adj_fold_x(GridGeom g, const double* __restrict__ mu, const double* base, double* out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.lf * g.nf) return;
    const int l = 1 + (int)(idx % g.lf), n = 1 + (int)(idx / g.lf);
    const size_t c = aidx(g.nx, l, n);
    double s[4];
#pragma unroll
    for (int k = 0; k < 4; k++) s[k] = base[4 * c + k] + mu[4 * c + k];
    for (int j = 0; j < GPM_NGC; j++) {
        for (int right = 0; right < 2; right++) {
            const int lg = right ? g.lf + 1 + j : -j;
            int sg;
            if (ghost_source(g.bc_type, lg, g.lf, &sg) != l) continue;
            const size_t cg = aidx(g.nx, lg, n);
            s[0] += mu[4 * cg + 0];
            s[1] += sg * mu[4 * cg + 1];
            s[2] += mu[4 * cg + 2];
            s[3] += mu[4 * cg + 3];
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) out[4 * c + k] = s[k];
}

void launch_fold(const GridGeom& g, double* mu, const double* base, double* out, cudaStream_t s) {
    const long long ny = (long long)g.nx * g.nf, nx = (long long)g.lf * g.nf;
    k_adj_fold_y<<<(int)((ny + 255) / 256), 256, 0, s>>>(g, mu);
    k_adj_fold_x<<<(int)((nx + 255) / 256), 256, 0, s>>>(g, mu, base, out);
}

template <int NGP>
void launch_adj_n(const AdjArgs& a, const GpWeights& w, cudaStream_t s) {
    const long long nfx = (long long)(a.g.lf + 1) * a.g.nf, nfy = (long long)a.g.lf * (a.g.nf + 1);
    k_adj_faces<0, NGP><<<(int)((nfx + 127) / 128), 128, 0, s>>>(a, w);
    k_adj_faces<1, NGP><<<(int)((nfy + 127) / 128), 128, 0, s>>>(a, w);
    const long long nc = (long long)a.g.nx * a.g.ny;
    k_adj_gather<NGP><<<(int)((nc + 127) / 128), 128, 0, s>>>(a, w);
    launch_fold(a.g, a.mu_pad, a.lam_out, a.lam_in, s);
}

}  // namespace

int gpm_adj_stage(const AdjArgs& a, const GpWeights& w, cudaStream_t s) {
    switch (a.g.ngp) {
    case 1: launch_adj_n<1>(a, w, s); break;
    case 2: launch_adj_n<2>(a, w, s); break;
    case 3: launch_adj_n<3>(a, w, s); break;
    case 4: launch_adj_n<4>(a, w, s); break;
    default: launch_adj_n<5>(a, w, s); break;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int gpm_adj_fold(const GridGeom& g, double* mu, const double* base, double* out, cudaStream_t s) {
    launch_fold(g, mu, base, out, s);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
