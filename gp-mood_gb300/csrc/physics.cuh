// physics.cuh -- device physics of the GP-MOOD step: pressure, HLLC, GP dot
// products, MOOD detection.  Included by stage_kernels.cu, which is compiled
// twice: GPM_EXACT=1 with --fmad=false (every expression rounds exactly like
// the reference's x86-64 build) and GPM_EXACT=0 with FMA contraction,
// reciprocal reuse, Newton reciprocals and square roots from the hardware
// approximations (fast_rcp.cuh), division-free DETECTION tests and, in the
// first pass, an HLLC with selects instead of branches.
//
// Reference routines: physics.f90:9-75,132-143 (Flux, c2p_local, pressure),
// mod_HLLC.f90:11-169 (HLLC_Flux), mod_GP_MOOD.f90:58-65 (dot products),
// mod_subroutine_MOOD.f90:41-131,191-238 (DETECTION checks, shock_detector).
#pragma once
#include "fast_rcp.cuh"
#include "gpm_common.h"

#ifndef GPM_EXACT
#error "GPM_EXACT must be defined"
#endif

#define GPM_GAMMA 1.4

struct __align__(32) Cell {
    double r, mx, my, e;
};

__device__ __forceinline__ Cell ld_cell(const double* p) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    return Cell{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ Cell ld_cell_cg(const double* p) {  // data written earlier in the same kernel chain
    const double2 a = __ldcg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldcg(reinterpret_cast<const double2*>(p) + 1);
    return Cell{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void st_cell(double* p, const Cell& c) {
    reinterpret_cast<double2*>(p)[0] = make_double2(c.r, c.mx);
    reinterpret_cast<double2*>(p)[1] = make_double2(c.my, c.e);
}

// x + 0.0 without an FP64 instruction.  A dot product written as
// 0 + p1 + p2 + ... (Fortran dot_product) differs from p1 + p2 + ... only by
// the sign of an exact zero result, so applying this at the end restores it.
__device__ __forceinline__ double plus_zero(double x) {
    return (__double_as_longlong(x) == (long long)0x8000000000000000ULL) ? 0.0 : x;
}

// Sign/NaN tests on the bit pattern (integer pipe, exact).
__device__ __forceinline__ bool is_nan(double x) {
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}
// (x <= 0) .or. ISNAN(x): a non-positive double has a non-positive signed bit
// pattern; a NaN with the sign bit set also does, and is caught either way.
__device__ __forceinline__ bool le_zero_or_nan(double x) {
    return (__double_as_longlong(x) <= 0LL) || is_nan(x);
}

// pressure(u), physics.f90:132-143: (y-1)*(E - 0.5*(mx^2+my^2)/rho)
__device__ __forceinline__ double pressure(const Cell& u) {
    return (GPM_GAMMA - 1.) * (u.e - (0.5 * (u.mx * u.mx + u.my * u.my) / u.r));
}

// Stencil offsets of the diamond stencil, GP_init.f90:97-138 ordering.
__host__ __device__ constexpr int st_ox(int m) {
    return m == 0 ? 0 : m == 1 ? -1 : m == 2 ? 0 : m == 3 ? 1 : m == 4 ? 0 : m == 5 ? -1 : m == 6 ? -1
         : m == 7 ? 1 : m == 8 ? 1 : m == 9 ? 0 : m == 10 ? -2 : m == 11 ? 0 : 2;
}
__host__ __device__ constexpr int st_oy(int m) {
    return m == 0 ? 0 : m == 1 ? 0 : m == 2 ? 1 : m == 3 ? 0 : m == 4 ? -1 : m == 5 ? -1 : m == 6 ? 1
         : m == 7 ? 1 : m == 8 ? -1 : m == 9 ? -2 : m == 10 ? 0 : m == 11 ? 2 : 0;
}
__host__ __device__ constexpr int np_of(int ord) { return ord == 1 ? 1 : (ord == 3 ? 5 : 13); }

// GP reconstruction of one face of one cell at one Gauss point (weights z):
// u[k] = sum_m z[m] * q[m][k], sequential in m (mod_GP_MOOD.f90:61).
template <int NP>
__device__ __forceinline__ void gp_recon_at(const double* __restrict__ z, const Cell* q, double* u) {
    double s0 = z[0] * q[0].r, s1 = z[0] * q[0].mx, s2 = z[0] * q[0].my, s3 = z[0] * q[0].e;
#pragma unroll
    for (int m = 1; m < NP; m++) {
        const double zm = z[m];
        s0 = s0 + zm * q[m].r;
        s1 = s1 + zm * q[m].mx;
        s2 = s2 + zm * q[m].my;
        s3 = s3 + zm * q[m].e;
    }
#if GPM_EXACT
    u[0] = plus_zero(s0); u[1] = plus_zero(s1); u[2] = plus_zero(s2); u[3] = plus_zero(s3);
#else
    u[0] = s0; u[1] = s1; u[2] = s2; u[3] = s3;
#endif
}

// ... and at all NGP Gauss points of the face (zface: NGP rows of 13).
template <int NP, int NGP>
__device__ __forceinline__ void gp_recon(const double* __restrict__ zface, const Cell* q, double (*u)[4]) {
#pragma unroll
    for (int g = 0; g < NGP; g++) gp_recon_at<NP>(zface + g * 13, q, u[g]);
}

#if !GPM_EXACT
__device__ __forceinline__ double cell_var(const Cell& c, int k) {
    return k == 0 ? c.r : (k == 1 ? c.mx : (k == 2 ? c.my : c.e));
}

// The three Gauss-point states of one face from the mirror-symmetric split
// (GpSym): same values as gp_recon<NP, 3> up to rounding, 32 instead of 39
// FP64 operations per variable at NP = 13.
template <int DIR, int NP>
__device__ __forceinline__ void gp_recon_sym3(const GpSym& c, const Cell* q, double (*u)[4]) {
    constexpr int NA = NP == 13 ? 5 : 3, NPR = NP == 13 ? 4 : 1;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        double a0 = c.a0[0] * cell_var(q[gpm_sym_axis(DIR, 0)], k);
        double a1 = c.a1[0] * cell_var(q[gpm_sym_axis(DIR, 0)], k);
#pragma unroll
        for (int i = 1; i < NA; i++) {
            const double v = cell_var(q[gpm_sym_axis(DIR, i)], k);
            a0 = a0 + c.a0[i] * v;
            a1 = a1 + c.a1[i] * v;
        }
        double b = 0.0;
#pragma unroll
        for (int i = 0; i < NPR; i++) {
            const double qm = cell_var(q[gpm_sym_pair(DIR, i, 0)], k), qmm = cell_var(q[gpm_sym_pair(DIR, i, 1)], k);
            const double S = qm + qmm, D = qm - qmm;
            a0 = a0 + c.al[i] * S;
            a1 = a1 + c.ga[i] * S;
            b = (i == 0) ? c.be[0] * D : b + c.be[i] * D;
        }
        u[0][k] = a0 + b;
        u[1][k] = a1;
        u[2][k] = a0 - b;
    }
}
#endif

// Primitive recovery of one face state, c2p_local (physics.f90:51-75): normal
// velocity vn, tangential velocity vt, pressure, sound speed, admissibility
// (vn^2 is formed by the one physical flux that needs it).
struct Prim {
    double vn, vt, p, c;
    bool adm;
    double vx;  // x-velocity, needed for the 1/(vx-vx) of an inadmissible state
#if !GPM_EXACT
    double ir;  // 1/rho
#endif
};

template <int DIR>
__device__ __forceinline__ Prim c2p(const double* u, double ir_in = 0.0) {
    Prim s;
#if GPM_EXACT
    const double vx = u[1] / u[0];
    const double vy = u[2] / u[0];
    s.p = (GPM_GAMMA - 1.) * (u[3] - (0.5 * (u[1] * u[1] + u[2] * u[2]) / u[0]));
    s.c = sqrt(GPM_GAMMA * s.p / u[0]);
#else
    const double ir = ir_in;  // 1/rho, supplied by the caller
    const double vx = u[1] * ir;
    const double vy = u[2] * ir;
    s.p = (GPM_GAMMA - 1.) * (u[3] - 0.5 * (u[1] * vx + u[2] * vy));
    s.c = gpm_fast_sqrt(GPM_GAMMA * s.p * ir);  // NaN for p <= 0, which is inadmissible
    s.ir = ir;
#endif
    s.vx = vx;
    s.vn = DIR == 0 ? vx : vy;
    s.vt = DIR == 0 ? vy : vx;
    s.adm = !(le_zero_or_nan(u[0]) || le_zero_or_nan(s.p));
    return s;
}

// Physical flux F(u) in direction DIR, physics.f90:9-48 (admissible branch).
template <int DIR>
__device__ __forceinline__ void phys_flux(const double* u, const Prim& s, double* r) {
    if (DIR == 0) {
        r[0] = u[1];
        r[1] = u[0] * (s.vn * s.vn) + s.p;
        r[2] = u[2] * s.vn;
        r[3] = s.vn * (u[3] + s.p);
    } else {
        r[0] = u[2];
        r[1] = u[1] * s.vn;
        r[2] = u[0] * (s.vn * s.vn) + s.p;
        r[3] = s.vn * (u[3] + s.p);
    }
}

// HLLC_Flux, mod_HLLC.f90:11-169, with the symmetry-preserving u* (:121-123).
// Only the branch that the reference finally selects is evaluated; every
// skipped quantity is unused by that branch, so the result is unchanged.
template <int DIR>
__device__ __forceinline__ void hllc(const double* ul, const double* ur, double* F) {
#if GPM_EXACT
    const Prim L = c2p<DIR>(ul);
    const Prim R = c2p<DIR>(ur);
#else
    const double rr = gpm_fast_rcp(ul[0] * ur[0]);  // one reciprocal for both 1/rho
    const Prim L = c2p<DIR>(ul, ur[0] * rr);
    const Prim R = c2p<DIR>(ur, ul[0] * rr);
#endif
    const double SL = fmin(L.vn - L.c, R.vn - R.c);
    const double SR = fmax(L.vn + L.c, R.vn + R.c);
    if (!(L.adm && R.adm)) {  // :166
        const double bad = 1. / (R.vx - R.vx);
        F[0] = F[1] = F[2] = F[3] = bad;
        return;
    }
    if (SL >= 0.) {
        phys_flux<DIR>(ul, L, F);
        return;
    }
    const double numerL = SL - L.vn, numerR = SR - R.vn;
    double uStar = ul[0] * L.vn * numerL - ur[0] * R.vn * numerR;
    uStar = (R.p - L.p) + uStar;
    const double aL = ul[0] * numerL, aR = ur[0] * numerR;
#if GPM_EXACT
    uStar = uStar / (aL - aR);
#else
    uStar = uStar * gpm_fast_rcp(aL - aR);
#endif
    const bool left = (SL < 0.) && (uStar >= 0.);
    const bool right = (uStar < 0.) && (SR >= 0.);
    if (!left && !right) {
        phys_flux<DIR>(ur, R, F);
        return;
    }
    const double* u = left ? ul : ur;
    const Prim& s = left ? L : R;
    const double S = left ? SL : SR;
    const double a = left ? aL : aR;
    double Fk[4];
    phys_flux<DIR>(u, s, Fk);
    double st[4];
    st[0] = 1.;
    st[DIR == 0 ? 1 : 2] = uStar;
    st[DIR == 0 ? 2 : 1] = s.vt;
#if GPM_EXACT
    const double dStar = a / (S - uStar);
    st[3] = u[3] / u[0] + (uStar - s.vn) * (uStar + s.p / a);
#else
    const double den = S - uStar;
    const double inv = gpm_fast_rcp(a * den);  // one reciprocal for a/den and p/a
    const double dStar = a * a * inv;
    st[3] = u[3] * s.ir + (uStar - s.vn) * (uStar + s.p * den * inv);
#endif
#pragma unroll
    for (int k = 0; k < 4; k++) F[k] = Fk[k] + S * (st[k] * dStar - u[k]);
}

#if !GPM_EXACT
// Fast mode: hllc's arithmetic with the branches turned into selects.  Every
// lane evaluates the star state, and the selects keep what hllc's branch
// would have returned (the physical flux of the chosen side when the star
// state is not used), so the flux is hllc's for admissible states.  Returns
// false, with F undefined, when either state is inadmissible.  Without
// branches the solves of a face's Gauss points can be scheduled together.
template <int DIR>
__device__ __forceinline__ bool hllc_select(const double* ul, const double* ur, double* F) {
    const double rr = gpm_fast_rcp(ul[0] * ur[0]);
    const Prim L = c2p<DIR>(ul, ur[0] * rr);
    const Prim R = c2p<DIR>(ur, ul[0] * rr);
    const double SL = fmin(L.vn - L.c, R.vn - R.c);
    const double SR = fmax(L.vn + L.c, R.vn + R.c);
    const double numerL = SL - L.vn, numerR = SR - R.vn;
    double uStar = ul[0] * L.vn * numerL - ur[0] * R.vn * numerR;
    uStar = (R.p - L.p) + uStar;
    const double aL = ul[0] * numerL, aR = ur[0] * numerR;
    uStar = uStar * gpm_fast_rcp(aL - aR);
    const bool left = (SL < 0.) && (uStar >= 0.);
    const bool right = (uStar < 0.) && (SR >= 0.);
    const bool useL = (SL >= 0.) || left;  // whose physical flux hllc returns or corrects
    double u[4];
#pragma unroll
    for (int k = 0; k < 4; k++) u[k] = useL ? ul[k] : ur[k];
    Prim s;
    s.vn = useL ? L.vn : R.vn;
    s.vt = useL ? L.vt : R.vt;
    s.p = useL ? L.p : R.p;
    s.ir = useL ? L.ir : R.ir;
    const double S = left ? SL : SR;
    const double a = left ? aL : aR;
    double Fk[4];
    phys_flux<DIR>(u, s, Fk);
    double st[4];
    st[0] = 1.;
    st[DIR == 0 ? 1 : 2] = uStar;
    st[DIR == 0 ? 2 : 1] = s.vt;
    const double den = S - uStar;
    const double inv = gpm_fast_rcp(a * den);
    const double dStar = a * a * inv;
    st[3] = u[3] * s.ir + (uStar - s.vn) * (uStar + s.p * den * inv);
    const bool star = left || right;
#pragma unroll
    for (int k = 0; k < 4; k++) F[k] = star ? Fk[k] + S * (st[k] * dStar - u[k]) : Fk[k];
    return L.adm && R.adm;
}
#endif

// The same primitive recovery, physical flux and HLLC with the direction a
// runtime value (0: x, 1: y): every FP64 expression is the one hllc<DIR>
// evaluates, only the choice of normal and tangential components is a select,
// so in the exact mode (no FMA contraction) the result has the same bits; in
// the fast mode the compiler's contraction may differ at rounding level.  A
// warp whose lanes hold x and y faces then issues each FP64 instruction once
// instead of once per direction.
__device__ __forceinline__ Prim c2p_dyn(const double* u, int dir, double ir_in = 0.0) {
    Prim s;
#if GPM_EXACT
    const double vx = u[1] / u[0];
    const double vy = u[2] / u[0];
    s.p = (GPM_GAMMA - 1.) * (u[3] - (0.5 * (u[1] * u[1] + u[2] * u[2]) / u[0]));
    s.c = sqrt(GPM_GAMMA * s.p / u[0]);
#else
    const double ir = ir_in;
    const double vx = u[1] * ir;
    const double vy = u[2] * ir;
    s.p = (GPM_GAMMA - 1.) * (u[3] - 0.5 * (u[1] * vx + u[2] * vy));
    s.c = gpm_fast_sqrt(GPM_GAMMA * s.p * ir);  // NaN for p <= 0, which is inadmissible
    s.ir = ir;
#endif
    s.vx = vx;
    s.vn = dir == 0 ? vx : vy;
    s.vt = dir == 0 ? vy : vx;
    s.adm = !(le_zero_or_nan(u[0]) || le_zero_or_nan(s.p));
    return s;
}

__device__ __forceinline__ void phys_flux_dyn(const double* u, const Prim& s, int dir, double* r) {
    const double a = u[0] * (s.vn * s.vn) + s.p;   // normal momentum flux
    const double b = (dir == 0 ? u[2] : u[1]) * s.vn;  // tangential momentum flux
    r[0] = dir == 0 ? u[1] : u[2];
    r[1] = dir == 0 ? a : b;
    r[2] = dir == 0 ? b : a;
    r[3] = s.vn * (u[3] + s.p);
}

__device__ __forceinline__ void hllc_dyn(const double* ul, const double* ur, int dir, double* F) {
#if GPM_EXACT
    const Prim L = c2p_dyn(ul, dir);
    const Prim R = c2p_dyn(ur, dir);
#else
    const double rr = gpm_fast_rcp(ul[0] * ur[0]);
    const Prim L = c2p_dyn(ul, dir, ur[0] * rr);
    const Prim R = c2p_dyn(ur, dir, ul[0] * rr);
#endif
    const double SL = fmin(L.vn - L.c, R.vn - R.c);
    const double SR = fmax(L.vn + L.c, R.vn + R.c);
    if (!(L.adm && R.adm)) {
        const double bad = 1. / (R.vx - R.vx);
        F[0] = F[1] = F[2] = F[3] = bad;
        return;
    }
    if (SL >= 0.) {
        phys_flux_dyn(ul, L, dir, F);
        return;
    }
    const double numerL = SL - L.vn, numerR = SR - R.vn;
    double uStar = ul[0] * L.vn * numerL - ur[0] * R.vn * numerR;
    uStar = (R.p - L.p) + uStar;
    const double aL = ul[0] * numerL, aR = ur[0] * numerR;
#if GPM_EXACT
    uStar = uStar / (aL - aR);
#else
    uStar = uStar * gpm_fast_rcp(aL - aR);
#endif
    const bool left = (SL < 0.) && (uStar >= 0.);
    const bool right = (uStar < 0.) && (SR >= 0.);
    if (!left && !right) {
        phys_flux_dyn(ur, R, dir, F);
        return;
    }
    const double* u = left ? ul : ur;
    const Prim& s = left ? L : R;
    const double S = left ? SL : SR;
    const double a = left ? aL : aR;
    double Fk[4];
    phys_flux_dyn(u, s, dir, Fk);
    double st[4];
    st[0] = 1.;
    st[1] = dir == 0 ? uStar : s.vt;
    st[2] = dir == 0 ? s.vt : uStar;
#if GPM_EXACT
    const double dStar = a / (S - uStar);
    st[3] = u[3] / u[0] + (uStar - s.vn) * (uStar + s.p / a);
#else
    const double den = S - uStar;
    const double inv = gpm_fast_rcp(a * den);
    const double dStar = a * a * inv;
    st[3] = u[3] * s.ir + (uStar - s.vn) * (uStar + s.p * den * inv);
#endif
#pragma unroll
    for (int k = 0; k < 4; k++) F[k] = Fk[k] + S * (st[k] * dStar - u[k]);
}

// Left/right wave-speed bounds and physical fluxes, as HLL_Flux and LLF_Flux
// gather them (mod_HLL.f90:29-69, mod_LLF.f90:29-95); vxr is the right
// state's x velocity for the 1/(vx-vx) of an inadmissible pair.
struct LR {
    double vmcl, vpcl, vmcr, vpcr, Fl[4], Fr[4], vxr;
    bool adm;
};

template <int DIR>
__device__ __forceinline__ LR lr_gather(const double* ul, const double* ur) {
    LR r;
#if GPM_EXACT
    const Prim L = c2p<DIR>(ul), R = c2p<DIR>(ur);
#else
    const double rr = gpm_fast_rcp(ul[0] * ur[0]);
    const Prim L = c2p<DIR>(ul, ur[0] * rr), R = c2p<DIR>(ur, ul[0] * rr);
#endif
    r.vmcl = L.vn - L.c;
    r.vpcl = L.vn + L.c;
    r.vmcr = R.vn - R.c;
    r.vpcr = R.vn + R.c;
    phys_flux<DIR>(ul, L, r.Fl);
    phys_flux<DIR>(ur, R, r.Fr);
    r.vxr = R.vx;
    r.adm = L.adm && R.adm;
    return r;
}

// HLL_Flux, mod_HLL.f90:11-169.
template <int DIR>
__device__ __forceinline__ void hll(const double* ul, const double* ur, double* F) {
    const LR s = lr_gather<DIR>(ul, ur);
    const double SL = fmin(s.vmcl, s.vmcr), SR = fmax(s.vpcl, s.vpcr);
    if (!s.adm) {
        const double bad = 1. / (s.vxr - s.vxr);
        F[0] = F[1] = F[2] = F[3] = bad;
    } else if (SL > 0.) {
#pragma unroll
        for (int k = 0; k < 4; k++) F[k] = s.Fl[k];
    } else if (SR < 0.) {
#pragma unroll
        for (int k = 0; k < 4; k++) F[k] = s.Fr[k];
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) F[k] = ((SR * s.Fl[k] - SL * s.Fr[k]) + (SR * SL) * (ur[k] - ul[k])) / (SR - SL);
    }
}

// LLF_Flux, mod_LLF.f90:11-175.
template <int DIR>
__device__ __forceinline__ void llf(const double* ul, const double* ur, double* F) {
    const LR s = lr_gather<DIR>(ul, ur);
    if (!s.adm) {
        const double bad = 1. / (s.vxr - s.vxr);
        F[0] = F[1] = F[2] = F[3] = bad;
        return;
    }
    const double m = fmax(fmax(fmax(fabs(s.vmcl), fabs(s.vmcr)), fabs(s.vpcl)), fabs(s.vpcr));
#pragma unroll
    for (int k = 0; k < 4; k++) F[k] = 0.5 * (s.Fr[k] + s.Fl[k]) - (0.5 * m) * (ur[k] - ul[k]);
}

// unsplit_flux, mod_unsplit.f90:11-71.  An inadmissible pair gives
// 1/(no-no) where no holds the right state's vy^2, the last value c2p_local
// wrote to it.
template <int DIR>
__device__ __forceinline__ void unsplit(const double* ul, const double* ur, double* F) {
#if GPM_EXACT
    const Prim L = c2p<0>(ul), R = c2p<0>(ur);
#else
    const double rr = gpm_fast_rcp(ul[0] * ur[0]);
    const Prim L = c2p<0>(ul, ur[0] * rr), R = c2p<0>(ur, ul[0] * rr);
#endif
    // c2p<0>: vn = vx, vt = vy
    if (!(L.adm && R.adm)) {
        const double no = R.vt * R.vt;
        const double bad = 1. / (no - no);
        F[0] = F[1] = F[2] = F[3] = bad;
        return;
    }
    const double a = 1.1 * fmax(ul[0] * L.c, ur[0] * R.c);
    const double vnL = DIR == 0 ? L.vn : L.vt, vnR = DIR == 0 ? R.vn : R.vt;
    const double vtL = DIR == 0 ? L.vt : L.vn, vtR = DIR == 0 ? R.vt : R.vn;
    const double pistar = 0.5 * (L.p + R.p) - (0.5 * a) * (vnR - vnL);
    const double ustar = 0.5 * (vnL + vnR) - (0.5 * (R.p - L.p)) / a;
    const double trans = -(0.5 * a) * (vtR - vtL);
    const double* u = ustar > 0 ? ul : ur;
#pragma unroll
    for (int k = 0; k < 4; k++) F[k] = u[k] * ustar;
    F[DIR == 0 ? 1 : 2] = F[DIR == 0 ? 1 : 2] + pistar;
    F[DIR == 0 ? 2 : 1] = F[DIR == 0 ? 2 : 1] + trans;
    F[3] = F[3] + pistar * ustar;
}

// The Riemann solvers other than HLLC as one out-of-line function per
// direction, so that the many face-kernel instantiations inline only HLLC;
// states pass by value (no local-memory arrays on the HLLC path).
struct Flux4 {
    double f[4];
};

template <int DIR>
__device__ __noinline__ Flux4 riemann_other(int nflux, double l0, double l1, double l2, double l3, double r0,
                                            double r1, double r2, double r3) {
    const double ul[4] = {l0, l1, l2, l3}, ur[4] = {r0, r1, r2, r3};
    Flux4 F;
    if (nflux == 101) llf<DIR>(ul, ur, F.f);
    else if (nflux == 102) hll<DIR>(ul, ur, F.f);
    else unsplit<DIR>(ul, ur, F.f);
    return F;
}

// The Riemann solver of numFlux (mod_FE.f90:84-91); nflux is the same for
// every thread of a launch, so the switch does not diverge.
template <int DIR>
__device__ __forceinline__ void riemann(int nflux, const double* ul, const double* ur, double* F) {
    if (nflux == 100) {
        hllc<DIR>(ul, ur, F);
    } else {
        const Flux4 r = riemann_other<DIR>(nflux, ul[0], ul[1], ul[2], ul[3], ur[0], ur[1], ur[2], ur[3]);
        F[0] = r.f[0]; F[1] = r.f[1]; F[2] = r.f[2]; F[3] = r.f[3];
    }
}

// Face flux with Gauss quadrature, mod_FE.f90:80-98: sum_g Fg*w_g from zero.
template <int DIR, int NGP>
__device__ __forceinline__ void quad_flux(const double (*uL)[4], const double (*uR)[4], const double* gw, double* F,
                                          int nflux = 100) {
    double acc[4];
#if !GPM_EXACT
    if (nflux == 100) {  // HLLC without branches; NaN flux at an inadmissible Gauss point
        bool adm = true;
#pragma unroll
        for (int g = 0; g < NGP; g++) {
            double Fg[4];
            adm = hllc_select<DIR>(uL[g], uR[g], Fg) && adm;
#pragma unroll
            for (int k = 0; k < 4; k++) acc[k] = (g == 0) ? Fg[k] * gw[0] : acc[k] + Fg[k] * gw[g];
        }
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
#pragma unroll
        for (int k = 0; k < 4; k++) F[k] = adm ? acc[k] : nan;
        return;
    }
#endif
#pragma unroll
    for (int g = 0; g < NGP; g++) {
        double Fg[4];
        riemann<DIR>(nflux, uL[g], uR[g], Fg);
#pragma unroll
        for (int k = 0; k < 4; k++) acc[k] = (g == 0) ? Fg[k] * gw[0] : acc[k] + Fg[k] * gw[g];
    }
#if GPM_EXACT
#pragma unroll
    for (int k = 0; k < 4; k++) F[k] = plus_zero(acc[k]);
#else
#pragma unroll
    for (int k = 0; k < 4; k++) F[k] = acc[k];
#endif
}

// shock_detector, mod_subroutine_MOOD.f90:191-238, on Uin around (l, n), in
// two side-effect-free halves that the MOOD loop may evaluate on different
// warps: shock_flow, the compressive-flow tests divV < -max(dx,dy)^2 and
// Mach > 0.2, and shock_grad, the pressure-jump test gradP > 5.
#if GPM_EXACT
__device__ __forceinline__ bool shock_flow(const Cell& c, const Cell& L, const Cell& R, const Cell& B,
                                           const Cell& T, double dx, double dy) {
    double divV = (R.mx - L.mx) / dx + (T.my - B.my) / dy;
    divV = 0.5 * divV / c.r;
    divV = divV - 0.5 * (c.mx * (R.r - L.r) / dx + c.my * (T.r - B.r) / dy) / (c.r * c.r);
    const double Ca = 1.4 * pressure(c) / c.r;
    double Mach = (c.mx * c.mx + c.my * c.my) / (c.r * c.r);
    Mach = sqrt(Mach / Ca);
    const double m = fmax(dx, dy);
    return (divV < -(m * m)) && (Mach > 0.2);
}

__device__ __forceinline__ bool shock_grad(const Cell& L, const Cell& R, const Cell& B, const Cell& T, double dx,
                                           double dy) {
    const double pL = pressure(L), pR = pressure(R), pB = pressure(B), pT = pressure(T);
    const double gradP = 0.5 * (fabs(pR - pL) / fmin(pL, pR) / dx + fabs(pT - pB) / fmin(pB, pT) / dy);
    return gradP > 5.0;
}
#else
// Fast mode: p with a supplied 1/rho.
__device__ __forceinline__ double pressure_ir(const Cell& u, double ir) {
    return (GPM_GAMMA - 1.) * (u.e - 0.5 * (u.mx * u.mx + u.my * u.my) * ir);
}

// Fast mode: the same three tests with six Newton reciprocals (gpm_fast_rcp)
// in place of the nineteen IEEE divisions; the quantities agree with the
// exact form to rounding for admissible states.  A lone warp pays ~64 cycles
// per FP64 instruction, and a short MOOD pass waits on this chain.
__device__ __forceinline__ bool shock_flow(const Cell& c, const Cell& L, const Cell& R, const Cell& B,
                                           const Cell& T, double dx, double dy) {
    const double ixy = gpm_fast_rcp(dx * dy);
    const double idx = dy * ixy, idy = dx * ixy;
    const double ir = gpm_fast_rcp(c.r), ir2 = ir * ir;
    double divV = (R.mx - L.mx) * idx + (T.my - B.my) * idy;
    divV = 0.5 * divV * ir;
    divV = divV - 0.5 * (c.mx * (R.r - L.r) * idx + c.my * (T.r - B.r) * idy) * ir2;
    const double Ca = 1.4 * pressure_ir(c, ir) * ir;
    const double Mach = gpm_fast_sqrt((c.mx * c.mx + c.my * c.my) * ir2 * gpm_fast_rcp(Ca));  // NaN at rest: not > 0.2
    const double m = fmax(dx, dy);
    return (divV < -(m * m)) && (Mach > 0.2);
}

__device__ __forceinline__ bool shock_grad(const Cell& L, const Cell& R, const Cell& B, const Cell& T, double dx,
                                           double dy) {
    const double ixy = gpm_fast_rcp(dx * dy);
    const double idx = dy * ixy, idy = dx * ixy;
    const double rlr = gpm_fast_rcp(L.r * R.r), rbt = gpm_fast_rcp(B.r * T.r);
    const double pL = pressure_ir(L, R.r * rlr), pR = pressure_ir(R, L.r * rlr);
    const double pB = pressure_ir(B, T.r * rbt), pT = pressure_ir(T, B.r * rbt);
    const double gradP = 0.5 * (fabs(pR - pL) * gpm_fast_rcp(fmin(pL, pR)) * idx +
                                fabs(pT - pB) * gpm_fast_rcp(fmin(pB, pT)) * idy);
    return gradP > 5.0;
}
#endif

__device__ __forceinline__ bool shock_detector(const Cell& c, const Cell& L, const Cell& R, const Cell& B,
                                               const Cell& T, double dx, double dy) {
    return shock_flow(c, L, R, B, T, dx, dy) && shock_grad(L, R, B, T, dx, dy);
}

// An order-1 cell is never checked again (mod_subroutine_MOOD.f90:41), so a
// NaN or non-positive density or pressure in it survives the stage; callers
// report it (GPM_STATUS_NAN) without changing the result.
__device__ __forceinline__ bool inadmissible(const Cell& uo) {
    if (le_zero_or_nan(uo.r)) return true;
#if GPM_EXACT
    return le_zero_or_nan(pressure(uo));
#else
    return le_zero_or_nan(pressure_ir(uo, gpm_fast_rcp(uo.r)));
#endif
}

// DETECTION checks for one interior cell (mod_subroutine_MOOD.f90:41-131),
// in three parts that the MOOD loop may evaluate on different warps:
//   mood_uout_part  the tests that read Uout: positivity (:43-51) and the DMP
//                   bounds with the plateau test (:55-70); 0 passes, 1
//                   troubled, 2 the DMP bound is violated;
//   mood_shock_part the shock detector (:53, :191-238), on Uin only;
//   mood_u2_smooth  the U2 smooth-extremum test in x or in y (:74-119), on
//                   Uin only: GP second derivatives of rho at the 5 cross
//                   cells, each from that cell's own 5-point cross.
// A cell is troubled iff part 1 says 1, or it says 2, the shock detector
// fires and, with U2 on, neither direction is smooth.  Every part is side
// effect free, so evaluating them in any order, or all of them, gives the
// reference's decision.  uin points at Uin(1, l, n) of a padded array of row
// pitch 4*nx doubles.
#if GPM_EXACT
__device__ __forceinline__ int mood_uout_part(const Cell& uo, const double* __restrict__ uin, int nx,
                                              const GridGeom& g) {
    if (le_zero_or_nan(uo.r)) return 1;
    const double p = pressure(uo);
    if (le_zero_or_nan(p)) return 1;
    if (!g.dmp) return 0;
    const size_t row = (size_t)4 * nx;
    const double c = __ldg(uin), l = __ldg(uin - 4), r = __ldg(uin + 4), b = __ldg(uin - row), t = __ldg(uin + row);
    const double mn = fmin(fmin(fmin(fmin(c, l), b), t), r);
    const double mx = fmax(fmax(fmax(fmax(c, l), b), t), r);
    const double Mm = mx - mn;
    if (!(Mm > g.dx * g.dx * g.dx)) return 0;          // plateau, :68
    return ((uo.r > mx) || (uo.r < mn)) ? 2 : 0;        // :70
}
#else
// A double's bits as an integer whose signed order is the double's order
// (negative values have their magnitude bits flipped); its own inverse.
__device__ __forceinline__ long long ord_key(double x) {
    const long long b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double key_val(long long k) {
    return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL));
}

// Fast mode: the same tests in ~9 FP64-pipe instructions instead of ~24 (each
// double min, max and compare is one).  For rho > 0, p > 0 iff
// rho*E - (mx^2 + my^2)/2 > 0, so positivity needs no reciprocal; the DMP
// bounds are the integer min and max of the densities' order keys, and the
// bound test compares keys.  The decisions are the exact form's except where
// p is within rounding of 0, or a density of Uin is NaN (which fmin/fmax
// would skip).
__device__ __forceinline__ int mood_uout_part(const Cell& uo, const double* __restrict__ uin, int nx,
                                              const GridGeom& g) {
    if (le_zero_or_nan(uo.r)) return 1;
    const double ke2 = uo.mx * uo.mx + uo.my * uo.my;
    if (!(uo.r * uo.e - 0.5 * ke2 > 0.)) return 1;     // p <= 0 or NaN
    if (!g.dmp) return 0;
    const size_t row = (size_t)4 * nx;
    const long long c = ord_key(__ldg(uin)), l = ord_key(__ldg(uin - 4)), r = ord_key(__ldg(uin + 4));
    const long long b = ord_key(__ldg(uin - row)), t = ord_key(__ldg(uin + row));
    const long long mn = llmin(llmin(llmin(llmin(c, l), b), t), r);
    const long long mx = llmax(llmax(llmax(llmax(c, l), b), t), r);
    const double Mm = key_val(mx) - key_val(mn);
    if (!(Mm > g.dx * g.dx * g.dx)) return 0;          // plateau, :68
    const long long k = ord_key(uo.r);
    return (k > mx || k < mn) ? 2 : 0;                 // :70
}
#endif

__device__ __forceinline__ bool mood_shock_part(const double* __restrict__ uin, int nx, const GridGeom& g) {
    const size_t row = (size_t)4 * nx;
    const Cell C = ld_cell(uin), Lc = ld_cell(uin - 4), Rc = ld_cell(uin + 4);
    const Cell Bc = ld_cell(uin - row), Tc = ld_cell(uin + row);
    return shock_detector(C, Lc, Rc, Bc, Tc, g.dx, g.dy);
}

// The shock detector's two halves on their own, for warps that run one each.
__device__ __forceinline__ bool mood_shock_flow_part(const double* __restrict__ uin, int nx, const GridGeom& g) {
    const size_t row = (size_t)4 * nx;
    const Cell C = ld_cell(uin), Lc = ld_cell(uin - 4), Rc = ld_cell(uin + 4);
    const Cell Bc = ld_cell(uin - row), Tc = ld_cell(uin + row);
    return shock_flow(C, Lc, Rc, Bc, Tc, g.dx, g.dy);
}

__device__ __forceinline__ bool mood_shock_grad_part(const double* __restrict__ uin, int nx, const GridGeom& g) {
    const size_t row = (size_t)4 * nx;
    const Cell Lc = ld_cell(uin - 4), Rc = ld_cell(uin + 4);
    const Cell Bc = ld_cell(uin - row), Tc = ld_cell(uin + row);
    return shock_grad(Lc, Rc, Bc, Tc, g.dx, g.dy);
}

// DIR 0: the x test on D2x, 1: the y test on D2y.
template <int DIR>
__device__ __forceinline__ bool mood_u2_smooth(const double* __restrict__ uin, int nx, const GridGeom& g,
                                               const double* d2) {
    const size_t row = (size_t)4 * nx;
    const int ci_[5] = {-1, 0, 1, 0, 0}, cj_[5] = {0, 0, 0, -1, 1};  // (-1,0),(0,0),(1,0),(0,-1),(0,1)
    double D[5];
    if (g.u2_fd) {
        // POL_MOOD (:81-84): dot_product((1,-2,1), rho(l+i-1:l+i+1, n+j))/dx**2;
        // 1*a and -2*b are exact, so the sum is (a - 2b) + c in either FP mode.
        const ptrdiff_t step = DIR == 0 ? 4 : (ptrdiff_t)row;
        const double h = DIR == 0 ? g.dx : g.dy;
#pragma unroll
        for (int s = 0; s < 5; s++) {
            const double* base = uin + (ptrdiff_t)4 * ci_[s] + (ptrdiff_t)row * cj_[s];
            D[s] = ((__ldg(base - step) + -2. * __ldg(base)) + __ldg(base + step)) / (h * h);
        }
    } else {
#pragma unroll
        for (int s = 0; s < 5; s++) {
            const double* base = uin + (ptrdiff_t)4 * ci_[s] + (ptrdiff_t)row * cj_[s];
            double q[5];
#pragma unroll
            for (int k = 0; k < 5; k++) q[k] = __ldg(base + (ptrdiff_t)4 * st_ox(k) + (ptrdiff_t)row * st_oy(k));
            double sum = d2[0] * q[0];
#pragma unroll
            for (int k = 1; k < 5; k++) sum = sum + d2[k] * q[k];
            D[s] = sum;
        }
    }
    const double Xmin = fmin(fmin(fmin(fmin(D[0], D[1]), D[2]), D[3]), D[4]);
    const double Xmax = fmax(fmax(fmax(fmax(D[0], D[1]), D[2]), D[3]), D[4]);
    const double delta = g.u2_tol ? fmax(g.dx, g.dy) : 0.0;
    return (Xmin * Xmax > -delta) && ((fmax(fabs(Xmin), fabs(Xmax)) < delta) || (fabs(Xmin / Xmax) >= 1. / 2));
}

__device__ __forceinline__ bool mood_troubled(const Cell& uo, const double* __restrict__ uin, int nx,
                                              const GridGeom& g, const double* d2x, const double* d2y) {
    const int r = mood_uout_part(uo, uin, nx, g);
    if (r != 2) return r == 1;
    if (!mood_shock_part(uin, nx, g)) return false;
    if (!g.u2) return true;
    if (mood_u2_smooth<0>(uin, nx, g, d2x)) return false;
    return !mood_u2_smooth<1>(uin, nx, g, d2y);
}
