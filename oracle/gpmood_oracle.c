/*
 * gpmood_oracle.c -- CPU restatement of the GP-MOOD per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for the CUDA path, never shipped or
 * measured as the product).  Parity against the Fortran binary is unpinned (no
 * Fortran compiler exists here or on the GPU host); see gpmood_oracle.h for the
 * checks that pin this restatement instead.
 *
 * Every routine restates the reference Fortran expression by expression, in
 * the same evaluation order, so that a build with -ffp-contract=off gives the
 * bits gfortran -O3 gives on x86-64 (SSE2, no FMA).  Fortran facts honoured:
 *   - -fdefault-real-8 (gp-mood-code/Makefile:13): every default real literal
 *     and variable is a double, including q in DETECTION;
 *   - pressure() reads its dummy u through the name U (physics.f90:141);
 *   - gamma = 1.4 (constants.f90:9), so (y-1.) is the double 1.4 - 1.0;
 *   - dot_product/sum accumulate sequentially from zero.
 * NaN handling of MIN/MAX is unspecified in Fortran; this restatement uses
 * IEEE minNum/maxNum (fmin/fmax), and so does the CUDA path.
 */
#define __STDC_WANT_IEC_60559_TYPES_EXT__
#include "gpmood_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef _Float128 q128;

#define NGC 4
#define GAMMA 1.4
/* Fortran variable indices rho,momx,momy,ener = 1..4 (constants.f90:38). */
enum { RHO = 0, MOMX = 1, MOMY = 2, ENER = 3 };
/* Face ids iL,iT,iR,iB = 1..4 (constants.f90:40). */
enum { IL = 0, IT = 1, IR = 2, IB = 3 };

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------ */
/* GP weight precompute, GP_init.f90:26-357 and linalg.f90:5-95 (real(16)). */

/* Stencil offsets of the sphere stencil, GP_init.f90:97-138 (order-nested). */
static const int k_ixiy[13][2] = {
    {0, 0}, {-1, 0}, {0, 1}, {1, 0}, {0, -1},
    {-1, -1}, {-1, 1}, {1, 1}, {1, -1}, {0, -2}, {-2, 0}, {0, 2}, {2, 0}};

static int stcl_sz(int ord) /* GP_init.f90:14-23 */
{
    return ord == 1 ? 1 : ord == 3 ? 5 : ord == 5 ? 13 : 25;
}

typedef struct { q128 l16, dx16, dy16, pi16, ospi; } gpq;

/* Tpred_1D_fun, GP_init.f90:446-455 */
static q128 tpred_1d(const gpq* g, q128 delta, q128 h)
{
    q128 s2 = sqrtf128((q128)2);
    q128 expp = (delta + (q128)1 / 2) / (s2 * (g->l16 / h));
    q128 expm = (delta - (q128)1 / 2) / (s2 * (g->l16 / h));
    return sqrtf128(g->pi16 / 2) * (g->l16 / h) * (erff128(expp) - erff128(expm));
}

/* Tpred_d2x_1D_fun, GP_init.f90:431-443 */
static q128 tpred_d2x_1d(const gpq* g, q128 delta, q128 h)
{
    q128 fm = delta - (q128)0.5;
    q128 fp = delta + (q128)0.5;
    q128 lh = g->l16 / h;
    q128 expm = -(fm * fm) / (2 * (lh * lh));
    q128 expp = -(fp * fp) / (2 * (lh * lh));
    return ((q128)1 / (g->l16 * g->l16)) * (fm * expf128(expm) - fp * expf128(expp));
}

/* intg_kernel_SE, GP_init.f90:459-511: one factor of the separable integral. */
static q128 se_factor(const gpq* g, q128 d, q128 lod)
{
    q128 s2 = sqrtf128((q128)2);
    q128 a11 = (d + 1) / (s2 * lod);
    q128 a12 = (d - 1) / (s2 * lod);
    q128 a21 = -(((d + 1) * (d + 1)) / (2 * (lod * lod)));
    q128 a22 = -(((d - 1) * (d - 1)) / (2 * (lod * lod)));
    q128 a31 = d / (s2 * lod);
    q128 a32 = -(d * d) / (2 * (lod * lod));
    return (sqrtf128(g->pi16) * (lod * lod)) *
           (a11 * erff128(a11) + a12 * erff128(a12) + g->ospi * (expf128(a21) + expf128(a22)) -
            2 * (a31 * erff128(a31) + g->ospi * expf128(a32)));
}

static q128 intg_kernel_se(const gpq* g, q128 ddx, q128 ddy)
{
    q128 r = se_factor(g, ddx, g->l16 / g->dx16);
    return r * se_factor(g, ddy, g->l16 / g->dy16);
}

/* chol / reschol / invchol, linalg.f90:5-95 (row-major n x n). */
static void invchol(const q128* A, q128* AM1, int n)
{
    q128 L[13 * 13], y[13], x[13];
    memset(L, 0, sizeof L);
    for (int i = 0; i < n; i++) {
        q128 S = 0;
        for (int k = 0; k < i; k++) S = S + L[i * n + k] * L[i * n + k];
        L[i * n + i] = sqrtf128(A[i * n + i] - S);
        for (int j = i + 1; j < n; j++) {
            S = 0;
            for (int k = 0; k < i; k++) S = S + L[i * n + k] * L[j * n + k];
            L[j * n + i] = (A[j * n + i] - S) / L[i * n + i];
        }
    }
    for (int kk = 0; kk < n; kk++) {
        for (int i = 0; i < n; i++) {
            q128 b = (i == kk) ? (q128)1 : (q128)0;
            q128 S = 0;
            for (int j = 0; j < i; j++) S = S + L[i * n + j] * y[j];
            y[i] = (b - S) / L[i * n + i];
        }
        for (int i = n - 1; i >= 0; i--) {
            q128 S = 0;
            for (int j = i + 1; j < n; j++) S = S + L[j * n + i] * x[j]; /* LT(i,j) = L(j,i) */
            x[i] = (y[i] - S) / L[i * n + i];
        }
        for (int i = 0; i < n; i++) AM1[kk * n + i] = x[i];
    }
}

/* Gauss points (q128) and weights (double) of GP_init.f90:45-83.  ngp 1..3
 * points are quad expressions; ngp 4..5 points are double expressions. */
static void gauss_rule(int ngp, q128* pt, double* w)
{
    const double sq65 = sqrt(6. / 5), sq30 = sqrt(30.), third = 1. / 3;
    const double sq107 = sqrt(10. / 7), sq70 = sqrt(70.);
    q128 sq3 = sqrtf128((q128)3), sq35 = sqrtf128((q128)3 / 5);
    switch (ngp) {
    case 1: w[0] = 1.0; pt[0] = 0; break;
    case 2:
        w[0] = 0.5; w[1] = 0.5;
        pt[0] = -(q128)0.5 / sq3; pt[1] = (q128)0.5 / sq3;
        break;
    case 3:
        w[0] = 0.5 * 5. / 9; w[1] = 0.5 * 8. / 9; w[2] = 0.5 * 5. / 9;
        pt[0] = -(q128)0.5 * sq35; pt[1] = 0; pt[2] = (q128)0.5 * sq35;
        break;
    case 4:
        w[0] = 0.5 * (1. / 36) * (18. - sq30); w[1] = 0.5 * (1. / 36) * (18. + sq30);
        w[2] = 0.5 * (1. / 36) * (18. + sq30); w[3] = 0.5 * (1. / 36) * (18. - sq30);
        pt[0] = -0.5 * sqrt(3. / 7 + (2. / 7) * sq65);
        pt[1] = -0.5 * sqrt(3. / 7 - (2. / 7) * sq65);
        pt[2] = +0.5 * sqrt(3. / 7 - (2. / 7) * sq65);
        pt[3] = +0.5 * sqrt(3. / 7 + (2. / 7) * sq65);
        break;
    default:
        w[0] = 0.5 * (322. - 13 * sq70) / 900; w[1] = 0.5 * (322. + 13 * sq70) / 900;
        w[2] = 0.5 * 128. / 225;
        w[3] = 0.5 * (322. + 13 * sq70) / 900; w[4] = 0.5 * (322. - 13 * sq70) / 900;
        pt[0] = -0.5 * third * sqrt(5. + 2 * sq107);
        pt[1] = -0.5 * third * sqrt(5. - 2 * sq107);
        pt[2] = 0.;
        pt[3] = +0.5 * third * sqrt(5. - 2 * sq107);
        pt[4] = +0.5 * third * sqrt(5. + 2 * sq107);
        break;
    }
}

int orc_gp_presim(const orc_params* p, orc_gp* out)
{
    if (p->mord != 1 && p->mord != 3 && p->mord != 5) return -1;
    if (p->ngp < 1 || p->ngp > 5) return -1;
    memset(out, 0, sizeof *out);
    gpq g;
    g.dx16 = (q128)p->lx / p->lf;
    g.dy16 = (q128)p->ly / p->nf;
    g.l16 = (q128)p->ell_o_dx * (g.dx16 < g.dy16 ? g.dx16 : g.dy16); /* global_variables.f90:89 */
    g.pi16 = 4 * atanf128((q128)1);
    g.ospi = (q128)1 / sqrtf128(g.pi16);
    for (int k = 0; k < 13; k++) { out->ixiy[k][0] = k_ixiy[k][0]; out->ixiy[k][1] = k_ixiy[k][1]; }

    q128 gpt[5];
    gauss_rule(p->ngp, gpt, out->gauss_w);

    for (int ord = 1; ord <= p->mord; ord += 2) {
        int o = ord / 2, npt = stcl_sz(ord);
        q128 cov[13 * 13], inv[13 * 13];
        for (int k = 0; k < npt; k++)
            for (int h = 0; h < npt; h++)
                cov[k * npt + h] = intg_kernel_se(&g, (q128)(k_ixiy[k][0] - k_ixiy[h][0]),
                                                  (q128)(k_ixiy[k][1] - k_ixiy[h][1]));
        invchol(cov, inv, npt);
        /* error check, GP_init.f90:250-251: max |COV*INV - I| */
        q128 emax = 0;
        for (int i = 0; i < npt; i++)
            for (int j = 0; j < npt; j++) {
                q128 s = 0;
                for (int k = 0; k < npt; k++) s = s + cov[i * npt + k] * inv[k * npt + j];
                q128 e = fabsf128(s - (i == j ? (q128)1 : (q128)0));
                if (e > emax) emax = e;
            }
        out->inv_err[o] = (double)emax;

        for (int face = 0; face < 4; face++)
            for (int j = 0; j < p->ngp; j++) {
                q128 tp[13];
                for (int k = 0; k < npt; k++) {
                    q128 ix = k_ixiy[k][0], iy = k_ixiy[k][1], dxs, dys;
                    switch (face) { /* GP_init.f90:197-213 */
                    case IL: dxs = ix - (-(q128)1 / 2); dys = iy - gpt[j]; break;
                    case IT: dxs = ix - gpt[j]; dys = iy - ((q128)1 / 2); break;
                    case IR: dxs = ix - ((q128)1 / 2); dys = iy - gpt[j]; break;
                    default: dxs = ix - gpt[j]; dys = iy - (-(q128)1 / 2); break;
                    }
                    tp[k] = tpred_1d(&g, dxs, g.dx16);
                    tp[k] = tp[k] * tpred_1d(&g, dys, g.dy16);
                }
                double z[13];
                for (int h = 0; h < npt; h++) { /* matmul(T_pred, inv) rounded to double, :257 */
                    q128 s = 0;
                    for (int k = 0; k < npt; k++) s = s + tp[k] * inv[k * npt + h];
                    z[h] = (double)s;
                }
                double sum = 0.0; /* normalisation in double, :262 */
                for (int h = 0; h < npt; h++) sum = sum + z[h];
                for (int h = 0; h < npt; h++) out->zt[o][face][j][h] = z[h] / sum;
            }

        if (ord == 3) { /* GP_init.f90:231-242, 267-268 */
            q128 d2x[5], d2y[5];
            for (int k = 0; k < npt; k++) {
                q128 dkx = (q128)(k_ixiy[k][0] - k_ixiy[0][0]);
                q128 dky = (q128)(k_ixiy[k][1] - k_ixiy[0][1]);
                d2x[k] = tpred_d2x_1d(&g, dkx, g.dx16);
                d2x[k] = d2x[k] * tpred_1d(&g, dky, g.dy16);
                d2y[k] = tpred_d2x_1d(&g, dky, g.dy16);
                d2y[k] = d2y[k] * tpred_1d(&g, dkx, g.dx16);
            }
            for (int h = 0; h < npt; h++) {
                q128 sx = 0, sy = 0;
                for (int k = 0; k < npt; k++) {
                    sx = sx + d2x[k] * inv[k * npt + h];
                    sy = sy + d2y[k] * inv[k * npt + h];
                }
                out->d2x[h] = (double)sx;
                out->d2y[h] = (double)sy;
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Physics, physics.f90 and mod_HLLC.f90 */

double orc_pressure(const double u[4]) /* physics.f90:132-143 */
{
    return (GAMMA - 1.) * (u[ENER] - (0.5 * (u[MOMX] * u[MOMX] + u[MOMY] * u[MOMY]) / u[RHO]));
}

/* c2p_local, physics.f90:51-75 */
static void c2p_local(const double* u, double* vx, double* vy, double* vx2, double* vy2,
                      double* pres, double* c, int* adm)
{
    *vx = u[MOMX] / u[RHO];
    *vx2 = *vx * *vx;
    *vy = u[MOMY] / u[RHO];
    *vy2 = *vy * *vy;
    *pres = orc_pressure(u);
    *c = sqrt(GAMMA * *pres / u[RHO]);
    if (adm) {
        if ((u[RHO] <= 0.) || (*pres <= 0) || isnan(u[RHO]) || isnan(*pres)) *adm = 0;
    }
}

/* Flux, physics.f90:9-48 (admissible branch; the caller handles adm). */
static void phys_flux(const double* u, int dir, double vx, double vy, double vx2, double vy2,
                      double pres, double* r)
{
    if (dir == 1) {
        r[0] = u[MOMX];
        r[1] = u[RHO] * vx2 + pres;
        r[2] = u[MOMY] * vx;
        r[3] = vx * (u[ENER] + pres);
    } else {
        r[0] = u[MOMY];
        r[1] = u[MOMX] * vy;
        r[2] = u[RHO] * vy2 + pres;
        r[3] = vy * (u[ENER] + pres);
    }
}

/* HLLC_Flux, mod_HLLC.f90:11-169; dir 1 = x, 2 = y. */
void orc_hllc(const double* ul, const double* ur, int dir, double* F)
{
    double Fl[4], Fr[4], UstarL[4], UstarR[4];
    double vx, vy, vx2, vy2, pres, c;
    double vmcl, vpcl, vmcr, vpcr, SL, SR, vvL, vvR, presL, presR, other_velL, other_velR;
    int adm = 1, momdir, othermom;

    if (dir == 1) {
        momdir = MOMX; othermom = MOMY;
        c2p_local(ul, &vx, &vy, &vx2, &vy2, &pres, &c, &adm);
        vmcl = vx - c; vpcl = vx + c; vvL = vx; presL = pres; other_velL = vy;
        phys_flux(ul, dir, vx, vy, vx2, vy2, pres, Fl);
        c2p_local(ur, &vx, &vy, &vx2, &vy2, &pres, &c, &adm);
        vmcr = vx - c; vpcr = vx + c; vvR = vx; presR = pres; other_velR = vy;
        phys_flux(ur, dir, vx, vy, vx2, vy2, pres, Fr);
    } else {
        momdir = MOMY; othermom = MOMX;
        c2p_local(ul, &vx, &vy, &vx2, &vy2, &pres, &c, &adm);
        vmcl = vy - c; vpcl = vy + c; vvL = vy; presL = pres; other_velL = vx;
        phys_flux(ul, dir, vx, vy, vx2, vy2, pres, Fl);
        c2p_local(ur, &vx, &vy, &vx2, &vy2, &pres, &c, &adm);
        vmcr = vy - c; vpcr = vy + c; vvR = vy; presR = pres; other_velR = vx;
        phys_flux(ur, dir, vx, vy, vx2, vy2, pres, Fr);
    }
    SL = fmin(vmcl, vmcr);
    SR = fmax(vpcl, vpcr);

    if (!adm) { /* mod_HLLC.f90:166: 1/(vx-vx) with vx of the right state (+inf, or NaN) */
        for (int k = 0; k < 4; k++) F[k] = 1. / (vx - vx);
        return;
    }
    double numerL = SL - vvL, numerR = SR - vvR;
    double uStar = ul[RHO] * vvL * numerL - ur[RHO] * vvR * numerR; /* :121-123 */
    uStar = (presR - presL) + uStar;
    uStar = uStar / (ul[RHO] * numerL - ur[RHO] * numerR);
    double denomL = SL - uStar, denomR = SR - uStar;
    double dStarL = ul[RHO] * numerL / denomL;
    double dStarR = ur[RHO] * numerR / denomR;

    UstarL[RHO] = 1.;
    UstarL[momdir] = uStar;
    UstarL[othermom] = other_velL;
    UstarL[ENER] = ul[ENER] / ul[RHO] + (uStar - vvL) * (uStar + presL / (ul[RHO] * numerL));
    for (int k = 0; k < 4; k++) UstarL[k] = UstarL[k] * dStarL;

    UstarR[RHO] = 1.;
    UstarR[momdir] = uStar;
    UstarR[othermom] = other_velR;
    UstarR[ENER] = ur[ENER] / ur[RHO] + (uStar - vvR) * (uStar + presR / (ur[RHO] * numerR));
    for (int k = 0; k < 4; k++) UstarR[k] = UstarR[k] * dStarR;

    if (SL >= 0.) {
        for (int k = 0; k < 4; k++) F[k] = Fl[k];
    } else if ((SL < 0.) && (uStar >= 0.)) {
        for (int k = 0; k < 4; k++) F[k] = Fl[k] + SL * (UstarL[k] - ul[k]);
    } else if ((uStar < 0.) && (SR >= 0.)) {
        for (int k = 0; k < 4; k++) F[k] = Fr[k] + SR * (UstarR[k] - ur[k]);
    } else {
        for (int k = 0; k < 4; k++) F[k] = Fr[k];
    }
}

/* The left and right states' primitive data in the face-normal frame, as
 * HLL_Flux / LLF_Flux gather them (mod_HLL.f90:29-69, mod_LLF.f90:29-95). */
typedef struct { double vmcl, vpcl, vmcr, vpcr, Fl[4], Fr[4], vx_last; int adm; } lr_state;

static lr_state lr_gather(const double* ul, const double* ur, int dir)
{
    lr_state s;
    double vx, vy, vx2, vy2, pres, c;
    s.adm = 1;
    c2p_local(ul, &vx, &vy, &vx2, &vy2, &pres, &c, &s.adm);
    s.vmcl = (dir == 1 ? vx : vy) - c;
    s.vpcl = (dir == 1 ? vx : vy) + c;
    phys_flux(ul, dir, vx, vy, vx2, vy2, pres, s.Fl);
    c2p_local(ur, &vx, &vy, &vx2, &vy2, &pres, &c, &s.adm);
    s.vmcr = (dir == 1 ? vx : vy) - c;
    s.vpcr = (dir == 1 ? vx : vy) + c;
    phys_flux(ur, dir, vx, vy, vx2, vy2, pres, s.Fr);
    s.vx_last = vx;
    return s;
}

/* HLL_Flux, mod_HLL.f90:11-169 */
void orc_hll(const double* ul, const double* ur, int dir, double* F)
{
    lr_state s = lr_gather(ul, ur, dir);
    const double SL = fmin(s.vmcl, s.vmcr), SR = fmax(s.vpcl, s.vpcr);
    if (!s.adm) {
        for (int k = 0; k < 4; k++) F[k] = 1. / (s.vx_last - s.vx_last);
        return;
    }
    if (SL > 0.) {
        for (int k = 0; k < 4; k++) F[k] = s.Fl[k];
    } else if (SR < 0.) {
        for (int k = 0; k < 4; k++) F[k] = s.Fr[k];
    } else {
        for (int k = 0; k < 4; k++) F[k] = ((SR * s.Fl[k] - SL * s.Fr[k]) + (SR * SL) * (ur[k] - ul[k])) / (SR - SL);
    }
}

/* LLF_Flux, mod_LLF.f90:11-175 */
void orc_llf(const double* ul, const double* ur, int dir, double* F)
{
    lr_state s = lr_gather(ul, ur, dir);
    if (!s.adm) {
        for (int k = 0; k < 4; k++) F[k] = 1. / (s.vx_last - s.vx_last);
        return;
    }
    /* max(abs(vmcl), abs(vmcr), abs(vpcl), abs(vpcr)) */
    const double m = fmax(fmax(fmax(fabs(s.vmcl), fabs(s.vmcr)), fabs(s.vpcl)), fabs(s.vpcr));
    for (int k = 0; k < 4; k++) F[k] = 0.5 * (s.Fr[k] + s.Fl[k]) - (0.5 * m) * (ur[k] - ul[k]);
}

/* unsplit_flux, mod_unsplit.f90:11-71 */
void orc_unsplit(const double* ul, const double* ur, int dir, double* F)
{
    double vxL, vyL, vxR, vyR, pL, pR, cL, cR, no;
    int adm = 1;
    c2p_local(ul, &vxL, &vyL, &no, &no, &pL, &cL, &adm);
    c2p_local(ur, &vxR, &vyR, &no, &no, &pR, &cR, &adm); /* no = vy_R^2, written last */
    const double a = 1.1 * fmax(ul[RHO] * cL, ur[RHO] * cR);
    double pistar, ustar, trans;
    if (dir == 1) {
        pistar = 0.5 * (pL + pR) - (0.5 * a) * (vxR - vxL);
        ustar = 0.5 * (vxL + vxR) - (0.5 * (pR - pL)) / a;
        trans = -(0.5 * a) * (vyR - vyL);
    } else {
        pistar = 0.5 * (pL + pR) - (0.5 * a) * (vyR - vyL);
        ustar = 0.5 * (vyL + vyR) - (0.5 * (pR - pL)) / a;
        trans = -(0.5 * a) * (vxR - vxL);
    }
    if (!adm) {
        for (int k = 0; k < 4; k++) F[k] = 1. / (no - no);
        return;
    }
    const double* u = ustar > 0 ? ul : ur;
    for (int k = 0; k < 4; k++) F[k] = u[k] * ustar;
    if (dir == 1) {
        F[MOMX] = F[MOMX] + pistar;
        F[MOMY] = F[MOMY] + trans;
    } else {
        F[MOMY] = F[MOMY] + pistar;
        F[MOMX] = F[MOMX] + trans;
    }
    F[ENER] = F[ENER] + pistar * ustar;
}

/* ------------------------------------------------------------------ */
/* Grid helpers */

typedef struct { int lf, nf, nx, ny; } grid;
static grid mkgrid(const orc_params* p)
{
    grid g = {p->lf, p->nf, p->lf + 2 * NGC, p->nf + 2 * NGC};
    return g;
}
/* cell (l, n), l in lb..le = 1-ngc..lf+ngc */
#define CIDX(G, l, n) ((size_t)((n) + NGC - 1) * (size_t)(G).nx + (size_t)((l) + NGC - 1))
#define UP(U, G, l, n) ((U) + 4 * CIDX(G, l, n))

static double dx_of(const orc_params* p) { return (double)((q128)p->lx / p->lf); }
static double dy_of(const orc_params* p) { return (double)((q128)p->ly / p->nf); }

/* primitive_to_conservative, physics.f90:146-160 */
static void p2c(double r, double u, double v, double pr, double* out)
{
    out[RHO] = r;
    out[MOMX] = r * u;
    out[MOMY] = r * v;
    out[ENER] = ((pr / (GAMMA - 1.)) + 0.5 * r * (u * u + v * v));
}

/* f_DMR, IC.f90:336-355 */
static void f_dmr(double x, double y, double* r)
{
    double xmin = 1. / 6;
    double ymin = (x - xmin) * sqrt(3.);
    if (y > ymin) p2c(8., 7.1447096, -4.125, 116.5, r);
    else p2c(1.4, 0.0, 0.0, 1.0, r);
}

void orc_boundary(const orc_params* p, double* U, double t_rk) /* BC.f90:10-421 */
{
    grid G = mkgrid(p);
    const int lf = p->lf, nf = p->nf;
    const double dx = dx_of(p), dy = dy_of(p);
    if (p->bc_type == 17) { /* Neumann :18-43 */
        for (int n = 1 - NGC; n <= nf + NGC; n++) {
            for (int l = lf + 1; l <= lf + NGC; l++) memcpy(UP(U, G, l, n), UP(U, G, lf, n), 32);
            for (int l = 1 - NGC; l <= 0; l++) memcpy(UP(U, G, l, n), UP(U, G, 1, n), 32);
        }
        for (int l = 1 - NGC; l <= lf + NGC; l++) {
            for (int n = nf + 1; n <= nf + NGC; n++) memcpy(UP(U, G, l, n), UP(U, G, l, nf), 32);
            for (int n = 1 - NGC; n <= 0; n++) memcpy(UP(U, G, l, n), UP(U, G, l, 1), 32);
        }
    } else if (p->bc_type == 18) { /* Periodic :45-59 */
        for (int n = 1 - NGC; n <= nf + NGC; n++) {
            for (int i = 0; i < NGC; i++) memcpy(UP(U, G, lf + 1 + i, n), UP(U, G, 1 + i, n), 32);
            for (int i = 0; i < NGC; i++) memcpy(UP(U, G, 1 - NGC + i, n), UP(U, G, lf - NGC + 1 + i, n), 32);
        }
        for (int l = 1 - NGC; l <= lf + NGC; l++) {
            for (int i = 0; i < NGC; i++) memcpy(UP(U, G, l, nf + 1 + i), UP(U, G, l, 1 + i), 32);
            for (int i = 0; i < NGC; i++) memcpy(UP(U, G, l, 1 - NGC + i), UP(U, G, l, nf - NGC + 1 + i), 32);
        }
    } else if (p->bc_type == 20) { /* Reflective :89-135 */
        for (int n = 1 - NGC; n <= nf + NGC; n++) {
            int k = 0;
            for (int l = lf + 1; l <= lf + NGC; l++) {
                memcpy(UP(U, G, l, n), UP(U, G, lf - k, n), 32);
                k++;
                UP(U, G, l, n)[MOMX] = -UP(U, G, l, n)[MOMX];
            }
            k = 0;
            for (int l = 0; l >= 1 - NGC; l--) {
                memcpy(UP(U, G, l, n), UP(U, G, 1 + k, n), 32);
                k++;
                UP(U, G, l, n)[MOMX] = -UP(U, G, l, n)[MOMX];
            }
        }
        for (int l = 1 - NGC; l <= lf + NGC; l++) {
            int k = 0;
            for (int n = nf + 1; n <= nf + NGC; n++) {
                memcpy(UP(U, G, l, n), UP(U, G, l, nf - k), 32);
                k++;
                UP(U, G, l, n)[MOMY] = -UP(U, G, l, n)[MOMY];
            }
            k = 0;
            for (int n = 0; n >= 1 - NGC; n--) {
                memcpy(UP(U, G, l, n), UP(U, G, l, 1 + k), 32);
                k++;
                UP(U, G, l, n)[MOMY] = -UP(U, G, l, n)[MOMY];
            }
        }
    } else if (p->bc_type == 35) { /* DMR :283-341 */
        for (int n = 1 - NGC; n <= nf + NGC; n++) {
            double y = n * dy - dy / 2;
            for (int l = lf + 1; l <= lf + NGC; l++) f_dmr(l * dx - dx / 2, y, UP(U, G, l, n));
            for (int l = 1 - NGC; l <= 0; l++) f_dmr(l * dx - dx / 2, y, UP(U, G, l, n));
        }
        for (int l = 1 - NGC; l <= lf + NGC; l++) {
            double xmin = 1. / 6 + 10. * t_rk / (0.5 * sqrt(3.)) + 1. / sqrt(3.);
            double x = l * dx - dx / 2;
            for (int n = nf + 1; n <= nf + NGC; n++) {
                if (x < xmin) p2c(8., 7.1447096, -4.125, 116.5, UP(U, G, l, n));
                else p2c(1.4, 0.0, 0.0, 1.0, UP(U, G, l, n));
            }
            if (x > 1. / 6) {
                int k = 0;
                for (int n = 0; n >= 1 - NGC; n--) {
                    memcpy(UP(U, G, l, n), UP(U, G, l, 1 + k), 32);
                    k++;
                    UP(U, G, l, n)[MOMY] = -UP(U, G, l, n)[MOMY];
                }
            } else {
                for (int n = 0; n >= 1 - NGC; n--) p2c(8., 7.1447096, -4.125, 116.5, UP(U, G, l, n));
            }
        }
    } else if (p->bc_type == 19) { /* Dirichlet :61-87 */
        for (int n = 1 - NGC; n <= nf + NGC; n++) {
            for (int l = lf + 1; l <= lf + NGC; l++)
                p2c(1. + 0.2 * sin(5 * ((l * dx - dx / 2) - 4.5)), 0., 0., 1., UP(U, G, l, n));
            for (int l = 1 - NGC; l <= 0; l++) p2c(3.857143, 2.629369, 0., 10.33333, UP(U, G, l, n));
        }
        for (int l = 1 - NGC; l <= lf + NGC; l++) {
            for (int n = nf + 1; n <= nf + NGC; n++) memcpy(UP(U, G, l, n), UP(U, G, l, nf), 32);
            for (int n = 1 - NGC; n <= 0; n++) memcpy(UP(U, G, l, n), UP(U, G, l, 1), 32);
        }
    } else if (p->bc_type == 201 || p->bc_type == 301) { /* Mach800_BC :137-179, DoubleMach800_BC :181-237 */
        for (int n = 1 - NGC; n <= nf + NGC; n++) {
            for (int l = lf + 1; l <= lf + NGC; l++) memcpy(UP(U, G, l, n), UP(U, G, lf, n), 32);
            for (int l = 1 - NGC; l <= 0; l++) memcpy(UP(U, G, l, n), UP(U, G, 1, n), 32);
        }
        for (int l = 1 - NGC; l <= lf + NGC; l++)
            for (int n = nf + 1; n <= nf + NGC; n++) memcpy(UP(U, G, l, n), UP(U, G, l, nf), 32);
        if (p->bc_type == 301)
            for (int l = 1 - NGC; l <= lf + NGC; l++)
                for (int n = nf + 1; n <= nf + NGC; n++)
                    if (fabs((l * dx - dx / 2) - 0.75) <= 0.05) p2c(1.4, 0.0, -800.0, 1.0, UP(U, G, l, n));
        for (int l = 1 - NGC; l <= lf + NGC; l++)
            for (int n = 1 - NGC; n <= 0; n++) memcpy(UP(U, G, l, n), UP(U, G, l, 1), 32);
        for (int l = 1 - NGC; l <= lf + NGC; l++)
            for (int n = 1 - NGC; n <= 0; n++)
                if (fabs((l * dx - dx / 2) - 0.75) <= 0.05) p2c(1.4, 0.0, 800.0, 1.0, UP(U, G, l, n));
    } else if (p->bc_type == 401) { /* RMI_BC :239-281 */
        for (int n = 1 - NGC; n <= nf + NGC; n++)
            for (int l = 1 - NGC; l <= 0; l++) p2c(2.666666666666667, 2. * sqrt(1.4), 0., 4.5, UP(U, G, l, n));
        for (int n = 1 - NGC; n <= nf + NGC; n++)
            for (int l = lf + 1; l <= lf + NGC; l++) memcpy(UP(U, G, l, n), UP(U, G, lf, n), 32);
        for (int l = 1 - NGC; l <= lf + NGC; l++) {
            int k = 0;
            for (int n = nf + 1; n <= nf + NGC; n++) {
                memcpy(UP(U, G, l, n), UP(U, G, l, nf - k), 32);
                k++;
                UP(U, G, l, n)[MOMY] = -UP(U, G, l, n)[MOMY];
            }
            k = 0;
            for (int n = 0; n >= 1 - NGC; n--) {
                memcpy(UP(U, G, l, n), UP(U, G, l, 1 + k), 32);
                k++;
                UP(U, G, l, n)[MOMY] = -UP(U, G, l, n)[MOMY];
            }
        }
    } else if (p->bc_type == 402) { /* RT_BC :343-390, g = real(0.1, 4) (global_variables.f90:129) */
        const double grav = (double)0.1f;
        for (int n = 1 - NGC; n <= nf + NGC; n++) {
            int k = 0;
            for (int l = lf + 1; l <= lf + NGC; l++) {
                memcpy(UP(U, G, l, n), UP(U, G, lf - k, n), 32);
                k++;
                UP(U, G, l, n)[MOMX] = -UP(U, G, l, n)[MOMX];
            }
            k = 0;
            for (int l = 0; l >= 1 - NGC; l--) {
                memcpy(UP(U, G, l, n), UP(U, G, 1 + k, n), 32);
                k++;
                UP(U, G, l, n)[MOMX] = -UP(U, G, l, n)[MOMX];
            }
        }
        for (int l = 1 - NGC; l <= lf + NGC; l++) {
            int k = 0;
            for (int n = nf + 1; n <= nf + NGC; n++) {
                const double* q = UP(U, G, l, nf - k);
                const double pr = orc_pressure(q);
                p2c(q[RHO], q[MOMX] / q[RHO], -(q[MOMY] / q[RHO]), pr - 2 * k * dy * grav * q[RHO], UP(U, G, l, n));
                k++;
            }
            k = 0;
            for (int n = 0; n >= 1 - NGC; n--) {
                const double* q = UP(U, G, l, 1 + k);
                const double pr = orc_pressure(q);
                p2c(q[RHO], q[MOMX] / q[RHO], -(q[MOMY] / q[RHO]), pr + 2 * k * dy * grav * q[RHO], UP(U, G, l, n));
                k++;
            }
        }
    } else if (p->bc_type == 403) { /* KH_BC :392-414: periodic in x, Neumann in y */
        for (int n = 1 - NGC; n <= nf + NGC; n++) {
            for (int i = 0; i < NGC; i++) memcpy(UP(U, G, lf + 1 + i, n), UP(U, G, 1 + i, n), 32);
            for (int i = 0; i < NGC; i++) memcpy(UP(U, G, 1 - NGC + i, n), UP(U, G, lf - NGC + 1 + i, n), 32);
        }
        for (int l = 1 - NGC; l <= lf + NGC; l++) {
            for (int n = nf + 1; n <= nf + NGC; n++) memcpy(UP(U, G, l, n), UP(U, G, l, nf), 32);
            for (int n = 1 - NGC; n <= 0; n++) memcpy(UP(U, G, l, n), UP(U, G, l, 1), 32);
        }
    }
}

double orc_setdt(const orc_params* p, const double* U, double dtfinal) /* physics.f90:78-129 */
{
    grid G = mkgrid(p);
    const double dx = dx_of(p), dy = dy_of(p);
    /* deprecated/physics.f90:94-97: dx0 = Lx/lf0 in double */
    const int reduce = p->setdt_kind == 1 && p->lf0 > 0 && p->nf0 > 0;
    const double dx0 = reduce ? p->lx / p->lf0 : dx, dy0 = reduce ? p->ly / p->nf0 : dy;
    double dt = 1.0e30;
    for (int n = 1 - NGC; n <= p->nf + NGC; n++)
        for (int l = 1 - NGC; l <= p->lf + NGC; l++) {
            double vx, vy, vx2, vy2, pres, c;
            c2p_local(UP(U, G, l, n), &vx, &vy, &vx2, &vy2, &pres, &c, NULL);
            if (p->setdt_kind == 1) /* deprecated/physics.f90:106-118 */
                dt = fmin(dt, fmin(dx0 / (fabs(vx) + c), dy0 / (fabs(vy) + c)));
            else
                dt = fmin(dt, 1.0 / (1.0 / (dx / (fabs(vx) + c)) + 1.0 / (dy / (fabs(vy) + c))));
        }
    if (reduce) dt = dt * pow(dx / dx0, (double)p->mord / 4); /* deprecated/physics.f90:122-124 */
    dt = dt * p->cfl;
    if (dt > dtfinal) dt = dtfinal;
    return dt;
}

/* ------------------------------------------------------------------ */
/* Stepping context: the module-global arrays of global_variables.f90. */

struct orc_ctx {
    orc_params p;
    orc_gp gp;
    grid G;
    double dx, dy;
    size_t ncell;
    double *uh;    /* Uh(4, iL:iB, ngp, cell), global_variables.f90:29 */
    double *lfx;   /* L_Flux_x(4, face (l+1/2, n)) indexed by cell (l,n), mod_FE.f90:30 */
    double *lfy;   /* L_Flux_y(4, face (l, n+1/2)) indexed by cell (l,n), mod_FE.f90:31 */
    int *cellgpo;  /* CellGPO, :59 */
    unsigned char *detcell, *detfx, *detfy, *decrease;
    double *u1, *u2;
    double *rk4[5];  /* U3, U4, FU3, FU4, Fl of SSP_RK4_ (U1, U2 are u1, u2), on first use */
    int cc_col;      /* NN_GP_MOOD_CC_ blend column (the input count L), or -1 */
    float *cc_w;     /* values_NN(cc_col, n, 1:2) for n = 0..nf+1; NULL: no blend */
    double dt_sim;   /* deprecated/main.f90 slow-start step (0: off) */
    int pol_fd;      /* POL_MOOD: U2 from D2O2 finite differences (mod_subroutine_MOOD.f90:81-84) */
};

/* NN_GP_MOOD_CC_ (mod_NN_GP_MOOD_CC.f90:11-85): with w != NULL every face
 * state of order 1 is the cell value and every one of order 3 is
 * real(v1,8)*Uin + real(v2,8)*Uh, (v1, v2) = values_NN(l, n, :): (0, 1) except
 * column col of rows 1..nf, where w[2n], w[2n+1] hold the pair the
 * reference's network loop leaves there (mod_NN.f90:41,44 write
 * values_NN(L, n, :); Fortran reads `l` as the input count L). */
void orc_set_cc(orc_ctx* c, int col, const float* w)
{
    free(c->cc_w);
    c->cc_w = NULL;
    c->cc_col = -1;
    if (!w) return;
    const size_t n = 2 * (size_t)(c->p.nf + 2);
    c->cc_w = (float*)malloc(n * sizeof(float));
    if (!c->cc_w) return;
    memcpy(c->cc_w, w, n * sizeof(float));
    c->cc_col = col;
}

orc_ctx* orc_create(const orc_params* p)
{
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof *c);
    if (!c) return NULL;
    c->p = *p;
    c->dt_sim = p->slow_start > 0 ? fmin(p->slow_start, 1e30) : 0; /* dt_sim = min(1.e-10, dt), dt = 1e30 */
    if (orc_gp_presim(p, &c->gp) != 0) { free(c); return NULL; }
    if (p->method == 200 || p->method == 201) {
        /* POL_MOOD_ / Unlim_POL_ (mod_pol_MOOD.f90, mod_Unlim_Pol.f90): the
         * weights of pol_presim (GP_init.f90:359-419) at order 3, o3_coef of
         * constants.f90:61, Pol_zT_o3(point, face, gauss point); the stepping
         * is GP_MOOD's (DETECTION on) or GP_SE's (none). */
        const double oc[5] = {15. / 18, 1. / 3, 1. / (4 * sqrt(3.)), -1. / (4 * sqrt(3.)), -1. / 6};
        enum { M = 0, CN = 1, CT = 2, FT = 3, FN = 4 };
        const int tab[4][2][5] = {{{M, CN, FT, FN, CT}, {M, CN, CT, FN, FT}},  /* iL */
                                  {{M, CT, CN, FT, FN}, {M, FT, CN, CT, FN}},  /* iT */
                                  {{M, FN, FT, CN, CT}, {M, FN, CT, CN, FT}},  /* iR */
                                  {{M, CT, FN, FT, CN}, {M, FT, FN, CT, CN}}}; /* iB */
        for (int f = 0; f < 4; f++)
            for (int j = 0; j < 2; j++) {
                for (int m = 0; m < 13; m++) c->gp.zt[1][f][j][m] = 0.0;
                for (int m = 0; m < 5; m++) c->gp.zt[1][f][j][m] = oc[tab[f][j][m]];
                c->gp.zt[0][f][j][0] = 1.0;
            }
        c->pol_fd = p->method == 200;
        c->p.method = p->method == 200 ? 2 : 202;
    }
    if (p->method == 1) { /* FOG_ (mod_FOG.f90): Uh = Uin, no DETECTION: GP_SE at order 1 */
        c->p.method = 202;
        c->p.mord = 1;
    }
    c->G = mkgrid(p);
    c->dx = dx_of(p);
    c->dy = dy_of(p);
    c->ncell = (size_t)c->G.nx * c->G.ny;
    c->uh = (double*)malloc(c->ncell * 16 * p->ngp * sizeof(double));
    c->lfx = (double*)calloc(c->ncell * 4, sizeof(double));
    c->lfy = (double*)calloc(c->ncell * 4, sizeof(double));
    c->cellgpo = (int*)malloc(c->ncell * sizeof(int));
    c->detcell = (unsigned char*)malloc(c->ncell);
    c->detfx = (unsigned char*)malloc(c->ncell);
    c->detfy = (unsigned char*)malloc(c->ncell);
    c->decrease = (unsigned char*)malloc(c->ncell);
    c->u1 = (double*)malloc(c->ncell * 4 * sizeof(double));
    c->u2 = (double*)malloc(c->ncell * 4 * sizeof(double));
    if (!c->uh || !c->lfx || !c->lfy || !c->cellgpo || !c->detcell || !c->detfx || !c->detfy ||
        !c->decrease || !c->u1 || !c->u2) {
        orc_destroy(c);
        return NULL;
    }
    return c;
}

void orc_destroy(orc_ctx* c)
{
    if (!c) return;
    free(c->uh); free(c->lfx); free(c->lfy); free(c->cellgpo); free(c->detcell);
    free(c->detfx); free(c->detfy); free(c->decrease); free(c->u1); free(c->u2);
    for (int i = 0; i < 5; i++) free(c->rk4[i]);
    free(c->cc_w);
    free(c);
}

const orc_gp* orc_weights(const orc_ctx* c) { return &c->gp; }

#define UH(c, cell, face, g) ((c)->uh + (((size_t)(cell) * 4 + (face)) * (size_t)(c)->p.ngp + (g)) * 4)

/* GP_MOOD_ / GP_SE_ reconstruction, mod_GP_MOOD.f90:11-76 */
static void recons(orc_ctx* c, const double* Uin)
{
    const grid G = c->G;
    const int ngp = c->p.ngp, mord = c->p.mord;
    const int npt_m = stcl_sz(mord);
#pragma omp parallel for schedule(static)
    for (int n = 0; n <= G.nf + 1; n++)
        for (int l = 0; l <= G.lf + 1; l++) {
            size_t me = CIDX(G, l, n);
            double q[13][4];
            int done = 0;
            for (int i = 0; i < 4; i++) {
                int recon = 0, ord = 0;
                if (i == IL && c->detfx[CIDX(G, l - 1, n)]) {
                    ord = c->cellgpo[CIDX(G, l - 1, n)]; recon = 1;
                } else if (i == IR && c->detfx[me]) {
                    ord = c->cellgpo[CIDX(G, l + 1, n)]; recon = 1;
                } else if (i == IB && c->detfy[CIDX(G, l, n - 1)]) {
                    ord = c->cellgpo[CIDX(G, l, n - 1)]; recon = 1;
                } else if (i == IT && c->detfy[me]) {
                    ord = c->cellgpo[CIDX(G, l, n + 1)]; recon = 1;
                }
                if (!recon) continue;
                if (c->cellgpo[me] < ord) ord = c->cellgpo[me];
                if (c->p.method == 202) ord = mord; /* GP_SE_: always Mord, mod_GP_SE.f90:24 */
                if (!done) {
                    for (int j = 0; j < npt_m; j++)
                        memcpy(q[j], UP(Uin, G, l + k_ixiy[j][0], n + k_ixiy[j][1]), 32);
                    done = 1;
                }
                const int o = ord / 2, np = stcl_sz(ord);
                for (int j = 0; j < ngp; j++)
                    for (int k = 0; k < 4; k++) {
                        double s = 0.0;
                        for (int m = 0; m < np; m++) s = s + c->gp.zt[o][i][j][m] * q[m][k];
                        UH(c, me, i, j)[k] = s;
                    }
                if (c->cc_w) { /* mod_NN_GP_MOOD_CC.f90:63-70 */
                    double v1 = 0.0, v2 = 1.0;
                    if (l == c->cc_col && n >= 1 && n <= G.nf) {
                        v1 = (double)c->cc_w[2 * n];
                        v2 = (double)c->cc_w[2 * n + 1];
                    }
                    for (int j = 0; j < ngp; j++)
                        for (int k = 0; k < 4; k++) {
                            double* u = &UH(c, me, i, j)[k];
                            *u = ord == 1 ? q[0][k] : v1 * q[0][k] + v2 * *u;
                        }
                }
            }
        }
}

/* Face flux with Gauss quadrature, mod_FE.f90:80-98 (x) and :112-130 (y). */
static void face_flux(const orc_ctx* c, size_t cl, size_t cr, int dir, double* out)
{
    const int ngp = c->p.ngp;
    double Fg[5][4];
    for (int j = 0; j < ngp; j++) {
        const double* uL = UH(c, cl, dir == 1 ? IR : IT, j);
        const double* uR = UH(c, cr, dir == 1 ? IL : IB, j);
        switch (c->p.num_flux) { /* mod_FE.f90:84-91 */
        case 101: orc_llf(uL, uR, dir, Fg[j]); break;
        case 102: orc_hll(uL, uR, dir, Fg[j]); break;
        case 103: orc_unsplit(uL, uR, dir, Fg[j]); break;
        default: orc_hllc(uL, uR, dir, Fg[j]); break;
        }
    }
    for (int k = 0; k < 4; k++) {
        double s = 0.0;
        for (int j = 0; j < ngp; j++) s = s + Fg[j][k] * c->gp.gauss_w[j];
        out[k] = s;
    }
}

/* DETECTION, mod_subroutine_MOOD.f90:13-189.  Returns the number of
 * troubled cells (0 = MOOD_finished). */
static long long detection(orc_ctx* c, const double* Uin, double* Uout, double t_rk)
{
    const grid G = c->G;
    const orc_params* p = &c->p;
    const double dx = c->dx, dy = c->dy;
    orc_boundary(p, Uout, t_rk); /* :35 */

#pragma omp parallel for schedule(static)
    for (int n = 1; n <= G.nf; n++)
        for (int l = 1; l <= G.lf; l++) {
            size_t me = CIDX(G, l, n);
            int dec = 0;
            if (c->detcell[me] && c->cellgpo[me] > 1) {
                const double* uo = UP(Uout, G, l, n);
                if ((uo[RHO] <= 0.) || isnan(uo[RHO])) {
                    dec = 1;
                } else {
                    double pr = orc_pressure(uo);
                    if ((pr <= 0.) || isnan(pr)) {
                        dec = 1;
                    } else {
                        int shock = orc_shock_detector(p, Uin, l, n);
                        if (p->dmp && shock) {
                            double UB = UP(Uin, G, l, n - 1)[RHO], UL = UP(Uin, G, l - 1, n)[RHO];
                            double UM = UP(Uin, G, l, n)[RHO], UR = UP(Uin, G, l + 1, n)[RHO];
                            double UT = UP(Uin, G, l, n + 1)[RHO];
                            double mn = fmin(fmin(fmin(fmin(UM, UL), UB), UT), UR);
                            double mx = fmax(fmax(fmax(fmax(UM, UL), UB), UT), UR);
                            double Mm = mx - mn;
                            if (Mm > dx * dx * dx) { /* plateau, :68 */
                                if ((uo[RHO] > mx) || (uo[RHO] < mn)) {
                                    dec = 1;
                                    if (p->u2) { /* :74-119 */
                                        double D2x[3][3], D2y[3][3];
                                        for (int j = -1; j <= 1; j++)
                                            for (int i = -1; i <= 1; i++) {
                                                if (!(i == 0 || j == 0)) continue;
                                                if (c->pol_fd) { /* POL_MOOD, :81-84: D2O2 = (1,-2,1), /dx**2 */
                                                    const double m = UP(Uin, G, l + i, n + j)[RHO];
                                                    double sx = 0.0 + 1. * UP(Uin, G, l + i - 1, n + j)[RHO];
                                                    sx = sx + (-2.) * m;
                                                    sx = sx + 1. * UP(Uin, G, l + i + 1, n + j)[RHO];
                                                    double sy = 0.0 + 1. * UP(Uin, G, l + i, n + j - 1)[RHO];
                                                    sy = sy + (-2.) * m;
                                                    sy = sy + 1. * UP(Uin, G, l + i, n + j + 1)[RHO];
                                                    D2x[i + 1][j + 1] = sx / (dx * dx);
                                                    D2y[i + 1][j + 1] = sy / (dy * dy);
                                                    continue;
                                                }
                                                double q[5];
                                                for (int k = 0; k < 5; k++)
                                                    q[k] = UP(Uin, G, l + k_ixiy[k][0] + i, n + k_ixiy[k][1] + j)[RHO];
                                                double sx = 0.0, sy = 0.0;
                                                for (int k = 0; k < 5; k++) sx = sx + c->gp.d2x[k] * q[k];
                                                for (int k = 0; k < 5; k++) sy = sy + c->gp.d2y[k] * q[k];
                                                D2x[i + 1][j + 1] = sx;
                                                D2y[i + 1][j + 1] = sy;
                                            }
                                        double Xmin = fmin(fmin(fmin(fmin(D2x[0][1], D2x[1][1]), D2x[2][1]), D2x[1][0]), D2x[1][2]);
                                        double Xmax = fmax(fmax(fmax(fmax(D2x[0][1], D2x[1][1]), D2x[2][1]), D2x[1][0]), D2x[1][2]);
                                        double Ymin = fmin(fmin(fmin(fmin(D2y[0][1], D2y[1][1]), D2y[2][1]), D2y[1][0]), D2y[1][2]);
                                        double Ymax = fmax(fmax(fmax(fmax(D2y[0][1], D2y[1][1]), D2y[2][1]), D2y[1][0]), D2y[1][2]);
                                        double delta = 0.0;
                                        if (p->u2_tol) delta = fmax(dx, dy);
                                        if ((Xmin * Xmax > -delta) &&
                                            ((fmax(fabs(Xmin), fabs(Xmax)) < delta) || (fabs(Xmin / Xmax) >= 1. / 2)))
                                            dec = 0;
                                        else if ((Ymin * Ymax > -delta) &&
                                                 ((fmax(fabs(Ymin), fabs(Ymax)) < delta) || (fabs(Ymin / Ymax) >= 1. / 2)))
                                            dec = 0;
                                    }
                                }
                            }
                        }
                    }
                }
            }
            c->decrease[me] = (unsigned char)dec;
        }

    /* un-flag, :133-141 (serial: neighbouring cells share faces) */
    for (int n = 1; n <= G.nf; n++)
        for (int l = 1; l <= G.lf; l++) {
            size_t me = CIDX(G, l, n);
            if (!c->decrease[me]) {
                c->detcell[me] = 0;
                c->detfy[CIDX(G, l, n - 1)] = 0;
                c->detfy[me] = 0;
                c->detfx[CIDX(G, l - 1, n)] = 0;
                c->detfx[me] = 0;
            }
        }
    long long ndec = 0;
    for (int n = 1; n <= G.nf; n++) /* flag + cascade + reset, :148-185 */
        for (int l = 1; l <= G.lf; l++) {
            size_t me = CIDX(G, l, n);
            if (!c->decrease[me]) continue;
            ndec++;
            if (c->cellgpo[me] == 3) c->cellgpo[me] = 1;
            else if (c->cellgpo[me] > 3) c->cellgpo[me] = 3;
            size_t nb[5] = {CIDX(G, l, n - 1), CIDX(G, l - 1, n), me, CIDX(G, l + 1, n), CIDX(G, l, n + 1)};
            for (int k = 0; k < 5; k++) c->detcell[nb[k]] = 1;
            c->detfy[CIDX(G, l, n - 1)] = 1;
            c->detfy[me] = 1;
            c->detfx[me] = 1;
            c->detfx[CIDX(G, l - 1, n)] = 1;
            for (int k = 0; k < 5; k++) memcpy(Uout + 4 * nb[k], Uin + 4 * nb[k], 32);
        }
    return ndec;
}

int orc_shock_detector(const orc_params* p, const double* Uin, int l, int n) /* :191-238 */
{
    grid G = mkgrid(p);
    const double dx = dx_of(p), dy = dy_of(p);
    const double *uc = UP(Uin, G, l, n), *ul = UP(Uin, G, l - 1, n), *ur = UP(Uin, G, l + 1, n);
    const double *ub = UP(Uin, G, l, n - 1), *ut = UP(Uin, G, l, n + 1);
    double threshold1 = 5.0;
    double divV = (ur[MOMX] - ul[MOMX]) / dx + (ut[MOMY] - ub[MOMY]) / dy;
    divV = 0.5 * divV / uc[RHO];
    divV = divV - 0.5 * (uc[MOMX] * (ur[RHO] - ul[RHO]) / dx + uc[MOMY] * (ut[RHO] - ub[RHO]) / dy) /
                      (uc[RHO] * uc[RHO]);
    double Ca = 1.4 * orc_pressure(uc) / uc[RHO];
    double Mach = (uc[MOMX] * uc[MOMX] + uc[MOMY] * uc[MOMY]) / (uc[RHO] * uc[RHO]);
    Mach = sqrt(Mach / Ca);
    double pL = orc_pressure(ul), pR = orc_pressure(ur), pB = orc_pressure(ub), pT = orc_pressure(ut);
    double gradP = 0.5 * (fabs(pR - pL) / fmin(pL, pR) / dx + fabs(pT - pB) / fmin(pB, pT) / dy);
    if (p->csd_kind == 1) return (divV < -threshold1) && (gradP > threshold1); /* threshold2 = threshold1 */
    if (p->csd_kind == 2) return 1;
    double mxd = fmax(dx, dy);
    return (divV < -(mxd * mxd)) && (Mach > 0.2) && (gradP > threshold1);
}

int orc_forward_euler(orc_ctx* c, double* Uin, double* Uout, double dt, double t_rk,
                      const signed char* init_order, signed char* final_order, long long* counters)
{
    const grid G = c->G;
    const orc_params* p = &c->p;
    const size_t nc = c->ncell;
    for (size_t i = 0; i < nc; i++) c->cellgpo[i] = p->mord; /* mod_FE.f90:48 */
    if (init_order)                                         /* a-priori gate, :51-56 */
        for (int n = 1; n <= G.nf; n++)
            for (int l = 1; l <= G.lf; l++)
                c->cellgpo[CIDX(G, l, n)] = init_order[(size_t)(n - 1) * G.lf + (l - 1)];
    memset(c->detcell, 1, nc); /* :58-60 */
    memset(c->detfx, 1, nc);
    memset(c->detfy, 1, nc);
    orc_boundary(p, Uin, t_rk); /* :64 */
    memcpy(Uout, Uin, nc * 32); /* :66 */

    const int mood = (p->method == 2);
    int passes = 0;
    for (;;) { /* :69-174 */
        passes++;
        recons(c, Uin);
        /* Faces: the serial loop of :75-145 computes each flagged face once and
         * applies it to its two cells.  Computing all flagged fluxes first and
         * then accumulating per cell in the loop's visiting order (y face below,
         * x face left, x face right, y face above) gives the same bits. */
#pragma omp parallel for schedule(static)
        for (int n = 0; n <= G.nf; n++)
            for (int l = 0; l <= G.lf; l++) {
                size_t me = CIDX(G, l, n);
                if (c->detfx[me]) face_flux(c, me, CIDX(G, l + 1, n), 1, c->lfx + 4 * me);
                if (c->detfy[me]) face_flux(c, me, CIDX(G, l, n + 1), 2, c->lfy + 4 * me);
            }
        const double qx = dt / c->dx, qy = dt / c->dy;
#pragma omp parallel for schedule(static)
        for (int n = 0; n <= G.nf + 1; n++)
            for (int l = 0; l <= G.lf + 1; l++) {
                size_t me = CIDX(G, l, n);
                double* uo = Uout + 4 * me;
                const int dc = c->detcell[me];
                if (l <= G.lf && n >= 1) { /* y face (l, n-1) as its upper cell */
                    size_t f = CIDX(G, l, n - 1);
                    if (c->detfy[f] || dc)
                        for (int k = 0; k < 4; k++) uo[k] = uo[k] + qy * c->lfy[4 * f + k];
                }
                if (n <= G.nf && l >= 1) { /* x face (l-1, n) as its right cell */
                    size_t f = CIDX(G, l - 1, n);
                    if (c->detfx[f] || dc)
                        for (int k = 0; k < 4; k++) uo[k] = uo[k] + qx * c->lfx[4 * f + k];
                }
                if (n <= G.nf && l <= G.lf) { /* x face (l, n) as its left cell */
                    if (c->detfx[me] || dc)
                        for (int k = 0; k < 4; k++) uo[k] = uo[k] - qx * c->lfx[4 * me + k];
                }
                if (n <= G.nf && l <= G.lf) { /* y face (l, n) as its lower cell */
                    if (c->detfy[me] || dc)
                        for (int k = 0; k < 4; k++) uo[k] = uo[k] - qy * c->lfy[4 * me + k];
                }
            }
        long long ndec = 0;
        if (mood) {
            ndec = detection(c, Uin, Uout, t_rk);
        } else {
            orc_boundary(p, Uout, t_rk); /* keep ghosts consistent for the non-MOOD method */
        }
        if (counters) counters[0] += ndec;
        if (ndec == 0) break;
        if (passes > 1000) return -2;
    }
    if (counters) {
        counters[1] += passes;
        if (passes > counters[2]) counters[2] = passes;
    }
    if (final_order)
        for (int n = 1; n <= G.nf; n++)
            for (int l = 1; l <= G.lf; l++)
                final_order[(size_t)(n - 1) * G.lf + (l - 1)] = (signed char)c->cellgpo[CIDX(G, l, n)];
    if (p->integrator == 12) /* SSP_RK4 takes the increment dt*L(Uin), mod_FE.f90:188 */
        for (size_t i = 0; i < nc * 4; i++) Uout[i] = Uout[i] - Uin[i];
    return 0;
}

int orc_time_stepping(orc_ctx* c, double* Uin, double* Uout, double t, double dt,
                      const signed char* const* init_orders, signed char* const* stage_orders,
                      long long* counters)
{
    const size_t n4 = c->ncell * 4;
    int rc;
#define ORC_FE(k, in, out, trk) \
    orc_forward_euler(c, in, out, dt, trk, (init_orders && (k) < 3) ? init_orders[k] : NULL, \
                      (stage_orders && (k) < 3) ? stage_orders[k] : NULL, counters)
    const int integ = c->p.integrator ? c->p.integrator : 10;
    /* time_stepper.f90:17-21: t_rk = t unless SSP_RK3_ moves it */
    if (integ == 8) return ORC_FE(0, Uin, Uout, t);
    if (integ == 9) { /* SSP_RK2_, mod_SSP_RK2.f90:12-24 */
        if ((rc = ORC_FE(0, Uin, c->u1, t))) return rc;
        if ((rc = ORC_FE(1, c->u1, Uout, t))) return rc;
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n4; i++) Uout[i] = 0.5 * (Uin[i] + Uout[i]);
        return 0;
    }
    if (integ == 12) { /* SSP_RK4_, mod_SSP_RK4.f90:12-38 with the constants of constants.f90:46-51 */
        const double c1 = 0.391752226571890, a20 = 0.444370493651235, a21 = 0.555629506348765,
                     c2 = 0.368410593050371, a30 = 0.620101851488403, a32 = 0.379898148511597,
                     c3 = 0.251891774271694, a40 = 0.178079954393132, a43 = 0.821920045606868,
                     c4 = 0.544974750228521, f2 = 0.517231671970585, f3 = 0.096059710526147,
                     f4 = 0.386708617503269, ff3 = 0.063692468666290, ff4 = 0.226007483236906;
        for (int i = 0; i < 5; i++)
            if (!c->rk4[i] && !(c->rk4[i] = (double*)malloc(c->ncell * 32))) return -3;
        double *U1 = c->u1, *U2 = c->u2, *U3 = c->rk4[0], *U4 = c->rk4[1], *FU3 = c->rk4[2], *FU4 = c->rk4[3],
               *Fl = c->rk4[4];
        if ((rc = ORC_FE(0, Uin, Fl, t))) return rc;
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n4; i++) U1[i] = Uin[i] + c1 * Fl[i];
        if ((rc = ORC_FE(1, U1, Fl, t))) return rc;
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n4; i++) U2[i] = a20 * Uin[i] + a21 * U1[i] + c2 * Fl[i];
        if ((rc = ORC_FE(2, U2, Fl, t))) return rc;
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n4; i++) U3[i] = a30 * Uin[i] + a32 * U2[i] + c3 * Fl[i];
        if ((rc = ORC_FE(3, U3, FU3, t))) return rc;
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n4; i++) U4[i] = a40 * Uin[i] + a43 * U3[i] + c4 * FU3[i];
        if ((rc = ORC_FE(4, U4, FU4, t))) return rc;
#pragma omp parallel for schedule(static)
        for (size_t i = 0; i < n4; i++)
            Uout[i] = f2 * U2[i] + f3 * U3[i] + ff3 * FU3[i] + f4 * U4[i] + ff4 * FU4[i];
        return 0;
    }
#undef ORC_FE
    /* SSP_RK3_, mod_SSP_RK3.f90:12-39 */
    rc = orc_forward_euler(c, Uin, c->u1, dt, t, init_orders ? init_orders[0] : NULL,
                           stage_orders ? stage_orders[0] : NULL, counters);
    if (rc) return rc;
    rc = orc_forward_euler(c, c->u1, c->u2, dt, t + dt, init_orders ? init_orders[1] : NULL,
                           stage_orders ? stage_orders[1] : NULL, counters);
    if (rc) return rc;
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n4; i++) c->u2[i] = (0.75) * Uin[i] + 0.25 * c->u2[i];
    rc = orc_forward_euler(c, c->u2, Uout, dt, t + 0.5 * dt, init_orders ? init_orders[2] : NULL,
                           stage_orders ? stage_orders[2] : NULL, counters);
    if (rc) return rc;
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n4; i++) Uout[i] = (1. / 3) * Uin[i] + (2. / 3) * Uout[i];
    return 0;
}

/* ------------------------------------------------------------------ */
/* Initial conditions, IC.f90 */

typedef void (*icfun)(const orc_params*, double, double, double*);

static void fill_ic(const orc_params* p, double* U, icfun f)
{
    grid G = mkgrid(p);
    const double dx = dx_of(p), dy = dy_of(p);
    memset(U, 0, (size_t)G.nx * G.ny * 32);
    for (int n = 1 - NGC; n <= p->nf; n++) /* IC.f90:29-30 */
        for (int l = 1 - NGC; l <= p->lf; l++) f(p, l * dx - dx / 2, n * dy - dy / 2, UP(U, G, l, n));
    orc_boundary(p, U, 0.0); /* main.f90:125 */
}

static void ic_rp2d3(const orc_params* p, double x, double y, double* r) /* IC.f90:241-248 */
{
    (void)p;
    if ((x <= 0.8) && (y <= 0.8)) p2c(0.138, 1.206, 1.206, 0.029, r);
    if ((x >= 0.8) && (y <= 0.8)) p2c(0.5323, 0.0, 1.206, 0.3, r);
    if ((x <= 0.8) && (y >= 0.8)) p2c(0.5323, 1.206, 0.0, 0.3, r);
    if ((x >= 0.8) && (y >= 0.8)) p2c(1.5, 0.0, 0.0, 1.5, r);
}

static void ic_sedov(const orc_params* p, double x, double y, double* r) /* IC.f90:358-373 */
{
    const double dx = dx_of(p), dy = dy_of(p);
    double E = 1., m = dx < dy ? dx : dy, dr2 = (3.5 * m) * (3.5 * m), pi = 4 * atan(1.);
    double r2 = (x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5);
    if (sqrt(r2) < sqrt(dr2)) p2c(1.0, 0.0, 0.0, (1.4 - 1.) * E / (pi * dr2), r);
    else p2c(1.0, 0.0, 0.0, 1.e-5, r);
}

static void ic_dmr(const orc_params* p, double x, double y, double* r) { (void)p; f_dmr(x, y, r); }

/* f_isentropic_vortex, IC.f90:375-407 */
static void f_vortex(const orc_params* p, double x, double y, double xc, double yc, double t, double* res)
{
    const double pi = 4 * atan(1.);
    double beta = 5.0;
    double xp = x - t, yp = y - t;
    while (xp < 0.) xp = xp + 0.5 * p->lx;
    while (yp < 0.) yp = yp + 0.5 * p->ly;
    double r = sqrt((xp - xc) * (xp - xc) + (yp - yc) * (yp - yc));
    double rho = pow(1. - (1.4 - 1.) * (beta * beta / (8 * 1.4 * pi * pi)) * exp(1. - r * r), 1. / (1.4 - 1.));
    double vx = 1. - 0.5 * (beta / pi) * exp(0.5 * (1. - r * r)) * (yp - xc);
    double vy = 1. + 0.5 * (beta / pi) * exp(0.5 * (1. - r * r)) * (xp - yc);
    double pr = pow(rho, 1.4);
    p2c(rho, vx, vy, pr, res);
}

/* quadrature, IC.f90:491-534: 5x5 Gauss-Legendre cell average */
static void ic_vortex(const orc_params* p, double xm, double ym, double* r)
{
    const double dx = dx_of(p), dy = dy_of(p);
    double w[5], x[5];
    w[0] = (322.0 - 13.0 * sqrt(70.0)) / 900.0;
    w[1] = (322.0 + 13.0 * sqrt(70.0)) / 900.0;
    w[2] = 128.0 / 225.0;
    w[3] = (322.0 + 13.0 * sqrt(70.0)) / 900.0;
    w[4] = (322.0 - 13.0 * sqrt(70.0)) / 900.0;
    x[0] = -1.0 / 3.0 * sqrt(5.0 + 2.0 * sqrt(10.0 / 7.0));
    x[1] = -1.0 / 3.0 * sqrt(5.0 - 2.0 * sqrt(10.0 / 7.0));
    x[2] = 0.0;
    x[3] = +1.0 / 3.0 * sqrt(5.0 - 2.0 * sqrt(10.0 / 7.0));
    x[4] = +1.0 / 3.0 * sqrt(5.0 + 2.0 * sqrt(10.0 / 7.0));
    double ax = xm - dx / 2, bx = xm + dx / 2, ay = ym - dy / 2, by = ym + dy / 2;
    double lx = 0.5 * (bx - ax), cx = 0.5 * (ax + bx), ly = 0.5 * (by - ay), cy = 0.5 * (ay + by);
    double acc[4] = {0, 0, 0, 0}, f[4];
    for (int j = 0; j < 5; j++)
        for (int i = 0; i < 5; i++) {
            f_vortex(p, lx * x[i] + cx, ly * x[j] + cy, 0.5 * p->lx, 0.5 * p->ly, 0., f);
            for (int k = 0; k < 4; k++) acc[k] = acc[k] + w[j] * w[i] * f[k];
        }
    for (int k = 0; k < 4; k++) r[k] = (1. / (dx * dy)) * (acc[k] * lx * ly);
}

void orc_ic_rp2d3(const orc_params* p, double* U) { fill_ic(p, U, ic_rp2d3); }
void orc_ic_sedov(const orc_params* p, double* U) { fill_ic(p, U, ic_sedov); }
void orc_ic_dmr(const orc_params* p, double* U) { fill_ic(p, U, ic_dmr); }
void orc_ic_vortex(const orc_params* p, double* U) { fill_ic(p, U, ic_vortex); }

/* ------------------------------------------------------------------ */
/* main.f90:145-203 */
int orc_run(orc_ctx* c, double* U, double* t_io, int nsteps, long long* counters)
{
    double t = *t_io;
    int niter = 0;
    double* Ur = (double*)malloc(c->ncell * 32);
    if (!Ur) return -1;
    while ((t < c->p.tmax) && (niter < nsteps)) {
        niter++;
        double dtfinal = c->p.tmax - t;
        double dt = orc_setdt(&c->p, U, dtfinal);
        if (c->dt_sim > 0 && c->dt_sim < dt) { /* deprecated/main.f90: force a small dt for a slow start */
            dt = c->dt_sim;
            c->dt_sim = 2. * c->dt_sim;
        }
        int rc = orc_time_stepping(c, U, Ur, t, dt, NULL, NULL, counters);
        if (rc) { free(Ur); return rc; }
        t = t + dt;
        memcpy(U, Ur, c->ncell * 32);
    }
    free(Ur);
    *t_io = t;
    return niter;
}
