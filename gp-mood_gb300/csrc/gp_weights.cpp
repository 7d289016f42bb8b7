// gp_weights.cpp -- host precompute of the GP-SE reconstruction weights.
//
// Follows gp-mood-code/GP_init.f90:26-357 (GP_presim_sphere) and the
// Cholesky inverse of gp-mood-code/linalg.f90:5-95, in IEEE binary128 like the
// reference's real(16).  The weights are rounded to double once at the end,
// exactly where the reference rounds (GP_init.f90:257, 267-268), and the
// prediction weights are normalised to sum one in double (GP_init.f90:262).
//
// Squared-exponential kernel with length scale l; every quantity is an
// integral of the kernel over unit cells, so all distances are in cells:
//   covariance of two cell averages (GP_init.f90:459-511) and
//   prediction vector of a point value at a face Gauss point (:446-455),
//   second derivative at the cell centre (:431-443) for the U2 check.
#define __STDC_WANT_IEC_60559_TYPES_EXT__
#include <math.h>
#include <string.h>

#include "gpm_common.h"

namespace {

using f128 = _Float128;

// Diamond ("sphere") stencil, nested by order: 1 point, +4 (radius 1), +8 (radius 2).
// Ordering of gp-mood-code/GP_init.f90:97-138.
const int kStencil[13][2] = {{0, 0},  {-1, 0}, {0, 1},  {1, 0},  {0, -1}, {-1, -1}, {-1, 1},
                             {1, 1},  {1, -1}, {0, -2}, {-2, 0}, {0, 2},  {2, 0}};

int stencil_size(int ord) { return ord == 1 ? 1 : (ord == 3 ? 5 : 13); }

struct SeKernel {
    f128 ell;       // physical length scale, ell_o_dx * min(dx, dy)
    f128 hx, hy;    // cell sizes
    f128 pi, inv_sqrt_pi, sqrt2;

    // One factor of the cell-average covariance at separation d (cells), scale s = ell/h.
    f128 cov1d(f128 d, f128 s) const {
        const f128 a11 = (d + 1) / (sqrt2 * s);
        const f128 a12 = (d - 1) / (sqrt2 * s);
        const f128 a21 = -(((d + 1) * (d + 1)) / (2 * (s * s)));
        const f128 a22 = -(((d - 1) * (d - 1)) / (2 * (s * s)));
        const f128 a31 = d / (sqrt2 * s);
        const f128 a32 = -(d * d) / (2 * (s * s));
        return (sqrtf128(pi) * (s * s)) *
               (a11 * erff128(a11) + a12 * erff128(a12) + inv_sqrt_pi * (expf128(a21) + expf128(a22)) -
                2 * (a31 * erff128(a31) + inv_sqrt_pi * expf128(a32)));
    }
    f128 cov(f128 ddx, f128 ddy) const {
        f128 r = cov1d(ddx, ell / hx);
        return r * cov1d(ddy, ell / hy);
    }
    // Point value at offset d (cells) against the average of a unit cell.
    f128 pred1d(f128 d, f128 h) const {
        const f128 s = ell / h;
        const f128 up = (d + (f128)1 / 2) / (sqrt2 * s);
        const f128 dn = (d - (f128)1 / 2) / (sqrt2 * s);
        return sqrtf128(pi / 2) * s * (erff128(up) - erff128(dn));
    }
    // Second derivative (physical units) of pred1d at the cell centre.
    f128 pred1d_d2(f128 d, f128 h) const {
        const f128 m = d - (f128)0.5, p = d + (f128)0.5, s = ell / h;
        const f128 em = -(m * m) / (2 * (s * s));
        const f128 ep = -(p * p) / (2 * (s * s));
        return ((f128)1 / (ell * ell)) * (m * expf128(em) - p * expf128(ep));
    }
};

// Inverse of a symmetric positive definite matrix by Cholesky: A = L L^T, then
// one forward and one backward substitution per unit vector (linalg.f90:78-95).
void spd_inverse(const f128* a, f128* inv, int n) {
    f128 L[13][13] = {};
    for (int i = 0; i < n; i++) {
        f128 acc = 0;
        for (int k = 0; k < i; k++) acc = acc + L[i][k] * L[i][k];
        L[i][i] = sqrtf128(a[i * n + i] - acc);
        for (int j = i + 1; j < n; j++) {
            acc = 0;
            for (int k = 0; k < i; k++) acc = acc + L[i][k] * L[j][k];
            L[j][i] = (a[j * n + i] - acc) / L[i][i];
        }
    }
    for (int col = 0; col < n; col++) {
        f128 y[13], x[13];
        for (int i = 0; i < n; i++) {
            f128 acc = 0;
            for (int j = 0; j < i; j++) acc = acc + L[i][j] * y[j];
            y[i] = ((i == col ? (f128)1 : (f128)0) - acc) / L[i][i];
        }
        for (int i = n - 1; i >= 0; i--) {
            f128 acc = 0;
            for (int j = i + 1; j < n; j++) acc = acc + L[j][i] * x[j];
            x[i] = (y[i] - acc) / L[i][i];
        }
        for (int i = 0; i < n; i++) inv[col * n + i] = x[i];
    }
}

// Gauss-Legendre points on [-1/2, 1/2] and weights summing to one
// (GP_init.f90:45-83): rules up to 3 points are binary128 expressions, the
// 4- and 5-point rules are double expressions, as in the reference.
void gauss_rule(int ngp, f128* pt, double* w) {
    const f128 s3 = sqrtf128((f128)3), s35 = sqrtf128((f128)3 / 5);
    const double s65 = sqrt(6. / 5), s30 = sqrt(30.), s107 = sqrt(10. / 7), s70 = sqrt(70.);
    const double third = 1. / 3;
    if (ngp == 1) {
        pt[0] = 0; w[0] = 1.0;
    } else if (ngp == 2) {
        pt[0] = -(f128)0.5 / s3; pt[1] = (f128)0.5 / s3;
        w[0] = w[1] = 0.5;
    } else if (ngp == 3) {
        pt[0] = -(f128)0.5 * s35; pt[1] = 0; pt[2] = (f128)0.5 * s35;
        w[0] = w[2] = 0.5 * 5. / 9;
        w[1] = 0.5 * 8. / 9;
    } else if (ngp == 4) {
        const double inner = 0.5 * sqrt(3. / 7 - (2. / 7) * s65);
        const double outer = 0.5 * sqrt(3. / 7 + (2. / 7) * s65);
        pt[0] = -outer; pt[1] = -inner; pt[2] = inner; pt[3] = outer;
        w[0] = w[3] = 0.5 * (1. / 36) * (18. - s30);
        w[1] = w[2] = 0.5 * (1. / 36) * (18. + s30);
    } else {
        const double inner = 0.5 * third * sqrt(5. - 2 * s107);
        const double outer = 0.5 * third * sqrt(5. + 2 * s107);
        pt[0] = -outer; pt[1] = -inner; pt[2] = 0.; pt[3] = inner; pt[4] = outer;
        w[0] = w[4] = 0.5 * (322. - 13 * s70) / 900;
        w[1] = w[3] = 0.5 * (322. + 13 * s70) / 900;
        w[2] = 0.5 * 128. / 225;
    }
}

}  // namespace

double gpm_cell_size(double length, int n) { return (double)((_Float128)length / n); }

// pol_presim (GP_init.f90:359-419): the third-order polynomial weights of
// POL_MOOD / Unlim_POL replace the order-3 GP weights, 2 Gauss points per
// face, over the 5-point stencil (M, L, T, R, B); o3_coef is constants.f90:61.
// Order 1 keeps the weight 1.
extern "C" void gpm_pol_weights(GpWeights* w) {
    const double c[5] = {15. / 18, 1. / 3, 1. / (4 * sqrt(3.)), -1. / (4 * sqrt(3.)), -1. / 6};
    // kM, kCloseNrm, kCloseTrans, kFarTrans, kFarNrm = 0..4; [face iL, iT, iR, iB][gauss point][stencil point]
    static const int k[4][2][5] = {{{0, 1, 3, 4, 2}, {0, 1, 2, 4, 3}},
                                   {{0, 2, 1, 3, 4}, {0, 3, 1, 2, 4}},
                                   {{0, 4, 3, 1, 2}, {0, 4, 2, 1, 3}},
                                   {{0, 2, 4, 3, 1}, {0, 3, 4, 2, 1}}};
    for (int f = 0; f < 4; f++)
        for (int g = 0; g < 2; g++) {
            for (int m = 0; m < 13; m++) w->zt[1][f][g][m] = 0.0;
            for (int m = 0; m < 5; m++) w->zt[1][f][g][m] = c[k[f][g][m]];
            w->zt[0][f][g][0] = 1.0;
        }
}

extern "C" int gpm_gp_presim(double ell_o_dx, double lx, double ly, int lf, int nf, int mord, int ngp,
                             GpWeights* out, double inv_err[3]) {
    if (!(mord == 1 || mord == 3 || mord == 5) || ngp < 1 || ngp > GPM_MAXGP || lf < 1 || nf < 1)
        return -1;
    memset(out, 0, sizeof(*out));
    for (int o = 0; o < 3; o++) inv_err[o] = 0.0;

    SeKernel k;
    k.hx = (f128)lx / lf;
    k.hy = (f128)ly / nf;
    k.ell = (f128)ell_o_dx * (k.hx < k.hy ? k.hx : k.hy);
    k.pi = 4 * atanf128((f128)1);
    k.inv_sqrt_pi = (f128)1 / sqrtf128(k.pi);
    k.sqrt2 = sqrtf128((f128)2);

    f128 pts[GPM_MAXGP];
    gauss_rule(ngp, pts, out->gw);

    for (int ord = 1; ord <= mord; ord += 2) {
        const int o = ord / 2, np = stencil_size(ord);
        f128 K[13 * 13], Ki[13 * 13];
        for (int a = 0; a < np; a++)
            for (int b = 0; b < np; b++)
                K[a * np + b] = k.cov((f128)(kStencil[a][0] - kStencil[b][0]),
                                      (f128)(kStencil[a][1] - kStencil[b][1]));
        spd_inverse(K, Ki, np);

        f128 worst = 0;  // max |K Ki - I|, the GP_init.f90:250 self-check
        for (int i = 0; i < np; i++)
            for (int j = 0; j < np; j++) {
                f128 s = 0;
                for (int m = 0; m < np; m++) s = s + K[i * np + m] * Ki[m * np + j];
                const f128 e = fabsf128(s - (i == j ? (f128)1 : (f128)0));
                if (e > worst) worst = e;
            }
        inv_err[o] = (double)worst;

        // Face centre offsets (cells) of faces iL, iT, iR, iB and the direction
        // along which the Gauss points run (0 = along y, 1 = along x).
        const f128 half = (f128)1 / 2;
        const f128 fc[4][2] = {{-half, 0}, {0, half}, {half, 0}, {0, -half}};
        const int along_x[4] = {0, 1, 0, 1};
        for (int face = 0; face < 4; face++)
            for (int g = 0; g < ngp; g++) {
                const f128 px = along_x[face] ? pts[g] : fc[face][0];
                const f128 py = along_x[face] ? fc[face][1] : pts[g];
                f128 t[13];
                for (int a = 0; a < np; a++) {
                    t[a] = k.pred1d((f128)kStencil[a][0] - px, k.hx);
                    t[a] = t[a] * k.pred1d((f128)kStencil[a][1] - py, k.hy);
                }
                double z[13];
                for (int b = 0; b < np; b++) {
                    f128 s = 0;
                    for (int a = 0; a < np; a++) s = s + t[a] * Ki[a * np + b];
                    z[b] = (double)s;
                }
                double sum = 0.0;
                for (int b = 0; b < np; b++) sum = sum + z[b];
                for (int b = 0; b < np; b++) out->zt[o][face][g][b] = z[b] / sum;
            }

        if (ord == 3) {
            f128 dx2[5], dy2[5];
            for (int a = 0; a < np; a++) {
                const f128 ox = (f128)kStencil[a][0], oy = (f128)kStencil[a][1];
                dx2[a] = k.pred1d_d2(ox, k.hx);
                dx2[a] = dx2[a] * k.pred1d(oy, k.hy);
                dy2[a] = k.pred1d_d2(oy, k.hy);
                dy2[a] = dy2[a] * k.pred1d(ox, k.hx);
            }
            for (int b = 0; b < np; b++) {
                f128 sx = 0, sy = 0;
                for (int a = 0; a < np; a++) {
                    sx = sx + dx2[a] * Ki[a * np + b];
                    sy = sy + dy2[a] * Ki[a * np + b];
                }
                out->d2x[b] = (double)sx;
                out->d2y[b] = (double)sy;
            }
        }
    }
    if (ngp == 3) {  // mirror-symmetric split of zt for the fast kernels
        for (int o = 0; o < 3; o++) {
            const int na = o == 2 ? 5 : (o == 1 ? 3 : 1), npair = o == 2 ? 4 : (o == 1 ? 1 : 0);
            for (int face = 0; face < 4; face++) {
                const int dir = (face == 0 || face == 2) ? 0 : 1;
                const double (*z)[13] = out->zt[o][face];
                GpSym& sy = out->sym[o][face];
                for (int k = 0; k < na; k++) {
                    sy.a0[k] = z[0][gpm_sym_axis(dir, k)];
                    sy.a1[k] = z[1][gpm_sym_axis(dir, k)];
                }
                for (int k = 0; k < npair; k++) {
                    const int m = gpm_sym_pair(dir, k, 0), mm = gpm_sym_pair(dir, k, 1);
                    sy.al[k] = 0.5 * (z[0][m] + z[0][mm]);
                    sy.be[k] = 0.5 * (z[0][m] - z[0][mm]);
                    sy.ga[k] = z[1][m];
                }
            }
        }
        // orbit components of the left (x) and bottom (y) faces at order 5;
        // stencil indices: 0 (0,0), 1 (-1,0), 2 (0,1), 3 (1,0), 4 (0,-1),
        // 5 (-1,-1), 6 (-1,1), 7 (1,1), 8 (1,-1), 9 (0,-2), 10 (-2,0), 11 (0,2), 12 (2,0)
        auto split = [](const double* z, double* c13) {
            const double za = z[5], zb = z[8], zc = z[6], zd = z[7];
            c13[0] = z[0];
            c13[1] = 0.5 * (z[1] + z[3]);
            c13[2] = 0.5 * (z[10] + z[12]);
            c13[3] = 0.5 * (z[4] + z[2]);
            c13[4] = 0.5 * (z[9] + z[11]);
            c13[5] = 0.25 * (za + zb + zc + zd);
            c13[6] = 0.5 * (z[1] - z[3]);
            c13[7] = 0.5 * (z[10] - z[12]);
            c13[8] = 0.25 * (za - zb + zc - zd);
            c13[9] = 0.5 * (z[4] - z[2]);
            c13[10] = 0.5 * (z[9] - z[11]);
            c13[11] = 0.25 * (za + zb - zc - zd);
            c13[12] = 0.25 * (za - zb - zc + zd);
        };
        double c[13];
        split(out->zt[2][0][0], out->orb.x0);
        split(out->zt[2][0][1], c);
        for (int k = 0; k < 9; k++) out->orb.x1[k] = c[k];  // y-symmetric: groups 3, 4 vanish
        split(out->zt[2][3][0], out->orb.y0);
        split(out->zt[2][3][1], c);
        for (int k = 0; k < 6; k++) out->orb.y1[k] = c[k];  // x-symmetric: groups 2, 4 vanish
        for (int k = 0; k < 3; k++) out->orb.y1[6 + k] = c[9 + k];
    }
    return 0;
}
