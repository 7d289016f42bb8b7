"""GP weight precompute (GP_init.f90:26-357): the oracle pinned by the
reference's own inversion self-check and by an independent mpmath derivation,
and the product's host precompute checked bit for bit against the oracle."""
from __future__ import annotations

import numpy as np
import pytest

STENCIL = [(0, 0), (-1, 0), (0, 1), (1, 0), (0, -1), (-1, -1), (-1, 1), (1, 1), (1, -1), (0, -2), (-2, 0), (0, 2),
           (2, 0)]


def weights(oracle, **kw):
    p = oracle.make_params(kw.pop("lf", 256), kw.pop("nf", 256), **kw)
    g = oracle.gp_weights(p)
    return p, np.array(g.zt).reshape(3, 4, 5, 13), np.array(g.d2x), np.array(g.d2y), np.array(g.inv_err)


@pytest.mark.parametrize("ell", [12.0, 6.0, 3.0])
def test_inversion_selfcheck(oracle, ell):
    # GP_init.f90:250: "Error in the inversion of the main kernel matrix ... must be close to 0"
    _, _, _, _, err = weights(oracle, ell_o_dx=ell)
    assert err[0] < 1e-32
    assert err[1] < 1e-26
    assert err[2] < 1e-20


@pytest.mark.parametrize("ngp", [1, 2, 3, 4, 5])
def test_weights_normalised_and_mirrored(oracle, ngp):
    _, zt, _, _, _ = weights(oracle, ngp=ngp)
    for o, npt in ((0, 1), (1, 5), (2, 13)):
        for f in range(4):
            for g in range(ngp):
                assert abs(zt[o, f, g, :npt].sum() - 1.0) < 1e-14
    # iL is the mirror image of iR under x -> -x, with Gauss points unchanged.
    mirror = [STENCIL.index((-x, y)) for (x, y) in STENCIL]
    o = 2
    for g in range(ngp):
        np.testing.assert_allclose(zt[o, 0, g, :13], zt[o, 2, g, mirror], rtol=1e-12, atol=1e-14)
    assert zt[0, 0, 0, 0] == 1.0


def test_gauss_weights(oracle):
    p = oracle.make_params(64, 64, ngp=3)
    g = oracle.gp_weights(p)
    assert list(g.gauss_w)[:3] == [0.5 * 5. / 9, 0.5 * 8. / 9, 0.5 * 5. / 9]


def _mp_weights(ell_o_dx, ngp):
    """zT and d2 weights from first principles in 60-digit arithmetic: cell
    integrals of the SE kernel by mpmath.quad, a linear solve, and second
    derivatives by mpmath.diff (independent of the closed forms of GP_init.f90)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 60
    s = mp.mpf(ell_o_dx)  # length scale in cells (dx = dy)

    def k1(d):  # integral over two unit cells at separation d of exp(-(u-v)^2/(2 s^2))
        return mp.quad(lambda u: mp.quad(lambda v: mp.exp(-((u - v + d) ** 2) / (2 * s * s)), [-0.5, 0.5]), [-0.5, 0.5])

    def t1(x):  # point at offset x from a unit cell's centre, against the cell average
        return mp.quad(lambda u: mp.exp(-((x - u) ** 2) / (2 * s * s)), [-0.5, 0.5])

    k1c = {d: k1(d) for d in range(-4, 5)}
    if ngp == 3:
        pts = [-mp.sqrt(mp.mpf(3) / 5) / 2, mp.mpf(0), mp.sqrt(mp.mpf(3) / 5) / 2]
    else:
        pts = [-1 / (2 * mp.sqrt(3)), 1 / (2 * mp.sqrt(3))]
    out = {}
    for o, npt in ((1, 5), (2, 13)):
        st = STENCIL[:npt]
        K = mp.matrix(npt, npt)
        for a in range(npt):
            for b in range(npt):
                K[a, b] = k1c[st[a][0] - st[b][0]] * k1c[st[a][1] - st[b][1]]
        for face, (fx, fy, alongx) in enumerate(((-0.5, 0, False), (0, 0.5, True), (0.5, 0, False), (0, -0.5, True))):
            for g, gp in enumerate(pts):
                px, py = (gp, fy) if alongx else (fx, gp)
                T = mp.matrix([t1(st[a][0] - px) * t1(st[a][1] - py) for a in range(npt)])
                z = mp.lu_solve(K, T)  # K symmetric: T^T K^-1 = (K^-1 T)^T
                tot = sum(z)
                out[(o, face, g)] = [float(z[i] / tot) for i in range(npt)]
        if o == 1:
            d2 = []
            for a in range(npt):
                cx, cy = st[a]
                d2.append(mp.diff(lambda x: t1(cx - x), 0, 2) * t1(cy))
            zx = mp.lu_solve(K, mp.matrix(d2))
            out["d2x_cells"] = [float(v) for v in zx]
    return out


@pytest.mark.parametrize("ngp", [2, 3])
def test_weights_match_mpmath(oracle, ngp):
    lf = 64
    _, zt, d2x, _, _ = weights(oracle, lf=lf, nf=lf, ngp=ngp, ell_o_dx=12.0)
    ref = _mp_weights(12.0, ngp)
    worst = 0.0
    for (o, face, g), z in ((k, v) for k, v in ref.items() if isinstance(k, tuple)):
        got = zt[o, face, g, : len(z)]
        worst = max(worst, float(np.max(np.abs(got - np.array(z)))))
    # The R2 system is ill conditioned (cond ~ 1e24 at ell = 12 dx); the
    # reference's binary128 inverse still gives every weight to ~1e-9 absolute.
    assert worst < 1e-8, worst
    # Second derivatives: the mpmath value is per cell^2; the reference's is per length^2.
    dx = 1.0 / lf
    np.testing.assert_allclose(d2x, np.array(ref["d2x_cells"]) / dx ** 2, rtol=1e-7)


@pytest.mark.parametrize("knobs", [dict(), dict(ngp=2, mord=3), dict(ell_o_dx=6.0, ngp=5),
                                   dict(lf=96, nf=64, lx=4.0, ly=1.0, ngp=4), dict(lf=128, nf=128, lx=10., ly=10.)])
def test_product_weights_bitwise(oracle, pkg, knobs):
    """The library's own binary128 precompute gives the oracle's doubles exactly."""
    kw = dict(knobs)
    lf, nf = kw.pop("lf", 256), kw.pop("nf", 256)
    p, zt, d2x, d2y, err = weights(oracle, lf=lf, nf=nf, **kw)
    from gpmood_gb300.gpmood import default_params, gp_weights
    pp = default_params(lf=lf, nf=nf, **kw)
    zt_p, d2_p, err_p = gp_weights(pp)
    ngp = pp.ngp
    for o, npt in ((0, 1), (1, 5), (2, 13)):
        if 2 * o + 1 > pp.mord:
            continue
        assert np.array_equal(zt_p[o, :, :, :npt], zt[o, :, :ngp, :npt])
    if pp.mord >= 3:
        assert np.array_equal(d2_p[0], d2x) and np.array_equal(d2_p[1], d2y)
    np.testing.assert_allclose(err_p, err, rtol=0, atol=1e-30)
