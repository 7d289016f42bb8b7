"""Initial conditions of the benchmark problems (gp-mood-code/IC.f90), in numpy.

Each builder fills cells lb..lf x nb..nf as InitialCdt does (IC.f90:29-30);
the caller applies Boundary_C afterwards (main.f90:125), e.g. with
Solver.Boundary_C.  The mesh starts at 0: x_l = l*dx - dx/2 (mesh_init.f90:14-20).
"""
from __future__ import annotations

import numpy as np

from .gpmood import NGC, padded

GAMMA = 1.4


def _mesh(lf, nf, lx, ly):
    dx = lx / lf
    dy = ly / nf
    l = np.arange(1 - NGC, lf + NGC + 1, dtype=np.float64)
    n = np.arange(1 - NGC, nf + NGC + 1, dtype=np.float64)
    return l * dx - dx / 2, n * dy - dy / 2, dx, dy


def p2c(r, u, v, p):
    """primitive_to_conservative, physics.f90:146-160."""
    r, u, v, p = np.broadcast_arrays(*(np.asarray(a, dtype=np.float64) for a in (r, u, v, p)))
    return np.stack([r, r * u, r * v, (p / (GAMMA - 1.)) + 0.5 * r * (u * u + v * v)], axis=-1)


def _fill(lf, nf, lx, ly, fn) -> np.ndarray:
    xs, ys, dx, dy = _mesh(lf, nf, lx, ly)
    U = padded(lf, nf)
    X, Y = np.meshgrid(xs[: lf + NGC], ys[: nf + NGC])
    U[: nf + NGC, : lf + NGC] = fn(X, Y, dx, dy)
    return U


def rp2d3(lf: int, nf: int, lx: float = 1.0, ly: float = 1.0) -> np.ndarray:
    """Four-quadrant Riemann problem 3 split at 0.8 (IC.f90:241-248)."""
    def fn(x, y, dx, dy):
        out = np.zeros(x.shape + (4,))
        for cond, st in (((x <= 0.8) & (y <= 0.8), (0.138, 1.206, 1.206, 0.029)),
                         ((x >= 0.8) & (y <= 0.8), (0.5323, 0.0, 1.206, 0.3)),
                         ((x <= 0.8) & (y >= 0.8), (0.5323, 1.206, 0.0, 0.3)),
                         ((x >= 0.8) & (y >= 0.8), (1.5, 0.0, 0.0, 1.5))):
            out[cond] = p2c(*st)
        return out
    return _fill(lf, nf, lx, ly, fn)


def riemann4(lf, nf, split, states, lx=1.0, ly=1.0) -> np.ndarray:
    """Generic four-quadrant problem; states = (BL, BR, TL, TR) primitive tuples."""
    sx, sy = split
    def fn(x, y, dx, dy):
        out = np.zeros(x.shape + (4,))
        for cond, st in (((x <= sx) & (y <= sy), states[0]), ((x >= sx) & (y <= sy), states[1]),
                         ((x <= sx) & (y >= sy), states[2]), ((x >= sx) & (y >= sy), states[3])):
            out[cond] = p2c(*st)
        return out
    return _fill(lf, nf, lx, ly, fn)


def sedov(lf: int, nf: int, lx: float = 1.0, ly: float = 1.0, e0: float = 1.0, rho0: float = 1.0,
          p0: float = 1.e-5) -> np.ndarray:
    """Point blast (f_sedov, IC.f90:358-373): E0 spread over cells within 3.5 dx."""
    def fn(x, y, dx, dy):
        m = min(dx, dy)
        dr2 = (3.5 * m) * (3.5 * m)
        pi = 4 * np.arctan(1.)
        r2 = (x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5)
        inner = np.sqrt(r2) < np.sqrt(dr2)
        p = np.where(inner, (1.4 - 1.) * e0 / (pi * dr2), p0)
        return p2c(rho0, 0.0, 0.0, p)
    return _fill(lf, nf, lx, ly, fn)


def dmr(lf: int, nf: int, lx: float = 4.0, ly: float = 1.0) -> np.ndarray:
    """Mach-10 oblique shock at x=1/6, 60 degrees (f_DMR, IC.f90:336-355)."""
    def fn(x, y, dx, dy):
        ymin = (x - 1. / 6) * np.sqrt(3.)
        post = y > ymin
        out = np.where(post[..., None], p2c(8., 7.1447096, -4.125, 116.5)[None, None, :],
                       p2c(1.4, 0.0, 0.0, 1.0)[None, None, :])
        return out
    return _fill(lf, nf, lx, ly, fn)


def isentropic_vortex(lf: int, nf: int, lx: float = 10.0, ly: float = 10.0, beta: float = 5.0) -> np.ndarray:
    """Isentropic vortex centred at (Lx/2, Ly/2), 5x5 Gauss cell averages
    (f_isentropic_vortex + quadrature, IC.f90:375-407,491-534)."""
    pi = 4 * np.arctan(1.)
    w = np.array([(322.0 - 13.0 * np.sqrt(70.0)) / 900.0, (322.0 + 13.0 * np.sqrt(70.0)) / 900.0, 128.0 / 225.0,
                  (322.0 + 13.0 * np.sqrt(70.0)) / 900.0, (322.0 - 13.0 * np.sqrt(70.0)) / 900.0])
    xg = np.array([-1.0 / 3.0 * np.sqrt(5.0 + 2.0 * np.sqrt(10.0 / 7.0)), -1.0 / 3.0 * np.sqrt(5.0 - 2.0 * np.sqrt(10.0 / 7.0)),
                   0.0, 1.0 / 3.0 * np.sqrt(5.0 - 2.0 * np.sqrt(10.0 / 7.0)), 1.0 / 3.0 * np.sqrt(5.0 + 2.0 * np.sqrt(10.0 / 7.0))])
    xc, yc = 0.5 * lx, 0.5 * ly

    def point(x, y):
        xp, yp = x.copy(), y.copy()
        while (xp < 0).any():
            xp = np.where(xp < 0, xp + 0.5 * lx, xp)
        while (yp < 0).any():
            yp = np.where(yp < 0, yp + 0.5 * ly, yp)
        r = np.sqrt((xp - xc) * (xp - xc) + (yp - yc) * (yp - yc))
        rho = (1. - (1.4 - 1.) * (beta * beta / (8 * 1.4 * pi * pi)) * np.exp(1. - r * r)) ** (1. / (1.4 - 1.))
        vx = 1. - 0.5 * (beta / pi) * np.exp(0.5 * (1. - r * r)) * (yp - xc)
        vy = 1. + 0.5 * (beta / pi) * np.exp(0.5 * (1. - r * r)) * (xp - yc)
        return p2c(rho, vx, vy, rho ** 1.4)

    def fn(x, y, dx, dy):
        acc = np.zeros(x.shape + (4,))
        lxh, lyh = 0.5 * dx, 0.5 * dy
        for j in range(5):
            for i in range(5):
                acc = acc + w[j] * w[i] * point(lxh * xg[i] + x, lyh * xg[j] + y)
        return (1. / (dx * dy)) * (acc * lxh * lyh)
    return _fill(lf, nf, lx, ly, fn)


def _seq(x, y, items):
    """Fortran's sequence of `if (cond) U = p2c(state)`: later matches overwrite
    earlier ones; cells that match none keep 0 (Boundary_C fills ghosts)."""
    out = np.zeros(x.shape + (4,))
    for cond, st in items:
        cond = np.broadcast_to(cond, x.shape)
        val = p2c(*[np.broadcast_to(np.asarray(a, dtype=np.float64), x.shape) for a in st])
        out[cond] = val[cond]
    return out


PI = 4 * np.arctan(1.)  # constants.f90:9


def _erf(a):
    from math import erf
    return np.vectorize(erf, otypes=[np.float64])(a)


def sod_x(lf, nf, lx=1.0, ly=1.0):
    """Sod tube along x (IC.f90:33-35)."""
    return _fill(lf, nf, lx, ly, lambda x, y, dx, dy: _seq(x, y, [
        (x < 0.5, (1., 0., 0., 1.)), (x >= 0.5, (0.125, 0., 0., 0.1))]))


def sod_y(lf, nf, lx=1.0, ly=1.0):
    """Sod tube along y (IC.f90:51-53)."""
    return _fill(lf, nf, lx, ly, lambda x, y, dx, dy: _seq(x, y, [
        (y < 0.5, (1., 0., 0., 1.)), (y >= 0.5, (0.125, 0., 0., 0.1))]))


def sod_xy(lf, nf, lx=1.0, ly=1.0):
    """Sod tube along the diagonal (IC.f90:59-61)."""
    def fn(x, y, dx, dy):
        cut = -x + (np.sqrt(2.) - 1)
        return _seq(x, y, [(y < cut, (1., 0., 0., 1.)), (y >= cut, (0.125, 0., 0., 0.1))])
    return _fill(lf, nf, lx, ly, fn)


def sod_rotated(lf, nf, lx=2 * np.sqrt(2.), ly=2 * np.sqrt(2.)):
    """Periodic train of Sod tubes at 45 degrees (IC.f90:40-48)."""
    def fn(x, y, dx, dy):
        xp = x * np.cos(PI / 4) + y * np.sin(PI / 4)
        left = (xp < 0.5) | ((1.5 < xp) & (xp <= 2.5)) | ((3.5 < xp) & (xp < 4))
        return _seq(x, y, [(left, (1., 0., 0., 1.)), (~left, (0.125, 0., 0., 0.1))])
    return _fill(lf, nf, lx, ly, fn)


def slow_shock(lf, nf, lx=30.0, ly=1.0):
    """Slow-moving shock (LeVeque p. 348; IC.f90:37-40)."""
    return _fill(lf, nf, lx, ly, lambda x, y, dx, dy: _seq(x, y, [
        (x < 15., (5.6698, -1.4701, 0.0, 100.0)), (x >= 15., (1.0, -2.315811, 0.0, 1.0))]))


def lax(lf, nf, lx=2.0, ly=1.0):
    """Lax problem (IC.f90:55-57)."""
    return _fill(lf, nf, lx, ly, lambda x, y, dx, dy: _seq(x, y, [
        (x < 1., (0.445, 0.698, 0., 3.528)), (x >= 1., (0.5, 0., 0., 0.571))]))


def shu_osher(lf, nf, lx=9.0, ly=1.0):
    """Shu-Osher shock/entropy-wave problem (IC.f90:64-66); pair with the Dirichlet BC (19)."""
    def fn(x, y, dx, dy):
        return _seq(x, y, [(x <= 0.5, (3.857143, 2.629369, 0., 10.33333)),
                           (x > 0.5, (1. + 0.2 * np.sin(5 * (x - 4.5)), 0., 0., 1.))])
    return _fill(lf, nf, lx, ly, fn)


def shu_osher_rotated(lf, nf, lx=10 * 2 * np.sqrt(2.), ly=10 * 2 * np.sqrt(2.)):
    """Shu-Osher at 45 degrees (IC.f90:68-80)."""
    def fn(x, y, dx, dy):
        xp = x * np.cos(PI / 4) + y * np.sin(PI / 4)
        pre = (xp <= 1.0) | ((11. < xp) & (xp <= 21.)) | ((31. < xp) & (xp < 40.))
        return _seq(x, y, [(pre, (3.857143, 2.629369 * np.cos(PI / 4.), 2.629369 * np.sin(PI / 4.), 10.33333)),
                           (~pre, (1. + 0.2 * np.sin(5 * xp), 0., 0., 1.))])
    return _fill(lf, nf, lx, ly, fn)


def strong_rarefaction(lf, nf, lx=1.0, ly=1.0):
    """Two strong rarefactions (IC.f90:83-85)."""
    return _fill(lf, nf, lx, ly, lambda x, y, dx, dy: _seq(x, y, [
        (x <= 0.5, (1., -2., 0., 0.4)), (x > 0.5, (1., 2., 0., 0.4))]))


def blast(lf, nf, lx=1.0, ly=1.0):
    """Woodward-Colella blast waves (IC.f90:88-91); pair with reflective BCs."""
    return _fill(lf, nf, lx, ly, lambda x, y, dx, dy: _seq(x, y, [
        (x >= 0., (1., 0., 0., 1000.)), (x >= 0.1, (1., 0., 0., 0.1)), (x >= 0.9, (1., 0., 0., 100.))]))


def lin_gauss_x(lf, nf, lx=1.0, ly=1.0):
    """Advected Gaussian density, exact cell averages along x (IC.f90:95-107)."""
    def fn(x, y, dx, dy):
        a = -0.0886227 * _erf(5. - 10. * (x + dx / 2)) + 0.0886227 * _erf(5. - 10. * (x - dx / 2)) + dx
        return p2c(a / dx, 1., 0., 1. / GAMMA)
    return _fill(lf, nf, lx, ly, fn)


def _gauss_xy_avg(x, y, dx, dy):
    a = -0.0886227 * _erf(-5 * dx - 10 * x + 5.) + 0.0886227 * _erf(5 * dx - 10 * x + 5)
    a = a * (-0.0886227 * _erf(-5 * dy - 10 * y + 5.) + 0.0886227 * _erf(5 * dy - 10 * y + 5))
    return (a + dx * dy) / (dx * dy)


def lin_gauss_y(lf, nf, lx=1.0, ly=1.0):
    """Advected 2-D Gaussian moving in -y (IC.f90:109-123)."""
    return _fill(lf, nf, lx, ly, lambda x, y, dx, dy: p2c(_gauss_xy_avg(x, y, dx, dy), 0., -1., 1. / GAMMA))


def lin_gauss_xy(lf, nf, lx=1.0, ly=1.0):
    """Advected 2-D Gaussian moving in +x (the second assignment of IC.f90:126-138 stands)."""
    return _fill(lf, nf, lx, ly, lambda x, y, dx, dy: p2c(_gauss_xy_avg(x, y, dx, dy), 1., 0., 1. / GAMMA))


def implosion(lf, nf, lx=0.3, ly=0.3):
    """Implosion in a box (f_implosion, IC.f90:293-310); reflective BCs."""
    def fn(x, y, dx, dy):
        xx = x + dx * np.sqrt(2.) * 0.5
        yy = y + dy * np.sqrt(2.) * 0.5
        out = yy + xx > 0.15
        return _seq(x, y, [(out, (1., 0., 0., 1.)), (~out, (0.125, 0., 0., 0.14))])
    return _fill(lf, nf, lx, ly, fn)


def explosion(lf, nf, lx=1.5, ly=1.5):
    """Cylindrical explosion (f_explosion, IC.f90:312-326), evaluated at
    (x_l, y_n) below the diagonal and at (x_n, y_l) on and above it, as the
    reference's loop does (IC.f90:144-146; square grids)."""
    if lf != nf:
        raise ValueError("explosion indexes mesh_x by n: use a square grid")
    xs, ys, dx, dy = _mesh(lf, nf, lx, ly)
    U = padded(lf, nf)
    m = lf + NGC
    L, N = np.meshgrid(np.arange(m), np.arange(m))  # array indices of l, n
    X = np.where(N < L, xs[L], xs[N])
    Y = np.where(N < L, ys[N], ys[L])
    rad = np.sqrt(X ** 2 + Y ** 2)
    inner = rad < 0.4
    U[:m, :m] = _seq(X, Y, [(inner, (1., 0., 0., 1.)), (~inner, (0.125, 0., 0., 0.1))])
    return U


def _quadrants(lf, nf, lx, ly, rules):
    return _fill(lf, nf, lx, ly, lambda x, y, dx, dy: _seq(x, y, [(c(x, y), st) for c, st in rules]))


def rp2d4(lf, nf, lx=1.0, ly=1.0):
    """Four-quadrant Riemann problem 4 (f_RP_2D_4, IC.f90:251-258)."""
    return _quadrants(lf, nf, lx, ly, [
        (lambda x, y: (x <= 0.5) & (y <= 0.5), (1.1, 0.8939, 0.8939, 1.1)),
        (lambda x, y: (x >= 0.5) & (y <= 0.5), (0.5065, 0.0, 0.8939, 0.35)),
        (lambda x, y: (x <= 0.5) & (y >= 0.5), (0.5065, 0.8939, 0.0, 0.35)),
        (lambda x, y: (x >= 0.5) & (y >= 0.5), (1.1, 0.0, 0.0, 1.1))])


def rp2d6(lf, nf, lx=1.0, ly=1.0):
    """Four-quadrant Riemann problem 6 (f_RP_2D_6, IC.f90:260-269)."""
    return _quadrants(lf, nf, lx, ly, [
        (lambda x, y: (x <= 0.5) & (y >= 0.5), (2.0, 0.75, 0.5, 1.0)),
        (lambda x, y: (x >= 0.5) & (y >= 0.5), (1.0, 0.75, -0.5, 1.0)),
        (lambda x, y: (x <= 0.5) & (y <= 0.5), (1.0, -0.75, 0.5, 1.0)),
        (lambda x, y: (x >= 0.5) & (y <= 0.5), (3.0, -0.75, -0.5, 1.0))])


def rp2d12(lf, nf, lx=1.0, ly=1.0):
    """Four-quadrant Riemann problem 12 (f_RP_2D_12, IC.f90:271-280; note its strict x > 0.5, x < 0.5)."""
    return _quadrants(lf, nf, lx, ly, [
        (lambda x, y: (x <= 0.5) & (y <= 0.5), (0.8, 0.0, 0.0, 1.0)),
        (lambda x, y: (x > 0.5) & (y <= 0.5), (1.0, 0.0, 0.7276, 1.0)),
        (lambda x, y: (x < 0.5) & (y >= 0.5), (1.0, 0.7276, 0.0, 1.0)),
        (lambda x, y: (x >= 0.5) & (y >= 0.5), (0.5313, 0.0, 0.0, 0.4))])


def rp2d15(lf, nf, lx=1.0, ly=1.0):
    """Four-quadrant Riemann problem 15 (f_RP_2D_15, IC.f90:283-291)."""
    return _quadrants(lf, nf, lx, ly, [
        (lambda x, y: (x <= 0.5) & (y <= 0.5), (0.8, 0.1, -0.3, 0.4)),
        (lambda x, y: (x >= 0.5) & (y <= 0.5), (0.5313, 0.1, 0.4276, 0.4)),
        (lambda x, y: (x <= 0.5) & (y >= 0.5), (0.5197, -0.6259, -0.3, 0.4)),
        (lambda x, y: (x >= 0.5) & (y >= 0.5), (1.0, 0.1, -0.3, 1.0))])


def rp2d17(lf, nf, lx=1.0, ly=1.0):
    """Four-quadrant Riemann problem 17 (f_RP_2D_17, IC.f90:293-302)."""
    return _quadrants(lf, nf, lx, ly, [
        (lambda x, y: (x <= 0.5) & (y <= 0.5), (1.0625, 0.0, 0.2145, 0.4)),
        (lambda x, y: (x >= 0.5) & (y <= 0.5), (0.5197, 0.0, -1.1259, 0.4)),
        (lambda x, y: (x <= 0.5) & (y >= 0.5), (2.0, 0.0, -0.3, 1.0)),
        (lambda x, y: (x >= 0.5) & (y >= 0.5), (1.0, 0.0, -0.4, 1.0))])


def mach800(lf, nf, lx=1.5, ly=1.5, double=False):
    """Mach-800 jet(s) (IC.f90:170-190); pair with the Mach800 (201) or
    DoubleMach800 (301) BC.  The double version has an ambient density falling
    linearly from 14 to 0.14 across the domain and no jet cells in the IC."""
    def fn(x, y, dx, dy):
        if double:
            dens = (0.14 - 14.) / ly * y + 14.
        else:
            dens = np.full(x.shape, 14.)
        items = [(np.ones(x.shape, bool), (dens, 0.0, 0.0, 1.0))]
        if not double:
            items.append(((np.abs(x - 0.5 * lx) <= 0.05) & (y < dy), (1.4, 0.0, 800.0, 1.0)))
        return _seq(x, y, items)
    return _fill(lf, nf, lx, ly, fn)


def rmi(lf, nf, lx=6.0, ly=1.0):
    """Richtmyer-Meshkov: Mach-2 shock at x = 0.8 hitting an interface at
    x = y + 1 (f_rmi with sim_posn = y + 1, IC.f90:192-204,409-467); pair with the RMI BC (401)."""
    def fn(x, y, dx, dy):
        gam, mach2 = 1.4, 2. * 2.
        gamp, gamm = gam + 1., gam - 1.
        post = (1. * (gamp * mach2) / (gamm * mach2 + 2.0), 2. * np.sqrt(gam * 1. / 1.), 0.,
                1. * (2.0 * gam * mach2 - gamm) / gamp)
        posn = y + 1.0
        return _seq(x, y, [(x < 0.8, post), ((x >= 0.8) & (x < posn), (1., 0., 0., 1.)),
                           (~(x < 0.8) & ~((x >= 0.8) & (x < posn)), (3., 0., 0., 1.))])
    return _fill(lf, nf, lx, ly, fn)


def rt(lf, nf, lx=0.25, ly=1.0):
    """Rayleigh-Taylor (f_RT, IC.f90:469-489; its constants are real(4)); pair
    with the RT BC (402).  The reference has no gravity source term, only the
    hydrostatic ghost cells."""
    f32 = lambda v: float(np.float32(v))
    def fn(x, y, dx, dy):
        dens = np.where(y < ly / 2, f32(1), f32(2))
        pres = f32(5.0 / 2) + f32(0.1) * y
        vy = f32(0.01) * (1 + np.cos(2 * PI * (x - lx / 2) / lx)) * (1 + np.cos(2 * PI * (y - ly / 2) / ly)) / 4
        return p2c(dens, 0.0, vy, pres)
    return _fill(lf, nf, lx, ly, fn)


def kelvin_helmholtz(lf, nf, lx=1.0, ly=1.0, seed=0):
    """Kelvin-Helmholtz shear layer with Box-Muller noise (IC.f90:206-216,218-226);
    pair with the KH BC (403).  The reference seeds from the clock; here the
    noise comes from a seeded generator."""
    rng = np.random.default_rng(seed)
    def fn(x, y, dx, dy):
        def normal():
            u1, u2 = rng.random(x.shape), rng.random(x.shape)
            u1 = np.where(u1 > 0, u1, np.finfo(float).tiny)
            return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * 3.14159265358979323846 * u2)
        env = np.exp(-((y - 0.5) / 0.1) ** 2)
        r1, r2 = normal() * env, normal() * env
        low = y <= 0.5
        return _seq(x, y, [(low, (2., 0.5 + r1, r2, 2.5)), (~low, (1., -0.5 + r1, r2, 2.5))])
    return _fill(lf, nf, lx, ly, fn)


BATCH_SIZES = (64, 96, 128, 192, 256)


def random_riemann(seed: int, sizes=BATCH_SIZES):
    """One problem of the batched workload: a four-quadrant Riemann problem on
    [0,1]^2 whose quadrant states (rho ~ U[0.1,2], p ~ U[0.02,2],
    u, v ~ U[-1.5,1.5]), split point (~ U[0.3,0.8]^2) and square grid size
    (uniform over ``sizes``) are drawn from numpy's PCG64 seeded with ``seed``."""
    rng = np.random.default_rng(seed)
    n = int(sizes[rng.integers(len(sizes))])
    split = tuple(rng.uniform(0.3, 0.8, size=2))
    states = []
    for _ in range(4):
        r = rng.uniform(0.1, 2.0)
        u, v = rng.uniform(-1.5, 1.5, size=2)
        p = rng.uniform(0.02, 2.0)
        states.append((r, u, v, p))
    return riemann4(n, n, split, states), n
