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
