"""FP64 PyTorch autograd reference of GP-MOOD steps with frozen MOOD order masks.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA adjoint (gpmood_adj_*).
Only tests/ use it.  Every operation is a differentiable torch op on float64
tensors, so ``torch.autograd`` gives the exact Jacobian-transpose products of
the same map that the hand-written CUDA adjoint transposes.

The map, restated from the reference:
  Boundary_C for Neumann / periodic / reflective   BC.f90:10-421
  GP face states at the face order min(CellGPO)    mod_GP_MOOD.f90:58-65, mod_FE.f90:80-98
  HLLC_Flux with Gauss quadrature                  mod_HLLC.f90:11-169, mod_FE.f90:80-98
  flux-difference update                           mod_FE.f90:75-145
  SSP_RK3                                          mod_SSP_RK3.f90:12-39
States are interior tensors I[n, l, k] (nf, lf, 4); padded tensors carry the
4 ghost layers of the reference's U(4, lb:le, nb:ne) as (nf+8, lf+8, 4).
"""
from __future__ import annotations

import numpy as np
import torch

NGC = 4
GAMMA = 1.4
# Diamond stencil offsets (ox, oy) in GP_init.f90:97-138 order.
STENCIL = ((0, 0), (-1, 0), (0, 1), (1, 0), (0, -1), (-1, -1), (-1, 1), (1, 1), (1, -1), (0, -2), (-2, 0), (0, 2),
           (2, 0))
NP = (1, 5, 13)


def _ghost_map(n: int, bc: int):
    """Source index (0-based interior) and sign of every padded index along one axis."""
    src, sgn = [], []
    for i in range(1 - NGC, n + NGC + 1):
        if 1 <= i <= n:
            s, m = i, 1.0
        elif bc == 17:
            s, m = (1 if i <= 0 else n), 1.0
        elif bc == 18:
            s, m = (i + n if i <= 0 else i - n), 1.0
        elif bc == 20:
            s, m = (1 - i if i <= 0 else 2 * n + 1 - i), -1.0
        else:
            raise ValueError(f"BC_type {bc} has no adjoint reference")
        src.append(s - 1)
        sgn.append(m)
    return src, sgn


def boundary(I: torch.Tensor, bc: int) -> torch.Tensor:
    """Padded state whose ghosts are Boundary_C of the interior I."""
    nf, lf, _ = I.shape
    sx, gx = _ghost_map(lf, bc)
    sy, gy = _ghost_map(nf, bc)
    dev = I.device
    X = I.index_select(1, torch.tensor(sx, device=dev))
    fx = torch.ones(len(sx), 4, dtype=I.dtype, device=dev)
    fx[:, 1] = torch.tensor(gx, dtype=I.dtype, device=dev)  # mirror flips rho*u on x ghosts
    X = X * fx[None]
    Y = X.index_select(0, torch.tensor(sy, device=dev))
    fy = torch.ones(len(sy), 4, dtype=I.dtype, device=dev)
    fy[:, 2] = torch.tensor(gy, dtype=I.dtype, device=dev)
    return Y * fy[:, None]


def _c2p(u, d):
    r, mx, my, e = u.unbind(-1)
    vx, vy = mx / r, my / r
    p = (GAMMA - 1.) * (e - (0.5 * (mx * mx + my * my) / r))
    c = torch.sqrt(GAMMA * p / r)
    vn, vt = (vx, vy) if d == 0 else (vy, vx)
    return vn, vt, p, c


def _flux(u, vn, p, d):
    r, mx, my, e = u.unbind(-1)
    if d == 0:
        return torch.stack([mx, r * vn * vn + p, my * vn, vn * (e + p)], -1)
    return torch.stack([my, mx * vn, r * vn * vn + p, vn * (e + p)], -1)


def hllc(uL, uR, d):
    """HLLC_Flux (mod_HLLC.f90:11-169) of admissible states, direction d."""
    vnL, vtL, pL, cL = _c2p(uL, d)
    vnR, vtR, pR, cR = _c2p(uR, d)
    SL = torch.minimum(vnL - cL, vnR - cR)
    SR = torch.maximum(vnL + cL, vnR + cR)
    FL, FR = _flux(uL, vnL, pL, d), _flux(uR, vnR, pR, d)
    aL, aR = uL[..., 0] * (SL - vnL), uR[..., 0] * (SR - vnR)
    us = uL[..., 0] * vnL * (SL - vnL) - uR[..., 0] * vnR * (SR - vnR)
    us = ((pR - pL) + us) / (aL - aR)

    def star(u, F, vn, vt, p, S, a):
        dS = a / (S - us)
        one = torch.ones_like(us)
        st = [one, us, vt] if d == 0 else [one, vt, us]
        st.append(u[..., 3] / u[..., 0] + (us - vn) * (us + p / a))
        st = torch.stack(st, -1)
        return F + S[..., None] * (st * dS[..., None] - u)

    FsL = star(uL, FL, vnL, vtL, pL, SL, aL)
    FsR = star(uR, FR, vnR, vtR, pR, SR, aR)
    left = ((SL < 0) & (us >= 0))[..., None]
    right = ((us < 0) & (SR >= 0))[..., None]
    F = torch.where(left, FsL, torch.where(right, FsR, FR))
    return torch.where((SL >= 0)[..., None], FL, F)


def _face_states(X, zt, side_face, oi, ngp, sl_y, sl_x):
    """sum_m z[oi][face][g][m] * X[y+oy, x+ox] for a block of cells (slices of the padded grid)."""
    out = []
    for g in range(ngp):
        acc = None
        for m in range(NP[oi]):
            ox, oy = STENCIL[m]
            blk = X[sl_y.start + oy:sl_y.stop + oy, sl_x.start + ox:sl_x.stop + ox]
            term = float(zt[oi, side_face, g, m]) * blk
            acc = term if acc is None else acc + term
        out.append(acc)
    return out


def face_flux(X, order, zt, gw, ngp, d):
    """Quadrature flux of every x (d=0) or y (d=1) face at order min(CellGPO) of its two cells."""
    ny, nx, _ = X.shape
    lf, nf = nx - 2 * NGC, ny - 2 * NGC
    if d == 0:   # low cells l = 0..lf, n = 1..nf (padded columns 3..lf+3, rows 4..nf+3)
        lo_y, lo_x = slice(4, nf + 4), slice(3, lf + 4)
        hi_y, hi_x = slice(4, nf + 4), slice(4, lf + 5)
        fl, fh = 2, 0
    else:        # low cells l = 1..lf, n = 0..nf
        lo_y, lo_x = slice(3, nf + 4), slice(4, lf + 4)
        hi_y, hi_x = slice(4, nf + 5), slice(4, lf + 4)
        fl, fh = 1, 3
    o = torch.minimum(order[lo_y, lo_x], order[hi_y, hi_x])
    # Faces of another order get the cell averages as stand-in states, so that
    # no inadmissible unselected state puts a NaN into the gradient.
    cL, cR = X[lo_y, lo_x], X[hi_y, hi_x]
    F = None
    for oi, ordv in enumerate((1, 3, 5)):
        sel = (o == ordv)[..., None]
        if not bool(sel.any()):
            continue
        uL = _face_states(X, zt, fl, oi, ngp, lo_y, lo_x)
        uR = _face_states(X, zt, fh, oi, ngp, hi_y, hi_x)
        Fo = None
        for g in range(ngp):
            term = hllc(torch.where(sel, uL[g], cL), torch.where(sel, uR[g], cR), d) * float(gw[g])
            Fo = term if Fo is None else Fo + term
        Fo = torch.where(sel, Fo, torch.zeros_like(Fo))
        F = Fo if F is None else F + Fo
    return F


def stage(I, order, dt, dx, dy, zt, gw, ngp, bc):
    """One Forward_Euler stage at frozen orders: interior in, interior out."""
    X = boundary(I, bc)
    Fx = face_flux(X, order, zt, gw, ngp, 0)   # (nf, lf+1, 4)
    Fy = face_flux(X, order, zt, gw, ngp, 1)   # (nf+1, lf, 4)
    qx, qy = dt / dx, dt / dy
    return I + qy * Fy[:-1] + qx * Fx[:, :-1] - qx * Fx[:, 1:] - qy * Fy[1:]


def steps(I0, orders, dts, dx, dy, zt, gw, ngp, bc):
    """SSP_RK3 steps with frozen orders[step][stage] (padded int tensors) and dts[step]."""
    I = I0
    for s, dt in enumerate(dts):
        o0, o1, o2 = orders[s]
        I1 = stage(I, o0, dt, dx, dy, zt, gw, ngp, bc)
        I2 = 0.75 * I + 0.25 * stage(I1, o1, dt, dx, dy, zt, gw, ngp, bc)
        I = (1. / 3) * I + (2. / 3) * stage(I2, o2, dt, dx, dy, zt, gw, ngp, bc)
    return I


def weights(gp) -> tuple[np.ndarray, np.ndarray]:
    """(zt[3][4][5][13], gauss weights[5]) from the oracle's GP precompute struct."""
    return np.array(gp.zt, dtype=np.float64).reshape(3, 4, 5, 13), np.array(gp.gauss_w, dtype=np.float64)
