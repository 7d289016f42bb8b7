#!/usr/bin/env python
"""Generate the golden fixtures of tests/golden/ (run from the repository root):

  python tests/golden/make_golden.py

* gp_weights_mpmath.npz -- zT weights of the R1 (5-point) and R2 (13-point)
  stencils at ell = 12 dx for ngp = 2 and 3, and the R1 second-derivative
  weights, derived in 60-digit arithmetic by mpmath from first principles
  (cell integrals of the SE kernel by quadrature, a linear solve,
  differentiation by mpmath.diff), independent of the closed forms of
  gp-mood-code/GP_init.f90 that the oracle and the library restate.
* oracle_steps.npz -- states, time steps and per-stage MOOD order masks of
  the CPU oracle on four small problems after a few steps: 2DRP3 32^2
  (Neumann), Sedov 32^2 (reflecting), isentropic vortex 32^2 (periodic) and
  DMR 48x12 (DMR boundaries).  The oracle must keep reproducing them bit for
  bit and the CUDA exact mode must equal them; the reference itself cannot
  run on these machines (no Fortran compiler), so these pin the restatement
  against drift rather than against a reference run.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "oracle"))

STENCIL = [(0, 0), (-1, 0), (0, 1), (1, 0), (0, -1), (-1, -1), (-1, 1), (1, 1), (1, -1), (0, -2), (-2, 0), (0, 2),
           (2, 0)]

CASES = {
    # name: (ic, lf, nf, knobs, steps)
    "rp2d3": ("rp2d3", 32, 32, dict(bc=17, tmax=0.8), 6),
    "sedov": ("sedov", 32, 32, dict(bc=20, tmax=0.05), 6),
    "vortex": ("vortex", 32, 32, dict(bc=18, lx=10.0, ly=10.0, tmax=1.0), 6),
    "dmr": ("dmr", 48, 12, dict(bc=35, lx=4.0, ly=1.0, tmax=0.2), 4),
}


def mp_weights(ell_o_dx: float, ngp: int) -> dict:
    import mpmath as mp
    mp.mp.dps = 60
    s = mp.mpf(ell_o_dx)

    def k1(d):
        return mp.quad(lambda u: mp.quad(lambda v: mp.exp(-((u - v + d) ** 2) / (2 * s * s)), [-0.5, 0.5]),
                       [-0.5, 0.5])

    def t1(x):
        return mp.quad(lambda u: mp.exp(-((x - u) ** 2) / (2 * s * s)), [-0.5, 0.5])

    k1c = {d: k1(d) for d in range(-4, 5)}
    if ngp == 3:
        pts = [-mp.sqrt(mp.mpf(3) / 5) / 2, mp.mpf(0), mp.sqrt(mp.mpf(3) / 5) / 2]
    else:
        pts = [-1 / (2 * mp.sqrt(3)), 1 / (2 * mp.sqrt(3))]
    zt = np.zeros((3, 4, ngp, 13))
    zt[0, :, :, 0] = 1.0
    d2x = None
    for o, npt in ((1, 5), (2, 13)):
        st = STENCIL[:npt]
        K = mp.matrix(npt, npt)
        for a in range(npt):
            for b in range(npt):
                K[a, b] = k1c[st[a][0] - st[b][0]] * k1c[st[a][1] - st[b][1]]
        for face, (fx, fy, alongx) in enumerate(((-0.5, 0, False), (0, 0.5, True), (0.5, 0, False),
                                                 (0, -0.5, True))):
            for g, gp in enumerate(pts):
                px, py = (gp, fy) if alongx else (fx, gp)
                T = mp.matrix([t1(st[a][0] - px) * t1(st[a][1] - py) for a in range(npt)])
                z = mp.lu_solve(K, T)
                tot = sum(z)
                zt[o, face, g, :npt] = [float(z[i] / tot) for i in range(npt)]
        if o == 1:
            d2 = [mp.diff(lambda x, cx=cx: t1(cx - x), 0, 2) * t1(cy) for cx, cy in st]
            d2x = np.array([float(v) for v in mp.lu_solve(K, mp.matrix(d2))])  # per cell^2
    return {"zt": zt, "d2x_cells": d2x}


def main() -> int:
    import oracle as O
    O.build()
    w = {}
    for ngp in (2, 3):
        r = mp_weights(12.0, ngp)
        w[f"zt_ngp{ngp}"] = r["zt"]
        w[f"d2x_cells_ngp{ngp}"] = r["d2x_cells"]
    np.savez_compressed(HERE / "gp_weights_mpmath.npz", ell_o_dx=12.0, **w)

    out = {}
    for name, (ic, lf, nf, kn, nsteps) in CASES.items():
        p = O.make_params(lf, nf, **kn)
        U = O.initial_condition(p, ic)
        out[f"{name}_u0"] = U.copy()
        st = O.Stepper(p)
        t = 0.0
        dts, masks = [], []
        for _ in range(nsteps):
            dt = O.setdt(p, U, p.tmax - t)
            Ur = np.empty_like(U)
            m = st.time_stepping(U, Ur, t, dt, want_orders=True)
            dts.append(dt)
            masks.append(np.stack(m))
            t += dt
            U = Ur
        out[f"{name}_uN"] = U
        out[f"{name}_dt"] = np.array(dts)
        out[f"{name}_masks"] = np.stack(masks)
    np.savez_compressed(HERE / "oracle_steps.npz", **out)
    print("wrote", HERE / "gp_weights_mpmath.npz", HERE / "oracle_steps.npz")
    return 0


if __name__ == "__main__":
    sys.exit(main())
