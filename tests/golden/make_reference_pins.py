#!/usr/bin/env python
"""Extract the reference's own recorded outputs into tests/golden/reference_pins.npz
(run from the repository root, in a container where the reference is mounted):

  python tests/golden/make_reference_pins.py [/path/to/reference]

The reference has no tests, but its deprecated code line left per-cell output
of real runs under deprecated/plotter_revision/:

* Isentropic/isen_<run>_Lx20_<n>_ell_1.0_sphere_final_1<niter>.dat -- x, y,
  rho, ux, uy, p and CellGPO of every cell at step 0 and at the last step
  (deprecated/output.f90:62-87, written with list-directed 17-digit output, so
  every double is recorded exactly), and ..._error_L1.dat -- lf, nf, the L1
  density error against the initial state after one period and the GP
  inversion self-check (deprecated/output.f90 error(), GP_init.f90:250);
* 2DRP_C3/2drp_<run>_<n>[_noCSD]_slice_{x,y,xy,yx}.dat -- the final conserved
  state along row nf/2 and the density along column lf/2 and both diagonals
  (deprecated/output.f90:12-57); the step counts of those runs are in the
  names of their (absent) final snapshots, listed in the reference's
  .MISSING_LARGE_BLOBS.

The runs were made by deprecated/main.f90 with deprecated/physics.f90's Setdt
and the slow start of its main loop; the oracle restates those through its
setdt_kind / slow_start / csd_kind knobs.  Nothing here runs the oracle.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
PLOT = REF / "deprecated" / "plotter_revision"

# Isentropic vortex runs: name -> (file stem, n, knobs for the oracle)
VORTEX = {
    "vortex_gp3_rk3_50": ("isen_GP3rd_2quad_RK3_cfl0.8_HLLC", 50,
                          dict(mord=3, ngp=2, integrator=10, lf0=0)),
    "vortex_gp5_rk4_dtred_50": ("isen_GP5th_3quad_RK4_dtRed_cfl0.8_HLLC", 50,
                                dict(mord=5, ngp=3, integrator=12, lf0=50)),
}
# L1 anchors: (file stem, n) for both stencil orders and every recorded size
L1_STEMS = ("isen_GP3rd_2quad_RK3_cfl0.8_HLLC", "isen_GP5th_3quad_RK4_dtRed_cfl0.8_HLLC")
# 2DRP3 runs (configuration 3 of the 2-D Riemann problems, Neumann, ell = 12 dx,
# tmax = 0.8): name -> (file stem, n, noCSD?, knobs)
RP2D3 = {
    "rp2d3_gp3_rk3_200": ("2drp_GP3rd_2quad_RK3_noDtRed_cfl0p8_HLLC", 200, False, dict(mord=3, ngp=2, integrator=10)),
    "rp2d3_gp5_rk4_200": ("2drp_GP5th_3quad_RK4_noDtRed_cfl0p8_HLLC", 200, False, dict(mord=5, ngp=3, integrator=12)),
    "rp2d3_pol3_rk3_200": ("2drp_pol-mood3_2quad_RK3_noDtRed_cfl0p8_HLLC", 200, False,
                           dict(mord=3, ngp=2, integrator=10, method=200)),
    "rp2d3_gp3_rk3_400": ("2drp_GP3rd_2quad_RK3_noDtRed_cfl0p8_HLLC", 400, False, dict(mord=3, ngp=2, integrator=10)),
    "rp2d3_gp5_rk4_400": ("2drp_GP5th_3quad_RK4_noDtRed_cfl0p8_HLLC", 400, False, dict(mord=5, ngp=3, integrator=12)),
}


def read_table(path: Path) -> list[list[str]]:
    return [ln.split() for ln in path.read_text().splitlines() if ln.strip()]


def final_step(stem: str, n: int, suffix: str = "") -> int:
    """The last step of a run: the largest 1<niter> of its final_*.dat snapshots
    (present in the tree or listed as missing blobs)."""
    names = [p.name for p in PLOT.rglob(f"{stem}_*final_1*.dat")]
    blobs = REF / ".MISSING_LARGE_BLOBS"
    if blobs.exists():
        names += re.findall(r"[^\s/]+final_1\d{5}\.dat", blobs.read_text())
    pat = re.compile(re.escape(f"{stem}_{n}{suffix}_final_1") + r"(\d{5})\.dat$")
    pat2 = re.compile(re.escape(f"{stem}_Lx20_{n:03d}_ell_1.0_sphere_final_1") + r"(\d{5})\.dat$")
    steps = [int(m.group(1)) for nm in names for m in (pat.search(nm), pat2.search(nm)) if m]
    if not steps:
        raise SystemExit(f"no final snapshot name for {stem} {n}{suffix}")
    return max(steps)


def main() -> None:
    out: dict[str, np.ndarray] = {}
    meta: dict[str, dict] = {}
    iso = PLOT / "Isentropic"
    for name, (stem, n, kn) in VORTEX.items():
        steps = final_step(stem, n)
        f0 = read_table(iso / f"{stem}_Lx20_{n:03d}_ell_1.0_sphere_final_100000.dat")[1:]
        f1 = read_table(iso / f"{stem}_Lx20_{n:03d}_ell_1.0_sphere_final_1{steps:05d}.dat")[1:]
        out[f"{name}/init"] = np.array([[float(v) for v in r[2:6]] for r in f0]).reshape(n, n, 4)
        out[f"{name}/final"] = np.array([[float(v) for v in r[2:6]] for r in f1]).reshape(n, n, 4)
        out[f"{name}/ordr"] = np.array([int(r[6]) for r in f1], dtype=np.int8).reshape(n, n)
        meta[name] = dict(n=n, steps=steps, lx=20.0, tmax=20.0, ell_abs=1.0, bc=18, **kn,
                          source=f"deprecated/plotter_revision/Isentropic/{stem}_Lx20_{n:03d}_ell_1.0_sphere_final_"
                                 f"{{100000,1{steps:05d}}}.dat")
    rows = []
    for stem in L1_STEMS:
        for n in (50, 100, 200, 400):
            r = read_table(iso / f"{stem}_Lx20_{n:03d}_ell_1.0_sphere_error_L1.dat")[0]
            rows.append((1 if "GP3rd" in stem else 2, n, float(r[2]), float(r[3])))
    out["vortex_l1"] = np.array(rows)  # columns: 1 = GP3rd RK3 / 2 = GP5th RK4 dtRed, n, L1 error, inversion error
    rp = PLOT / "2DRP_C3"
    for name, (stem, n, nocsd, kn) in RP2D3.items():
        suf = "_noCSD" if nocsd else ""
        steps = final_step(stem, n, suf)
        sl = {k: np.array([[float(v) for v in r] for r in read_table(rp / f"{stem}_{n}{suf}_slice_{k}.dat")])
              for k in ("x", "y", "xy", "yx")}
        out[f"{name}/row"] = sl["x"][:, 1:5]      # U(1:4, 1:lf, nf/2)
        out[f"{name}/col"] = sl["y"][:, 1]        # U(rho, lf/2, 1:nf)
        out[f"{name}/diag"] = sl["xy"][:, 1]      # U(rho, l, l)
        out[f"{name}/anti"] = sl["yx"][:, 1]      # U(rho, l, nf-l+1)
        meta[name] = dict(n=n, steps=steps, tmax=0.8, bc=17, ell_o_dx=12.0, csd_kind=2 if nocsd else 0, **kn,
                          source=f"deprecated/plotter_revision/2DRP_C3/{stem}_{n}{suf}_slice_{{x,y,xy,yx}}.dat")
    out["meta"] = np.array(json.dumps(meta, sort_keys=True))
    np.savez_compressed(HERE / "reference_pins.npz", **out)
    print(f"wrote {HERE / 'reference_pins.npz'}: {len(meta)} runs")


if __name__ == "__main__":
    main()
