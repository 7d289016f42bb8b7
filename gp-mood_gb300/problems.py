"""The reference's shipped problem files (gp-mood-code/problems/*.f90) as presets.

Each entry carries the knobs of the file's `parameters` module (CFL,
integrator, method, ell_o_dx, Mord, ngp, DMP, U2, U2_tol, numFlux, lf, nf,
tmax, nmax, Lx, Ly, BC_type) and the initial condition of its `problem`
(IC.f90), built by `gpmood_gb300.ic`.  `setup(name)` returns the Solver
keyword arguments and the initial state (ghosts left to Boundary_C, as
InitialCdt leaves them):

    kw, U0 = problems.setup("2DRP3_GPMOOD", lf=128, nf=128)
    with Solver(**kw) as s:
        s.Boundary_C(U0, 0.0); s.set_state(U0, 0.0); s.advance(1 << 30)
"""
from __future__ import annotations

from . import ic
from .gpmood import (DMR, FE, FOG, GP_MOOD, HLL, HLLC, KH, MACH800, NEUMANN, PERIODIC, REFLECTIVE, RT, SSP_RK3,
                     UNSPLIT)

# (integrator, method, mord, ngp, dmp/u2/u2_tol, numFlux, lf, nf, tmax, nmax, Lx, Ly, BC_type, IC builder)
_FILES = {
    "2DRP12": (SSP_RK3, GP_MOOD, 3, 2, 1, HLLC, 256, 256, 0.25, 9999, 1., 1., NEUMANN, "rp2d12"),
    "2DRP15_FOG": (FE, FOG, 3, 1, 1, UNSPLIT, 256, 256, 0.2, 9999, 1., 1., NEUMANN, "rp2d15"),
    "2DRP15_GPMOOD": (SSP_RK3, GP_MOOD, 3, 2, 1, UNSPLIT, 256, 256, 0.2, 9999, 1., 1., NEUMANN, "rp2d15"),
    "2DRP17": (SSP_RK3, GP_MOOD, 3, 2, 1, HLLC, 256, 256, 0.3, 9999, 1., 1., NEUMANN, "rp2d17"),
    "2DRP3_FOG": (FE, FOG, 3, 1, 1, UNSPLIT, 256, 256, 0.8, 9999, 1., 1., NEUMANN, "rp2d3"),
    "2DRP3_GPMOOD": (SSP_RK3, GP_MOOD, 3, 2, 1, UNSPLIT, 256, 256, 0.8, 9999, 1., 1., NEUMANN, "rp2d3"),
    "2DRP3_GPMOOD_noDMP": (SSP_RK3, GP_MOOD, 3, 2, 0, UNSPLIT, 256, 256, 0.8, 9999, 1., 1., NEUMANN, "rp2d3"),
    "2DRP4_FOG": (FE, FOG, 3, 1, 1, UNSPLIT, 256, 256, 0.25, 9999, 1., 1., NEUMANN, "rp2d4"),
    "2DRP4_GPMOOD": (SSP_RK3, GP_MOOD, 3, 2, 1, UNSPLIT, 256, 256, 0.25, 9999, 1., 1., NEUMANN, "rp2d4"),
    "2DRP6": (SSP_RK3, GP_MOOD, 3, 2, 1, HLLC, 256, 256, 0.3, 9999, 1., 1., NEUMANN, "rp2d6"),
    "KH_FOG": (FE, FOG, 3, 1, 1, UNSPLIT, 256, 256, 1.0, 9999, 1., 1., KH, "kelvin_helmholtz"),
    "KH_GPMOOD": (SSP_RK3, GP_MOOD, 3, 2, 1, UNSPLIT, 256, 256, 1.0, 9999, 1., 1., KH, "kelvin_helmholtz"),
    "Mach800_FOG": (FE, FOG, 3, 1, 0, HLL, 256, 256, 0.005, 999999, 1.5, 1.5, MACH800, "mach800"),
    "Mach800_GPMOOD": (SSP_RK3, GP_MOOD, 3, 2, 1, HLL, 256, 256, 0.005, 999999, 1.5, 1.5, MACH800, "mach800"),
    "Mach800_GPMOOD_noDMP": (SSP_RK3, GP_MOOD, 3, 2, 0, HLL, 256, 256, 0.005, 99999, 1.5, 1.5, MACH800, "mach800"),
    "RT": (SSP_RK3, GP_MOOD, 3, 2, 1, UNSPLIT, 64, 3 * 64, 12.4, 99999, 0.5, 1.5, RT, "rt"),
    "dmr": (SSP_RK3, GP_MOOD, 3, 2, 1, HLLC, 512, 128, 0.25, 9999, 4., 1., DMR, "dmr"),
    "explosion": (SSP_RK3, GP_MOOD, 3, 2, 1, HLLC, 256, 256, 3.2, 9999, 1.5, 1.5, NEUMANN, "explosion"),
    "implosion": (SSP_RK3, GP_MOOD, 3, 2, 1, HLLC, 256, 256, 2.5, 9999, 0.3, 0.3, REFLECTIVE, "implosion"),
    "sedov_FOG": (FE, FOG, 3, 1, 0, UNSPLIT, 256, 256, 0.05, 9999, 1., 1., NEUMANN, "sedov"),
    "sedov_GPMOOD": (SSP_RK3, GP_MOOD, 3, 2, 1, UNSPLIT, 256, 256, 0.05, 9999, 1., 1., NEUMANN, "sedov"),
    "sedov_GPMOOD_noDMP": (SSP_RK3, GP_MOOD, 3, 2, 0, UNSPLIT, 256, 256, 0.05, 9999, 1., 1., NEUMANN, "sedov"),
    "shu_osher_FOG": (FE, FOG, 3, 1, 1, HLL, 512, 512, 1.8, 9999, 28.2842712474619, 28.2842712474619, PERIODIC,
                      "shu_osher_rotated"),
    "shu_osher_GPMOOD": (SSP_RK3, GP_MOOD, 3, 2, 1, HLL, 512, 512, 1.8, 9999, 28.2842712474619, 28.2842712474619,
                         PERIODIC, "shu_osher_rotated"),
}

NAMES = tuple(_FILES)


def knobs(name: str) -> dict:
    """Solver keyword arguments of problem file `name` (CFL 0.8, ell_o_dx 12 in every file)."""
    integ, method, mord, ngp, checks, nflux, lf, nf, tmax, nmax, lx, ly, bc, _ = _FILES[name]
    return dict(cfl=0.8, ell_o_dx=12.0, integrator=integ, method=method, mord=mord, ngp=ngp, dmp=checks, u2=checks,
                u2_tol=checks, num_flux=nflux, lf=lf, nf=nf, tmax=tmax, nmax=nmax, lx=lx, ly=ly, bc_type=bc)


def setup(name: str, lf: int | None = None, nf: int | None = None, **overrides):
    """(Solver kwargs, initial state) of problem file `name`, optionally on another grid."""
    kw = knobs(name)
    if lf is not None:
        kw["lf"] = lf
    if nf is not None:
        kw["nf"] = nf
    kw.update(overrides)
    builder = _FILES[name][-1]
    U0 = getattr(ic, builder)(kw["lf"], kw["nf"], lx=kw["lx"], ly=kw["ly"])
    return kw, U0
