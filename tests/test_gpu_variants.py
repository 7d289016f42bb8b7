"""Riemann solvers and integrators beside HLLC / SSP-RK3 (numFlux LLF, HLL,
unsplit: mod_LLF.f90, mod_HLL.f90, mod_unsplit.f90; integrator FE, SSP-RK2,
SSP-RK4: time_stepper.f90, mod_SSP_RK2.f90, mod_SSP_RK4.f90, with
Forward_Euler returning the increment for SSP-RK4, mod_FE.f90:188).

Exact mode: bit-identical states, time steps and final-stage order masks to
the oracle; fast mode: relative L1 <= 1e-12."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import nan_equal

pytestmark = pytest.mark.gpu

VARIANTS = {
    # name: (integrator, num_flux, mord, ngp)
    "llf": (10, 101, 5, 3),
    "hll": (10, 102, 5, 3),
    "unsplit": (10, 103, 5, 3),
    "fe": (8, 100, 5, 3),
    "rk2": (9, 100, 5, 3),
    "rk4": (12, 100, 5, 3),
    "shipped_2drp3": (10, 103, 3, 2),  # problems/2DRP3_GPMOOD.f90: Mord 3, ngp 2, unsplit
    "rk4_hll": (12, 102, 5, 3),
    # Gauss points per face 1, 2, 4, 5 (GP_init.f90:45-83) and the first-order method
    "ngp1": (10, 100, 5, 1),
    "ngp2": (10, 100, 5, 2),
    "ngp4": (10, 100, 5, 4),
    "ngp5": (10, 100, 5, 5),
    "mord1": (10, 100, 1, 1),
}


def _run(pkg, oracle, name, fp_mode, nsteps=5, ic="rp2d3", n=48, bc=17, tmax=0.8):
    integ, nflux, mord, ngp = VARIANTS[name]
    p = oracle.make_params(n, n, bc=bc, tmax=tmax, mord=mord, ngp=ngp, integrator=integ, num_flux=nflux)
    U = oracle.initial_condition(p, ic)
    st = oracle.Stepper(p)
    Ug = U.copy()
    t = 0.0
    with pkg.Solver(lf=n, nf=n, bc_type=bc, tmax=tmax, mord=mord, ngp=ngp, integrator=integ, num_flux=nflux,
                    fp_mode=fp_mode) as s:
        for step in range(nsteps):
            dt = oracle.setdt(p, U, p.tmax - t)
            dtg = s.Setdt(Ug, p.tmax - t)
            Ur = np.empty_like(U)
            st.time_stepping(U, Ur, t, dt)
            Ugr = np.empty_like(Ug)
            s.time_stepping(Ug, Ugr, t, dtg)
            yield step, dt, dtg, Ur, Ugr
            t += dt
            U, Ug = Ur, Ugr


@pytest.mark.parametrize("name", list(VARIANTS))
def test_variant_exact_mode_bitwise(pkg, oracle, name):
    for step, dt, dtg, Ur, Ugr in _run(pkg, oracle, name, pkg.FP_EXACT):
        assert dtg == dt, (step, dtg, dt)
        assert nan_equal(Ugr, Ur), (step, np.nanmax(np.abs(Ugr - Ur)))


@pytest.mark.parametrize("name", ["unsplit", "rk4", "hll", "ngp2", "ngp5"])
def test_variant_fast_mode_tolerance(pkg, oracle, name):
    for step, dt, dtg, Ur, Ugr in _run(pkg, oracle, name, pkg.FP_FAST):
        pass
    I = (slice(4, -4), slice(4, -4))
    for k in range(4):
        rel = np.abs(Ugr[I + (k,)] - Ur[I + (k,)]).sum() / np.abs(Ur[I + (k,)]).sum()
        assert rel <= 1e-12, (k, rel)
