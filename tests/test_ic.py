"""Initial conditions of IC.f90 (gp-mood_gb300/ic.py): shapes, admissible
states, the reference's overwrite order, and a few oracle steps of each
problem with its boundary condition."""
from __future__ import annotations

import numpy as np
import pytest


def _ic():
    import __graft_entry__ as ge
    ge.import_package()
    from gpmood_gb300 import ic
    return ic


NGC = 4
BUILDERS = ["sod_x", "sod_y", "sod_xy", "sod_rotated", "slow_shock", "lax", "shu_osher", "shu_osher_rotated",
            "strong_rarefaction", "blast", "lin_gauss_x", "lin_gauss_y", "lin_gauss_xy", "implosion", "explosion",
            "rp2d3", "rp2d4", "rp2d6", "rp2d12", "rp2d15", "rp2d17", "dmr", "sedov", "mach800", "rmi", "rt",
            "kelvin_helmholtz", "isentropic_vortex"]


def _pressure(U):
    return 0.4 * (U[..., 3] - 0.5 * (U[..., 1] ** 2 + U[..., 2] ** 2) / U[..., 0])


@pytest.mark.parametrize("name", BUILDERS)
def test_builder_fills_admissible_states(name):
    ic = _ic()
    lf = nf = 24
    U = getattr(ic, name)(lf, nf)
    assert U.shape == (nf + 2 * NGC, lf + 2 * NGC, 4)
    filled = U[: nf + NGC, : lf + NGC]  # lb..lf x nb..nf, as InitialCdt (IC.f90:29-30)
    interior = U[NGC: nf + NGC, NGC: lf + NGC]
    assert np.isfinite(filled).all()
    assert (interior[..., 0] > 0).all() and (_pressure(interior) > 0).all()
    assert not U[nf + NGC:].any() and not U[:, lf + NGC:].any()  # high ghosts: Boundary_C's


def test_sod_y_is_sod_x_transposed():
    ic = _ic()
    a, b = ic.sod_x(32, 32), ic.sod_y(32, 32)
    bt = np.transpose(b, (1, 0, 2))[..., [0, 2, 1, 3]]
    assert np.array_equal(a, bt)


def test_quadrant_overwrite_order():
    """f_RP_2D_12 uses strict inequalities in two quadrants: on the split
    lines the later assignments win, as in the sequential Fortran ifs."""
    ic = _ic()
    U = ic.rp2d12(2, 2, lx=1.0, ly=1.0)  # cells at x, y = 0.25, 0.75
    assert np.allclose(U[NGC, NGC], ic.p2c(0.8, 0.0, 0.0, 1.0))
    assert np.allclose(U[NGC + 1, NGC + 1], ic.p2c(0.5313, 0.0, 0.0, 0.4))


def test_blast_keeps_ghost_left_empty():
    ic = _ic()
    U = ic.blast(40, 4)
    assert not U[:, :NGC].any()  # x < 0: no branch of IC.f90:88-91 matches
    assert np.allclose(U[NGC, NGC], ic.p2c(1., 0., 0., 1000.))


@pytest.mark.parametrize("name,bc,kw", [("shu_osher", 19, {}), ("mach800", 201, {}),
                                        ("mach800", 301, {"double": True}), ("rmi", 401, {}), ("rt", 402, {}),
                                        ("kelvin_helmholtz", 403, {}), ("implosion", 20, {}),
                                        ("lin_gauss_xy", 18, {})])
def test_problem_steps_with_its_boundary(oracle, name, bc, kw):
    ic = _ic()
    lf, nf = 32, 16
    defaults = {"shu_osher": (9.0, 1.0), "mach800": (1.5, 1.5), "rmi": (6.0, 1.0), "rt": (0.25, 1.0),
                "kelvin_helmholtz": (1.0, 1.0), "implosion": (0.3, 0.3), "lin_gauss_xy": (1.0, 1.0)}
    lx, ly = defaults[name]
    U = getattr(ic, name)(lf, nf, lx=lx, ly=ly, **kw)
    p = oracle.make_params(lf, nf, bc=bc, lx=lx, ly=ly, tmax=10.0)
    oracle.boundary(p, U)
    st = oracle.Stepper(p)
    t = 0.0
    for _ in range(3):
        dt = oracle.setdt(p, U, p.tmax - t)
        assert dt > 0
        Ur = np.empty_like(U)
        st.time_stepping(U, Ur, t, dt)
        t += dt
        U = Ur
    assert np.isfinite(U[NGC:-NGC, NGC:-NGC]).all()


def test_shu_osher_left_state_is_the_dirichlet_inflow(oracle):
    ic = _ic()
    U = ic.shu_osher(36, 4)
    V = U.copy()
    p = oracle.make_params(36, 4, bc=19, lx=9.0, ly=1.0)
    oracle.boundary(p, V)
    assert np.array_equal(V[NGC + 1, 0], U[NGC + 1, NGC])  # ghost (l = -3) = first cell, both p2c(3.857143, ...)


@pytest.mark.parametrize("name,oname,lx,ly", [("rp2d3", "rp2d3", 1.0, 1.0), ("sedov", "sedov", 1.0, 1.0),
                                             ("dmr", "dmr", 4.0, 1.0), ("isentropic_vortex", "vortex", 10.0, 10.0)])
def test_builders_match_the_oracle_ics(oracle, name, oname, lx, ly):
    """ic.py's builders followed by Boundary_C (main.f90:125) equal the CPU
    restatement's initial states (IC.f90 plus Boundary_C); the vortex's exp
    and power agree to a few ulp."""
    ic = _ic()
    lf, nf = 40, 24
    p = oracle.make_params(lf, nf, lx=lx, ly=ly, bc={"dmr": 35, "vortex": 18}.get(oname, 17))
    Uo = oracle.initial_condition(p, oname)
    Ui = getattr(ic, name)(lf, nf, lx=lx, ly=ly)
    oracle.boundary(p, Ui)
    if name in ("rp2d3", "dmr"):
        assert np.array_equal(Ui, Uo)
    else:
        np.testing.assert_allclose(Ui, Uo, rtol=1e-14, atol=1e-14)
