"""The reference's shipped problem files as presets (gp-mood_gb300/problems.py):
every knob set passes the C ABI's validation, every initial state is
admissible, and the oracle steps each on a small grid.  FOG (method 1) is the
oracle's GP_SE at order 1 with one Gauss point, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest


def _pkg():
    import __graft_entry__ as ge
    return ge.import_package()


@pytest.fixture(scope="module")
def problems():
    _pkg()
    from gpmood_gb300 import problems
    return problems


def _small(kw):
    lf, nf = kw["lf"], kw["nf"]
    s = max(lf, nf) // 32
    return max(lf // s, 8), max(nf // s, 8)


def test_every_shipped_file_is_a_preset(problems):
    assert len(problems.NAMES) == 24


@pytest.mark.parametrize("name", [
    "2DRP12", "2DRP15_FOG", "2DRP15_GPMOOD", "2DRP17", "2DRP3_FOG", "2DRP3_GPMOOD", "2DRP3_GPMOOD_noDMP", "2DRP4_FOG",
    "2DRP4_GPMOOD", "2DRP6", "KH_FOG", "KH_GPMOOD", "Mach800_FOG", "Mach800_GPMOOD", "Mach800_GPMOOD_noDMP", "RT",
    "dmr", "explosion", "implosion", "sedov_FOG", "sedov_GPMOOD", "sedov_GPMOOD_noDMP", "shu_osher_FOG",
    "shu_osher_GPMOOD"])
def test_preset_validates_and_steps(problems, oracle, name):
    pkg = _pkg()
    from gpmood_gb300.gpmood import gp_weights
    kw = problems.knobs(name)
    gp_weights(pkg.default_params(**kw))  # the C ABI's validation and weights, host only
    lf, nf = _small(kw)
    if name == "explosion":
        nf = lf
    kw, U = problems.setup(name, lf=lf, nf=nf)
    p = oracle.make_params(lf, nf, lx=kw["lx"], ly=kw["ly"], tmax=kw["tmax"], mord=kw["mord"], ngp=kw["ngp"],
                           method=kw["method"], bc=kw["bc_type"], dmp=kw["dmp"], u2=kw["u2"], u2_tol=kw["u2_tol"],
                           integrator=kw["integrator"], num_flux=kw["num_flux"])
    oracle.boundary(p, U)
    st = oracle.Stepper(p)
    t = 0.0
    for _ in range(2):
        dt = oracle.setdt(p, U, p.tmax - t)
        Ur = np.empty_like(U)
        st.time_stepping(U, Ur, t, dt)
        t += dt
        U = Ur
    assert np.isfinite(U[4:-4, 4:-4]).all()


def test_fog_is_gp_se_at_first_order(oracle):
    """mod_FOG.f90 sets every face state to the cell value: the oracle's FOG
    equals GP_SE at Mord 1, ngp 1 bit for bit (FE, unsplit, as 2DRP3_FOG)."""
    kw = dict(bc=17, tmax=0.8, ngp=1, integrator=8, num_flux=103)
    a = oracle.make_params(32, 32, mord=3, method=1, **kw)
    b = oracle.make_params(32, 32, mord=1, method=202, **kw)
    U = oracle.initial_condition(a, "rp2d3")
    runs = []
    for p in (a, b):
        st, V, t = oracle.Stepper(p), U.copy(), 0.0
        for _ in range(3):
            dt = oracle.setdt(p, V, p.tmax - t)
            Vr = np.empty_like(V)
            st.time_stepping(V, Vr, t, dt)
            t += dt
            V = Vr
        runs.append(V)
    assert np.array_equal(runs[0], runs[1])


def test_fog_needs_one_gauss_point():
    pkg = _pkg()
    from gpmood_gb300.gpmood import gp_weights
    with pytest.raises(pkg.GpmoodError):
        gp_weights(pkg.default_params(method=1, ngp=2))
