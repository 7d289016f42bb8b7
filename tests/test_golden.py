"""The committed golden fixtures (tests/golden/make_golden.py).

CPU: the oracle reproduces its own recorded steps bit for bit (no drift), and
both the oracle's and the library's GP weights agree with the 60-digit mpmath
derivation.  GPU: the CUDA exact mode equals the recorded states, time steps
and per-stage MOOD masks without running the oracle at all."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from conftest import nan_equal

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = {
    "rp2d3": ("rp2d3", 32, 32, dict(bc=17, tmax=0.8)),
    "sedov": ("sedov", 32, 32, dict(bc=20, tmax=0.05)),
    "vortex": ("vortex", 32, 32, dict(bc=18, lx=10.0, ly=10.0, tmax=1.0)),
    "dmr": ("dmr", 48, 12, dict(bc=35, lx=4.0, ly=1.0, tmax=0.2)),
}


@pytest.fixture(scope="module")
def steps():
    return dict(np.load(GOLDEN / "oracle_steps.npz"))


@pytest.fixture(scope="module")
def mpw():
    return dict(np.load(GOLDEN / "gp_weights_mpmath.npz"))


@pytest.mark.parametrize("case", list(CASES))
def test_oracle_reproduces_golden_steps(oracle, steps, case):
    ic, lf, nf, kn = CASES[case]
    p = oracle.make_params(lf, nf, **kn)
    U = oracle.initial_condition(p, ic)
    assert nan_equal(U, steps[f"{case}_u0"])
    st = oracle.Stepper(p)
    t = 0.0
    for k, dt_ref in enumerate(steps[f"{case}_dt"]):
        dt = oracle.setdt(p, U, p.tmax - t)
        assert dt == dt_ref, (k, dt, dt_ref)
        Ur = np.empty_like(U)
        m = st.time_stepping(U, Ur, t, dt, want_orders=True)
        assert np.array_equal(np.stack(m), steps[f"{case}_masks"][k])
        t += dt
        U = Ur
    assert nan_equal(U, steps[f"{case}_uN"])


@pytest.mark.parametrize("ngp", [2, 3])
def test_weights_match_golden_mpmath(oracle, pkg, mpw, ngp):
    """Oracle (binary128 restatement) and library GP weights against the
    60-digit derivation: 1e-8 absolute on the ill-conditioned R2 system,
    1e-7 relative on the R1 second derivatives."""
    lf = 64
    p = oracle.make_params(lf, lf, ngp=ngp, ell_o_dx=float(mpw["ell_o_dx"]))
    g = oracle.gp_weights(p)
    zt_o = np.array(g.zt).reshape(3, 4, 5, 13)[:, :, :ngp]
    zt_l, d2, _ = pkg.gp_weights(pkg.default_params(lf=lf, nf=lf, ngp=ngp, ell_o_dx=float(mpw["ell_o_dx"])))
    ref = mpw[f"zt_ngp{ngp}"]
    for zt in (zt_o, zt_l):
        for o, npt in ((1, 5), (2, 13)):
            assert np.max(np.abs(zt[o, :, :, :npt] - ref[o, :, :, :npt])) < 1e-8
    np.testing.assert_allclose(np.array(g.d2x)[:5], mpw[f"d2x_cells_ngp{ngp}"] * lf * lf, rtol=1e-7)
    np.testing.assert_allclose(d2[0], mpw[f"d2x_cells_ngp{ngp}"] * lf * lf, rtol=1e-7)


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(CASES))
def test_cuda_exact_mode_equals_golden(pkg, steps, case):
    ic, lf, nf, kn = CASES[case]
    kw = dict(lf=lf, nf=nf, fp_mode=pkg.FP_EXACT, tmax=kn["tmax"], bc_type=kn["bc"], lx=kn.get("lx", 1.0),
              ly=kn.get("ly", 1.0))
    U = steps[f"{case}_u0"].copy()
    t = 0.0
    with pkg.Solver(**kw) as s:
        for k, dt_ref in enumerate(steps[f"{case}_dt"]):
            dt = s.Setdt(U, kn["tmax"] - t)
            assert dt == dt_ref, (k, dt, dt_ref)
            Ur = np.empty_like(U)
            s.time_stepping(U, Ur, t, dt)
            masks = np.stack([s.stage_orders(st) for st in range(3)])
            assert np.array_equal(masks, steps[f"{case}_masks"][k]), k
            t += dt
            U = Ur
    assert nan_equal(U, steps[f"{case}_uN"])
