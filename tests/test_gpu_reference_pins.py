"""The CUDA path against the reference's own recorded outputs, through the C ABI.

tests/golden/reference_pins.npz holds final states of runs the reference's
deprecated code line recorded (tests/golden/make_reference_pins.py).  Those
runs took their time steps from deprecated/physics.f90's Setdt with the slow
start of deprecated/main.f90; the host side of this test restates that loop
(the oracle's Setdt with setdt_kind = 1), and every step runs through
gpmood_time_stepping, which is gp-mood-code's time_stepping unchanged.

Exact mode: the 2DRP3 slices after 487-1037 steps with MOOD active are equal
bit for bit; fast mode stays within 1e-8 relative L1 of them (the final-time
tolerance of the design).  The vortex from its recorded initial state stays
within 1e-13 (fast mode 1e-12) of its recorded final state."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from test_reference_pins import cons, deprecated_params, prim, slices

pytestmark = pytest.mark.gpu

PINS = Path(__file__).resolve().parent / "golden" / "reference_pins.npz"


@pytest.fixture(scope="module")
def pins():
    z = np.load(PINS)
    return z, json.loads(str(z["meta"]))


def run_recorded(pkg, oracle, m, U, fp_mode):
    """deprecated/main.f90's loop: Setdt, the slow start, time_stepping, t += dt."""
    p = deprecated_params(oracle, m)
    n = m["n"]
    kw = dict(lf=n, nf=n, fp_mode=fp_mode, tmax=m["tmax"], bc_type=m["bc"], lx=p.lx, ly=p.ly, mord=m["mord"],
              ngp=m["ngp"], integrator=m["integrator"], method=m.get("method", 2), ell_o_dx=p.ell_o_dx)
    t, steps, dt_sim = 0.0, 0, 1e-10
    with pkg.Solver(**kw) as s:
        while t < m["tmax"]:
            steps += 1
            dt = oracle.setdt(p, U, m["tmax"] - t)
            if dt_sim < dt:
                dt, dt_sim = dt_sim, 2.0 * dt_sim
            Ur = np.empty_like(U)
            s.time_stepping(U, Ur, t, dt)
            t += dt
            U = Ur
        status = s.counters().status_flags
    return U, t, steps, status


@pytest.mark.parametrize("name", ["rp2d3_gp3_rk3_200", "rp2d3_pol3_rk3_200", "rp2d3_gp5_rk4_200",
                                  "rp2d3_gp3_rk3_400", "rp2d3_gp5_rk4_400"])
def test_exact_mode_reproduces_the_recorded_2drp3_runs(pkg, oracle, pins, name):
    z, meta = pins
    m = meta[name]
    U0 = oracle.initial_condition(deprecated_params(oracle, m), "rp2d3")
    U, t, steps, status = run_recorded(pkg, oracle, m, U0, pkg.FP_EXACT)
    assert (t, steps, status) == (0.8, m["steps"], 0)
    for k, v in slices(U, m["n"]).items():
        assert np.array_equal(v, z[f"{name}/{k}"]), (k, np.abs(v - z[f"{name}/{k}"]).max())


@pytest.mark.parametrize("name", ["rp2d3_gp3_rk3_200", "rp2d3_gp5_rk4_200"])
def test_fast_mode_stays_near_the_recorded_2drp3_runs(pkg, oracle, pins, name):
    z, meta = pins
    m = meta[name]
    U0 = oracle.initial_condition(deprecated_params(oracle, m), "rp2d3")
    U, t, steps, _ = run_recorded(pkg, oracle, m, U0, pkg.FP_FAST)
    assert t == 0.8 and abs(steps - m["steps"]) <= 1
    got, ref = slices(U, m["n"]), {k: z[f"{name}/{k}"] for k in ("row", "col", "diag", "anti")}
    for k in range(4):
        rel = np.abs(got["row"][:, k] - ref["row"][:, k]).sum() / np.abs(ref["row"][:, k]).sum()
        assert rel <= 1e-8, (k, rel)
    for k in ("col", "diag", "anti"):
        rel = np.abs(got[k] - ref[k]).sum() / np.abs(ref[k]).sum()
        assert rel <= 1e-8, (k, rel)


@pytest.mark.parametrize("fp", ["exact", "fast"])
def test_vortex_from_the_recorded_state(pkg, oracle, pins, fp):
    z, meta = pins
    name = "vortex_gp5_rk4_dtred_50"
    m = meta[name]
    n = m["n"]
    p = deprecated_params(oracle, m)
    U0 = oracle.padded(n, n)
    U0[4:-4, 4:-4] = cons(z[f"{name}/init"])
    oracle.boundary(p, U0, 0.0)
    U, t, steps, status = run_recorded(pkg, oracle, m, U0, pkg.FP_EXACT if fp == "exact" else pkg.FP_FAST)
    assert (t, steps, status) == (20.0, m["steps"], 0)
    tol = 1e-13 if fp == "exact" else 1e-12  # fast mode: FMA contraction over 210 steps
    assert np.abs(prim(U[4:-4, 4:-4]) - z[f"{name}/final"]).max() <= tol
