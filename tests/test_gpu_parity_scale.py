"""Parity at the benchmark configurations' sizes and over whole runs, through the C ABI.

* 2DRP3 at 256^2 (the CPU-runnable configuration: Mord 5, ngp 3, ell = 12 dx,
  HLLC, SSP-RK3, CFL 0.8), 10 steps: exact mode bit for bit, fast mode within
  1e-12 relative L1 per field with identical CellGPO masks.
* The 2048^2 Sedov point blast that bench.py times, in bench.py's fast mode,
  10 steps from t = 0 through the device-resident loop: 1e-12 and identical
  masks against the oracle (OpenMP on the host cores).
* Whole runs to t_final (the main.f90:145-203 loop) on the shock problems:
  2DRP3 128^2 and 256^2 (the CPU-runnable configuration) to 0.8, Sedov 128^2
  and 256^2 to 0.05, DMR 256x64 to 0.2.  Exact mode bit for bit; fast mode
  within 1e-8 relative L1 per field.
* The per-step counters (count_detected_cell of mod_subroutine_MOOD.f90:153,
  printed as a percentage at main.f90:165-167, and the MOOD pass counts)
  against the oracle's.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import nan_equal

pytestmark = pytest.mark.gpu

I = (slice(4, -4), slice(4, -4))

WHOLE = {
    # name: (ic, lf, nf, bc, lx, ly, tmax)
    "rp2d3_128": ("rp2d3", 128, 128, 17, 1.0, 1.0, 0.8),
    "sedov_128": ("sedov", 128, 128, 20, 1.0, 1.0, 0.05),
    "dmr_256x64": ("dmr", 256, 64, 35, 4.0, 1.0, 0.2),
    # the CPU-runnable benchmark configuration itself, and Sedov at the same size
    "rp2d3_256": ("rp2d3", 256, 256, 17, 1.0, 1.0, 0.8),
    "sedov_256": ("sedov", 256, 256, 20, 1.0, 1.0, 0.05),
}


def rel_l1(a, b):
    return [np.abs(a[I + (k,)] - b[I + (k,)]).sum() / np.abs(b[I + (k,)]).sum() for k in range(4)]


def solver(pkg, lf, nf, bc, lx, ly, tmax, fp):
    return pkg.Solver(lf=lf, nf=nf, bc_type=bc, lx=lx, ly=ly, tmax=tmax, fp_mode=fp)


def test_rp2d3_256_ten_steps_exact_and_fast(pkg, oracle):
    lf = nf = 256
    p = oracle.make_params(lf, nf, bc=17, tmax=0.8)
    U = oracle.initial_condition(p, "rp2d3")
    U0 = U.copy()
    st = oracle.Stepper(p)
    t = 0.0
    masks = []
    states = []
    for _ in range(10):
        dt = oracle.setdt(p, U, p.tmax - t)
        Ur = np.empty_like(U)
        masks.append(st.time_stepping(U, Ur, t, dt, want_orders=True)[2])
        states.append((t, dt))
        t += dt
        U = Ur
    with solver(pkg, lf, nf, 17, 1.0, 1.0, 0.8, pkg.FP_EXACT) as s:
        Ug = U0.copy()
        tg = 0.0
        for k in range(10):
            dtg = s.Setdt(Ug, p.tmax - tg)
            assert dtg == states[k][1]
            Ugr = np.empty_like(Ug)
            s.time_stepping(Ug, Ugr, tg, dtg)
            assert np.array_equal(s.orders(), masks[k])
            tg += dtg
            Ug = Ugr
    assert nan_equal(Ug, U)
    with solver(pkg, lf, nf, 17, 1.0, 1.0, 0.8, pkg.FP_FAST) as s:
        s.set_state(U0, 0.0)
        assert s.advance(10) == 10
        Uf, tf, _ = s.get_state()
        assert np.array_equal(s.orders(), masks[-1])
    assert abs(tf - t) <= 1e-12 * t
    assert max(rel_l1(Uf, U)) <= 1e-12


def test_sedov_2048_fast_mode_ten_steps(pkg, oracle):
    """The workload bench.py times, in its fast mode, against the oracle."""
    n = 2048
    p = oracle.make_params(n, n, bc=20, tmax=0.05)
    U = oracle.initial_condition(p, "sedov")
    U0 = U.copy()
    st = oracle.Stepper(p)
    t = 0.0
    for _ in range(9):
        dt = oracle.setdt(p, U, p.tmax - t)
        Ur = np.empty_like(U)
        st.time_stepping(U, Ur, t, dt)
        t += dt
        U = Ur
    dt = oracle.setdt(p, U, p.tmax - t)
    Ur = np.empty_like(U)
    mask = st.time_stepping(U, Ur, t, dt, want_orders=True)[2]
    t += dt
    U = Ur
    with solver(pkg, n, n, 20, 1.0, 1.0, 0.05, pkg.FP_FAST) as s:
        s.set_state(U0, 0.0)
        assert s.advance(10) == 10
        Ug, tg, _ = s.get_state()
        mask_g = s.orders()
        assert s.counters().max_passes_stage > 1  # the MOOD loop ran
    assert abs(tg - t) <= 1e-12 * t
    assert max(rel_l1(Ug, U)) <= 1e-12
    assert np.array_equal(mask_g, mask)


@pytest.fixture(scope="module")
def whole_runs(oracle):
    """The oracle's main loop to t_final on each case (run once per module)."""
    out = {}
    for name, (ic, lf, nf, bc, lx, ly, tmax) in WHOLE.items():
        p = oracle.make_params(lf, nf, bc=bc, lx=lx, ly=ly, tmax=tmax)
        U = oracle.initial_condition(p, ic)
        U0 = U.copy()
        t, n = oracle.Stepper(p).run(U, 0.0, 10 ** 6)
        assert t == tmax
        out[name] = (U0, U, t, n)
    return out


@pytest.mark.parametrize("name", list(WHOLE))
def test_whole_run_exact_mode_bitwise(pkg, whole_runs, name):
    ic, lf, nf, bc, lx, ly, tmax = WHOLE[name]
    U0, U, t, n = whole_runs[name]
    with solver(pkg, lf, nf, bc, lx, ly, tmax, pkg.FP_EXACT) as s:
        s.set_state(U0, 0.0)
        assert s.advance(10 ** 6) == n
        Ug, tg, ng = s.get_state()
    assert (tg, ng) == (t, n)
    assert nan_equal(Ug, U)


@pytest.mark.parametrize("name", list(WHOLE))
def test_whole_run_fast_mode_final_time_tolerance(pkg, whole_runs, name):
    ic, lf, nf, bc, lx, ly, tmax = WHOLE[name]
    U0, U, t, n = whole_runs[name]
    with solver(pkg, lf, nf, bc, lx, ly, tmax, pkg.FP_FAST) as s:
        s.set_state(U0, 0.0)
        s.advance(10 ** 6)
        Ug, tg, ng = s.get_state()
    assert tg == t
    rel = rel_l1(Ug, U)
    assert max(rel) <= 1e-8, (rel, ng, n)


@pytest.mark.parametrize("case", ["dmr", "rp2d3"])
def test_counters_match_the_oracle(pkg, oracle, case):
    """detected_last_step = count_detected_cell of the step (every DETECTION
    pass of every stage, mod_subroutine_MOOD.f90:153, reset at stage 1,
    mod_FE.f90:39-43); mood_passes_last_step = the Forward_Euler loop's
    iterations summed over the stages; max_passes_stage their maximum."""
    ic, lf, nf, bc, lx, ly, tmax = {"dmr": ("dmr", 96, 24, 35, 4.0, 1.0, 0.2),
                                    "rp2d3": ("rp2d3", 64, 64, 17, 1.0, 1.0, 0.8)}[case]
    p = oracle.make_params(lf, nf, bc=bc, lx=lx, ly=ly, tmax=tmax)
    U = oracle.initial_condition(p, ic)
    st = oracle.Stepper(p)
    Ug = U.copy()
    t = 0.0
    total = 0
    with solver(pkg, lf, nf, bc, lx, ly, tmax, pkg.FP_EXACT) as s:
        for step in range(8):
            before = list(st.counters)
            dt = oracle.setdt(p, U, tmax - t)
            Ur = np.empty_like(U)
            st.time_stepping(U, Ur, t, dt)
            dtg = s.Setdt(Ug, tmax - t)
            Ugr = np.empty_like(Ug)
            s.time_stepping(Ug, Ugr, t, dtg)
            c = s.counters()
            assert c.detected_last_step == st.counters[0] - before[0], step
            assert c.mood_passes_last_step == st.counters[1] - before[1], step
            assert c.max_passes_stage == st.counters[2], step
            total += c.detected_last_step
            assert c.detected_total == total
            t += dt
            U, Ug = Ur, Ugr
    assert total > 0
