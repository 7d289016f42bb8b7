"""Failure paths of the kernels' bounded waits, driven without a faulty GPU.

Every spin-wait in the kernels is bounded: the grid barrier of the
cooperative MOOD loop and the gate's tensor-core (tcgen05) MMA waits give up
after ~1 s, set a status bit and fail the step with GPMOOD_E_CUDA while the
context stays usable.  gpmood_set_wait_limit (a test hook) shortens those
bounds to a few polls, so the waits run out on a healthy GPU; nothing hangs
and nothing faults: the bound is what ends each wait, and the gate waits for
its MMAs in flight before it frees their tensor memory.  After the limit is
lifted the same context steps normally, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import nan_equal

pytestmark = pytest.mark.gpu


def test_grid_barrier_timeout_fails_the_step_and_the_context_recovers(pkg, oracle):
    n = 256
    p = oracle.make_params(n, n, bc=17, tmax=0.8)
    U = oracle.initial_condition(p, "rp2d3")
    dt = oracle.setdt(p, U, p.tmax)
    ref = np.empty_like(U)
    st = oracle.Stepper(p)
    st.time_stepping(U.copy(), ref, 0.0, dt)
    assert st.counters[0] > 100  # MOOD lists long enough for the multi-CTA loop and its grid barrier
    with pkg.Solver(lf=n, nf=n, bc_type=17, tmax=0.8, fp_mode=pkg.FP_EXACT) as s:
        s.set_wait_limit(1)
        out = np.empty_like(U)
        with pytest.raises(pkg.GpmoodError) as e:
            s.time_stepping(U.copy(), out, 0.0, dt)
        assert e.value.code == -2 and "barrier" in str(e.value)
        assert s.counters().status_flags & 8
        s.set_wait_limit(0)
        out = np.empty_like(U)
        s.time_stepping(U.copy(), out, 0.0, dt)
    assert nan_equal(out, ref)


def test_gate_tensor_core_wait_timeout_fails_the_step_and_the_context_recovers(pkg):
    from gpmood_gb300 import ic, nn_train as T
    n = 128
    params = T.init_params(0)
    U = ic.rp2d3(n, n)
    kw = dict(lf=n, nf=n, bc_type=17, tmax=0.8, method=pkg.NN_GP_MOOD, fp_mode=pkg.FP_FAST)

    def start(s):
        s.Boundary_C(U, 0.0)
        s.set_state(U, 0.0)
        s.set_nn(params)

    with pkg.Solver(**kw) as r:
        start(r)
        assert r.advance(2) == 2
        ref, tref, _ = r.get_state()
    with pkg.Solver(**kw) as s:
        start(s)
        s.set_wait_limit(1)
        with pytest.raises(pkg.GpmoodError) as e:
            s.advance(1)
        # the hook bounds the MOOD loop's grid barrier too, so either timeout may be reported first
        assert e.value.code == -2 and "timed out" in str(e.value)
        assert s.counters().status_flags & 16
        s.set_wait_limit(0)
        start(s)
        assert s.advance(2) == 2
        got, t, _ = s.get_state()
    assert t == tref
    assert nan_equal(got, ref)


def test_wait_limit_rejects_negative_polls(pkg):
    with pkg.Solver(lf=16, nf=16) as s:
        with pytest.raises(pkg.GpmoodError) as e:
            s.set_wait_limit(-1)
        assert e.value.code == -1
