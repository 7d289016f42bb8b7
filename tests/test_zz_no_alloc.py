"""gpmood_time_stepping_noalloc: the step entry point that allocates nothing.

Some callers cannot let a library allocate GPU memory: a host that owns all
device memory through its own pool, or a real-time loop that must not stall in
cudaMalloc.  This entry point serves them with a static device buffer sized for
grids up to (lf+8)*(nf+8) <= 264*264.  Here it is called through the C ABI and
checked against the allocating entry point gpmood_time_stepping_dev on two
calls in a row: bit for bit in the exact floating-point mode, and within the
fast mode's parity tolerance (1e-12 relative L1 per field) in the fast mode.
It also reports the same status bits and the same MOOD-cap error, and rejects
grids beyond its buffer.  This file is collected last on purpose."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import nan_equal

pytestmark = pytest.mark.gpu

CASES = {
    # name: (ic, lf, nf, knobs)
    "sedov": ("sedov", 64, 64, dict(bc_type=20, tmax=0.05)),
    "rp2d3": ("rp2d3", 64, 64, dict(bc_type=17, tmax=0.8)),
    "rp2d3_fast": ("rp2d3", 64, 64, dict(bc_type=17, tmax=0.8, fp_mode=1)),
    "dmr": ("dmr", 96, 24, dict(bc_type=35, lx=4.0, ly=1.0, tmax=0.2)),
    "vortex_gp_se": ("vortex", 48, 48, dict(bc_type=18, lx=10.0, ly=10.0, tmax=1.0, method=202)),
    "rp2d3_hll_r1": ("rp2d3", 40, 56, dict(bc_type=17, tmax=0.8, num_flux=102, mord=3, ngp=2)),
}


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    return torch


def _noalloc(lib):
    f = lib.gpmood_time_stepping_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.POINTER(C.c_int)]
    f.restype = C.c_int
    return f


def _rel_l1(a, b):
    I = (slice(4, -4), slice(4, -4))
    return max(np.abs(a[I + (k,)] - b[I + (k,)]).sum() / np.abs(b[I + (k,)]).sum() for k in range(4))


def _two_calls(pkg, oracle, case, plant=None, max_mood_iters=0):
    """Two steps in a row through both entry points; returns per call
    (dev result, noalloc result, dev status, noalloc status, noalloc rc)."""
    torch = _torch()
    ic, lf, nf, kn = CASES[case]
    p = oracle.make_params(lf, nf, bc=kn["bc_type"], lx=kn.get("lx", 1.0), ly=kn.get("ly", 1.0), tmax=kn["tmax"],
                           method=kn.get("method", 2), mord=kn.get("mord", 5), ngp=kn.get("ngp", 3),
                           num_flux=kn.get("num_flux", 100))
    U0 = oracle.initial_condition(p, ic)
    if plant is not None:
        plant(U0)
    dt = oracle.setdt(p, U0, kn["tmax"])
    s = pkg.Solver(lf=lf, nf=nf, max_mood_iters=max_mood_iters, **kn)
    noalloc = _noalloc(s.lib)
    dev = torch.device("cuda:0")
    ref_in = torch.from_numpy(U0.copy()).to(dev)
    new_in = torch.from_numpy(U0.copy()).to(dev)
    ref_out = torch.empty_like(ref_in)
    new_out = torch.empty_like(new_in)
    out = []
    t = 0.0
    try:
        for call in range(2):
            torch.cuda.synchronize()
            before = s.counters().status_flags
            dev_rc = 0
            try:
                s.time_stepping_dev(ref_in.data_ptr(), ref_out.data_ptr(), t, dt)
            except pkg.GpmoodError as e:
                dev_rc = e.code
            dev_status = s.counters().status_flags & ~before
            st = C.c_int(-1)
            rc = noalloc(C.byref(s.p), C.c_void_p(new_in.data_ptr()), C.c_void_p(new_out.data_ptr()), t, dt, None,
                         C.byref(st))
            torch.cuda.synchronize()
            out.append((ref_out.cpu().numpy(), new_out.cpu().numpy(), ref_in.cpu().numpy(), new_in.cpu().numpy(),
                        dev_rc, rc, dev_status, st.value))
            t += dt
            ref_in, ref_out = ref_out, ref_in
            new_in, new_out = new_out, new_in
    finally:
        s.close()
    return out


@pytest.mark.parametrize("case", list(CASES))
def test_noalloc_matches_allocating_entry_point(pkg, oracle, case):
    fast = CASES[case][3].get("fp_mode", 0) == 1
    for call, (a, b, ain, bin_, dev_rc, rc, dev_st, st) in enumerate(_two_calls(pkg, oracle, case)):
        assert (dev_rc, rc) == (0, 0), (call, dev_rc, rc)
        assert st == dev_st == 0, (call, st, dev_st)
        if fast:
            assert _rel_l1(b, a) <= 1e-12, (call, _rel_l1(b, a))
        else:
            assert nan_equal(a, b), f"call {call}: max |diff| = {np.nanmax(np.abs(a - b))}"
            assert nan_equal(ain, bin_)  # the inout ghosts of the input agree too


def test_noalloc_reports_a_state_left_in_an_order_one_cell(pkg, oracle):
    """A negative pressure planted in the input (on the host): both entry
    points lower the cells around it to first order, set status bit 0 and
    still succeed, with the same result."""
    def plant(U):
        j, i = 4 + 20, 4 + 30
        U[j, i, 3] = 0.5 * (U[j, i, 1] ** 2 + U[j, i, 2] ** 2) / U[j, i, 0] - 1.0

    a, b, _, _, dev_rc, rc, dev_st, st = _two_calls(pkg, oracle, "rp2d3", plant=plant)[0]
    assert (dev_rc, rc) == (0, 0)
    assert st & 1 and dev_st & 1
    assert nan_equal(a, b)


def test_noalloc_mood_cap_is_an_error_after_the_whole_step(pkg, oracle):
    """max_mood_iters = 1: both entry points return GPMOOD_E_MOOD_CAP (-3)
    with status bit 1, after running every stage, and agree on the output."""
    a, b, _, _, dev_rc, rc, dev_st, st = _two_calls(pkg, oracle, "rp2d3", max_mood_iters=1)[0]
    assert dev_rc == rc == -3
    assert st & 2 and dev_st & 2
    assert nan_equal(a, b)


def test_noalloc_rejects_grids_beyond_its_scratch(pkg):
    torch = _torch()
    params = pkg.default_params(lf=512, nf=512)
    lib = pkg.load_library()
    noalloc = _noalloc(lib)
    u = torch.zeros((520, 520, 4), dtype=torch.float64, device="cuda")
    rc = noalloc(C.byref(params), C.c_void_p(u.data_ptr()), C.c_void_p(u.data_ptr()), 0.0, 1e-6, None, None)
    assert rc == -1
    buf = C.create_string_buffer(512)
    lib.gpmood_last_error(None, buf, 512)
    assert b"too large" in buf.value
