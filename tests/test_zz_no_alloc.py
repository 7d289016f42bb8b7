"""gpmood_time_stepping_noalloc: the step entry point that allocates nothing.

It serves callers that cannot let the library allocate GPU memory (a host that
owns all device memory through its own pool, a real-time loop that must not
stall in cudaMalloc); its scratch is a static device buffer sized for grids up
to (lf+8)*(nf+8) <= 264*264.  Checked here against the allocating entry point
gpmood_time_stepping_dev on two calls in a row, bit for bit in the exact
floating-point mode (the tolerance the parity tests use for that mode), called
through the C ABI.  This file is collected last on purpose."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    f = lib.gpmood_time_stepping_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_void_p]
    f.restype = C.c_int
    return f


@pytest.mark.parametrize("case", ["sedov", "rp2d3"])
def test_noalloc_matches_allocating_entry_point(pkg, oracle, case):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lf = nf = 64
    bc = 20 if case == "sedov" else 17
    tmax = 0.05 if case == "sedov" else 0.8
    p = oracle.make_params(lf, nf, bc=bc, tmax=tmax)
    U0 = oracle.initial_condition(p, case)
    dt = oracle.setdt(p, U0, tmax)

    s = pkg.Solver(lf=lf, nf=nf, bc_type=bc, tmax=tmax, fp_mode=pkg.FP_EXACT)
    lib = s.lib
    noalloc = _noalloc(lib)
    params = s.p

    dev = torch.device("cuda:0")
    ref_in = torch.from_numpy(U0.copy()).to(dev)
    new_in = torch.from_numpy(U0.copy()).to(dev)
    ref_out = torch.empty_like(ref_in)
    new_out = torch.empty_like(new_in)
    t = 0.0
    for call in range(2):
        torch.cuda.synchronize()
        s.time_stepping_dev(ref_in.data_ptr(), ref_out.data_ptr(), t, dt)
        rc = noalloc(C.byref(params), C.c_void_p(new_in.data_ptr()), C.c_void_p(new_out.data_ptr()), t, dt, None)
        assert rc == 0, s._err(None)
        torch.cuda.synchronize()
        a = ref_out.cpu().numpy()
        b = new_out.cpu().numpy()
        assert np.array_equal(a, b), f"call {call}: max |diff| = {np.max(np.abs(a - b))}"
        # The inout ghosts of the input agree too.
        assert np.array_equal(ref_in.cpu().numpy(), new_in.cpu().numpy())
        t += dt
        ref_in, ref_out = ref_out, ref_in
        new_in, new_out = new_out, new_in
    s.close()


def test_noalloc_rejects_grids_beyond_its_scratch(pkg):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    params = pkg.default_params(lf=512, nf=512)
    lib = pkg.load_library()
    noalloc = _noalloc(lib)
    u = torch.zeros((520, 520, 4), dtype=torch.float64, device="cuda")
    rc = noalloc(C.byref(params), C.c_void_p(u.data_ptr()), C.c_void_p(u.data_ptr()), 0.0, 1e-6, None)
    assert rc == -1
    buf = C.create_string_buffer(512)
    lib.gpmood_last_error(None, buf, 512)
    assert b"too large" in buf.value
