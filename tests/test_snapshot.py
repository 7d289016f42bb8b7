"""Snapshot / restart and dataset files in the reference's field layout
(gp-mood_gb300/snapshot.py; output.f90:77-192,302-400, reader.f90:12-120)."""
from __future__ import annotations

import numpy as np
import pytest


def _mod():
    import __graft_entry__ as ge
    ge.import_package()
    from gpmood_gb300 import snapshot
    return snapshot


def test_snapshot_round_trip_on_cpu(tmp_path, oracle):
    S = _mod()
    p = oracle.make_params(40, 24, bc=17)
    U = oracle.initial_condition(p, "rp2d3")
    oracle.boundary(p, U)
    orders = np.full((24, 40), 5, np.int8)
    orders[3, 7] = 3
    S.save_snapshot(tmp_path / "snap.npz", U, 0.125, 17, orders, cfl=0.8, problem="2DRP3", method="GP_MOOD")
    snap = S.load_snapshot(tmp_path / "snap.npz")
    assert (snap["lf"], snap["nf"], snap["niter"], snap["time"]) == (40, 24, 17, 0.125)
    assert snap["rho"].shape == (24, 40) and snap["ordr"].dtype == np.int32 and snap["ordr"][3, 7] == 3
    assert snap["problem"] == "2DRP3" and snap["method"] == "GP_MOOD" and float(snap["CFL"]) == 0.8
    W = S.conservative_to_primitive(U[4:-4, 4:-4])
    assert np.array_equal(snap["p"], W[..., 3])
    V = S.state_from_snapshot(snap)
    # primitive -> conservative rounds: the restart state is equal to rounding
    np.testing.assert_allclose(V[4:-4, 4:-4], U[4:-4, 4:-4], rtol=1e-15, atol=1e-15)
    assert not V[:4].any()  # ghosts are left for Boundary_C


def test_dataset_file_layout(tmp_path):
    S = _mod()
    rng = np.random.default_rng(3)
    x = rng.normal(size=(100, 36)).astype(np.float32)
    y = (rng.uniform(size=100) < 0.3).astype(np.float32)
    S.save_dataset(tmp_path / "ds.npz", x, y, problem="Sedov", method="GP_MOOD")
    with np.load(tmp_path / "ds.npz") as z:
        assert z["labels"].shape == (2, 100) and z["inputs"].shape == (36, 100)
        assert z["labels"].dtype == np.float32 and z["inputs"].dtype == np.float32
        # (1, 0): the MOOD loop lowered the cell; (0, 1): it kept the top order
        assert np.array_equal(z["labels"][0], y) and np.array_equal(z["labels"][1], 1 - y)
    x2, y2 = S.load_dataset(tmp_path / "ds.npz")
    assert np.array_equal(x2, x) and np.array_equal(y2, y)


@pytest.mark.gpu
def test_restart_continues_the_run(tmp_path, pkg, oracle):
    """10 steps straight vs 5 steps, snapshot, restart in a new context, 5 steps."""
    p = oracle.make_params(64, 64, bc=17, tmax=0.8)
    U0 = oracle.initial_condition(p, "rp2d3")
    kw = dict(lf=64, nf=64, bc_type=17, tmax=0.8, fp_mode=pkg.FP_EXACT)
    with pkg.Solver(**kw) as s:
        s.Boundary_C(U0, 0.0)
        s.set_state(U0, 0.0)
        s.advance(10)
        ref, tref, _ = s.get_state()
    with pkg.Solver(**kw) as s:
        s.set_state(U0, 0.0)
        s.advance(5)
        s.save_snapshot(tmp_path / "r.npz", problem="2DRP3")
    with pkg.Solver(**kw) as s:
        snap = s.restore(tmp_path / "r.npz")
        assert snap["method"] == "GP_MOOD"
        s.advance(5)
        got, t, _ = s.get_state()
    assert abs(t - tref) <= 1e-12 * tref
    I = (slice(4, -4), slice(4, -4))
    for k in range(4):
        rel = np.abs(got[I + (k,)] - ref[I + (k,)]).sum() / np.abs(ref[I + (k,)]).sum()
        assert rel <= 1e-12, (k, rel)
