"""Batched stepping of many problems of uneven size (gpmood_batch_*): every
problem of a batch must evolve exactly as it does alone in its own context
(bit for bit in the exact mode; to rounding in the fast mode)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problems(pkg, seeds, sizes):
    from gpmood_gb300 import ic
    out = []
    for sd in seeds:
        U, n = ic.random_riemann(sd, sizes)
        with pkg.Solver(lf=n, nf=n, bc_type=17, tmax=1e30) as s:
            s.Boundary_C(U, 0.0)
        out.append((U, n))
    return out


@pytest.mark.parametrize("fp_mode", [0, 1])
def test_batch_equals_single_problem_runs(pkg, fp_mode):
    probs = _problems(pkg, range(7), (32, 48, 64))
    sizes = [(n, n) for _, n in probs]
    nsteps = 6
    with pkg.Batch(sizes, lf=32, nf=32, bc_type=17, tmax=1e30, fp_mode=fp_mode) as b:
        for i, (U, _) in enumerate(probs):
            b.set_state(i, U, 0.0)
        b.advance(nsteps)
        st = b.stats()
        assert st["steps"] == nsteps and st["status"] == 0
        assert st["interior_cells"] == sum(n * n for _, n in probs)
        got = [b.get_state(i) for i in range(len(probs))]
    for i, (U, n) in enumerate(probs):
        with pkg.Solver(lf=n, nf=n, bc_type=17, tmax=1e30, fp_mode=fp_mode) as s:
            s.set_state(U, 0.0)
            assert s.advance(nsteps) == nsteps
            Us, ts, _ = s.get_state()
        Ub, tb = got[i]
        I = (slice(4, -4), slice(4, -4))
        if fp_mode == 0:
            assert tb == ts, (i, tb, ts)
            assert np.array_equal(Ub[I], Us[I]), (i, np.abs(Ub - Us).max())
        else:
            assert abs(tb - ts) <= 1e-14 * ts, (i, tb, ts)
            # FMA contraction is the compiler's choice per kernel, so the
            # batched and single-problem kernels may round differently
            for k in range(4):
                rel = np.abs(Ub[I + (k,)] - Us[I + (k,)]).sum() / np.abs(Us[I + (k,)]).sum()
                assert rel <= 1e-13, (i, k, rel)


def test_autotune_keeps_results(pkg):
    probs = _problems(pkg, range(10, 16), (32, 64))
    sizes = [(n, n) for _, n in probs]
    finals = []
    for tune in (False, True):
        with pkg.Batch(sizes, lf=32, nf=32, bc_type=17, tmax=1e30, fp_mode=0) as b:
            for i, (U, _) in enumerate(probs):
                b.set_state(i, U, 0.0)
            if tune:
                k, ms = b.autotune()
                assert 0 <= k < 4 and np.all(ms[:4] > 0) and ms[4] == 0  # exact mode: no cell tile
            b.advance(4)
            finals.append([b.get_state(i)[0] for i in range(len(probs))])
            graphed = b.stats()["graphed"]
    assert graphed in (1, -1)
    for a, c in zip(*finals):
        assert np.array_equal(a, c)
