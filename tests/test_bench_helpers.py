"""bench.py's host-side helpers on CPU: the L1 error against a twice finer run
and the relative L1 difference used by the whole-run reports."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def padded(field):
    nf, lf = field.shape
    U = np.zeros((nf + 8, lf + 8, 4))
    U[4:-4, 4:-4, 0] = field
    U[4:-4, 4:-4, 1:] = 1.0
    return U


def test_l1_error_against_block_averages_of_the_finer_run():
    rng = np.random.default_rng(3)
    fine = rng.uniform(0.5, 2.0, size=(8, 16))
    coarse_exact = fine.reshape(4, 2, 8, 2).mean(axis=(1, 3))
    lx, ly = 4.0, 1.0
    assert bench.l1_density_error(padded(coarse_exact), padded(fine), lx, ly) == 0.0
    bumped = coarse_exact.copy()
    bumped[1, 2] += 0.25
    # one cell off by 0.25, cell area (4/8) * (1/4)
    assert abs(bench.l1_density_error(padded(bumped), padded(fine), lx, ly) - 0.25 * 0.5 * 0.25) < 1e-15


def test_relative_l1_per_field():
    a = padded(np.full((4, 4), 2.0))
    b = padded(np.full((4, 4), 1.0))
    rel = bench._rel_l1(a, b)
    assert rel[0] == 1.0 and rel[1:] == [0.0, 0.0, 0.0]
