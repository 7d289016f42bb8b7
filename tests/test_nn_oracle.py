"""The CPU reference of the MLP gate (oracle/nn_oracle.py): its BF16 rounding,
features and analytic gradient, checked on the CPU."""
from __future__ import annotations

import numpy as np
import pytest


@pytest.fixture(scope="module")
def nno():
    import __graft_entry__ as ge
    ge.import_oracle()
    import nn_oracle
    return nn_oracle


def test_bf16_rounding(nno):
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.14159265, 1e-20, 65504.0], dtype=np.float32)
    b = nno.bf16(x)
    assert b[0] == 1.0 and b[3] == -2.5
    assert b[1] == 1.0            # tie 1 + 2^-8 rounds to even (1.0)
    assert b[2] == np.float32(1.0078125)
    assert abs(b[4] - 3.140625) < 1e-7
    assert np.all((b.view(np.uint32) & 0xFFFF) == 0)


def test_features_definition(nno, oracle):
    p = oracle.make_params(32, 32, bc=17)
    U = oracle.initial_condition(p, "rp2d3")
    x, cst = nno.features(U, 32, 32)
    assert x.shape == (32 * 32, 36) and x.dtype == np.float32
    # a cell in the lower-left quadrant is constant; one next to the x-split is not
    assert cst[0]
    i = 5 * 32 + 25  # (l, n) = (26, 6): the split at x = 0.8 lies between cells 25 and 26
    assert not cst[i]
    # feature v*9 + j is variable v at cross point j divided by the stencil max-abs of v
    l, n = 26, 6
    pts = [U[4 + n - 1 + dy, 4 + l - 1 + dx].astype(np.float32) for dx, dy in nno.CROSS]
    q = np.stack(pts, axis=1)  # [4, 9]
    ref = q * (np.float32(1.0) / np.abs(q).max(axis=1, keepdims=True))
    assert np.array_equal(x[i].reshape(4, 9), ref)
    assert np.all(np.abs(x) <= 1.0 + 1e-7)


def test_gradient_matches_finite_differences(nno):
    rng = np.random.default_rng(1)
    n = 64
    x = rng.uniform(-1, 1, size=(n, 36)).astype(np.float32)
    y = (rng.uniform(size=n) < 0.3).astype(np.float32)
    p = rng.uniform(-0.3, 0.3, size=nno.NPARAMS)
    loss, g = nno.loss_grad(p, x, y, pos_weight=2.0, emulate_bf16=False)
    for idx in rng.choice(p.size, 40, replace=False):
        e = np.zeros_like(p)
        e[idx] = 1e-6
        lp, _ = nno.loss_grad(p + e, x, y, 2.0, emulate_bf16=False)
        lm, _ = nno.loss_grad(p - e, x, y, 2.0, emulate_bf16=False)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(g).max()), (idx, fd, g[idx])
