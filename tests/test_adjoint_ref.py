"""The FP64 torch autograd reference of the frozen-mask step (oracle/adjoint_ref.py),
pinned to the CPU oracle on CPU: with the oracle's own per-stage order masks
and dt, its steps reproduce the oracle's states; its gradient matches central
differences of itself."""
from __future__ import annotations

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402


def _ref():
    ge.import_oracle()
    import adjoint_ref
    return adjoint_ref


def _oracle_run(oracle, ic, lf, nf, nsteps, **kw):
    p = oracle.make_params(lf, nf, **kw)
    U = oracle.initial_condition(p, ic)
    U0 = U.copy()
    st = oracle.Stepper(p)
    t = 0.0
    orders, dts = [], []
    for _ in range(nsteps):
        dt = oracle.setdt(p, U, p.tmax - t)
        Ur = np.empty_like(U)
        masks = st.time_stepping(U, Ur, t, dt, want_orders=True)
        pad = []
        for m in masks:  # ghost cells keep CellGPO = Mord
            o = np.full((nf + 8, lf + 8), p.mord, dtype=np.int8)
            o[4:-4, 4:-4] = m
            pad.append(torch.from_numpy(o))
        orders.append(pad)
        dts.append(dt)
        t += dt
        U = Ur
    return p, U0, U, orders, dts


@pytest.mark.parametrize("ic,lf,nf,kw", [
    ("vortex", 32, 32, dict(bc=18, lx=10.0, ly=10.0, tmax=1.0)),
    ("rp2d3", 32, 32, dict(bc=17, tmax=0.8)),
    ("sedov", 32, 32, dict(bc=20, tmax=0.05)),
])
def test_reference_steps_match_oracle(oracle, ic, lf, nf, kw):
    R = _ref()
    p, U0, UN, orders, dts = _oracle_run(oracle, ic, lf, nf, 4, **kw)
    zt, gw = R.weights(oracle.gp_weights(p))
    dx, dy = p.lx / lf, p.ly / nf
    I0 = torch.from_numpy(U0[4:-4, 4:-4].copy())
    IN = R.steps(I0, orders, dts, dx, dy, zt, gw, p.ngp, p.bc_type).numpy()
    ref = UN[4:-4, 4:-4]
    assert any((o[4:-4, 4:-4] < p.mord).any() for oo in orders for o in oo) or ic == "vortex"
    for k in range(4):
        err = np.abs(IN[..., k] - ref[..., k]).sum() / np.abs(ref[..., k]).sum()
        assert err <= 1e-13, (k, err)


def test_reference_gradient_matches_central_differences(oracle):
    R = _ref()
    p, U0, _, orders, dts = _oracle_run(oracle, "vortex", 16, 16, 2, bc=18, lx=10.0, ly=10.0, tmax=1.0)
    zt, gw = R.weights(oracle.gp_weights(p))
    dx, dy = p.lx / 16, p.ly / 16

    def J(I):
        IN = R.steps(I, orders, dts, dx, dy, zt, gw, p.ngp, p.bc_type)
        return (IN[..., 0] ** 2).sum() * dx * dy

    I0 = torch.from_numpy(U0[4:-4, 4:-4].copy()).requires_grad_(True)
    J(I0).backward()
    g = I0.grad
    gen = torch.Generator().manual_seed(0)
    eps = 1e-6
    for _ in range(4):
        v = torch.randn(I0.shape, generator=gen, dtype=torch.float64)
        with torch.no_grad():
            jp = R.steps(I0 + eps * v, orders, dts, dx, dy, zt, gw, p.ngp, p.bc_type)[..., 0]
            jm = R.steps(I0 - eps * v, orders, dts, dx, dy, zt, gw, p.ngp, p.bc_type)[..., 0]
        fd = (math.fsum((jp ** 2).flatten().tolist()) - math.fsum((jm ** 2).flatten().tolist())) * dx * dy / (2 * eps)
        ad = float((g * v).sum())
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_reference_gradient_is_finite_with_lowered_orders(oracle):
    R = _ref()
    p, U0, _, orders, dts = _oracle_run(oracle, "rp2d3", 32, 32, 3, bc=17, tmax=0.8)
    assert any((o[4:-4, 4:-4] < p.mord).any() for oo in orders for o in oo)
    zt, gw = R.weights(oracle.gp_weights(p))
    I0 = torch.from_numpy(U0[4:-4, 4:-4].copy()).requires_grad_(True)
    IN = R.steps(I0, orders, dts, 1 / 32, 1 / 32, zt, gw, p.ngp, p.bc_type)
    ((IN[..., 0] ** 2).sum()).backward()
    assert torch.isfinite(I0.grad).all()
