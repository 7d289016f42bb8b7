"""The hand-written CUDA adjoint (gpmood_adj_*) behind torch.autograd.

Workload: isentropic vortex, beta = 5, u = v = 1, 128x128 periodic cells on
[0,10]^2 (the [-5,5]^2 problem shifted to the reference's mesh origin), Mord 5,
ngp 3, 50 SSP-RK3 steps with every step's MOOD order masks and dt frozen,
J = sum(rho^2) dx dy at the last step, gradient with respect to the initial
conserved state, checkpoints every 10 steps.

Checks:
  * frozen replay of the recording reproduces the forward run bit for bit;
  * the CUDA vector-Jacobian product equals FP64 torch autograd of the same
    frozen map (oracle/adjoint_ref.py) to 1e-10 relative (max norm);
  * central differences with eps = 1e-6 along 32 seeded random directions
    match <grad, v> to 2e-6 relative (6e-7 observed: the O(eps^2) truncation);
  * checkpoint spacing does not change the gradient (bitwise);
  * shock problems with lowered orders (Neumann, reflective boundaries) match
    the torch reference as well.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402

pytestmark = pytest.mark.gpu

LF = NF = 128
NSTEPS = 50
EVERY = 10


def _ref():
    ge.import_oracle()
    import adjoint_ref
    return adjoint_ref


def _vortex(pkg, lf=LF, nf=NF, fp_mode=0):
    from gpmood_gb300 import ic
    s = pkg.Solver(lf=lf, nf=nf, lx=10.0, ly=10.0, bc_type=pkg.PERIODIC, tmax=1e30, fp_mode=fp_mode)
    U = ic.isentropic_vortex(lf, nf, 10.0, 10.0, beta=5.0)
    s.Boundary_C(U, 0.0)
    return s, U


def _J(u, dx, dy):
    return (u[4:-4, 4:-4, 0] ** 2).sum() * dx * dy


def _J_exact(u, dx, dy):
    r = u[4:-4, 4:-4, 0].double().cpu().numpy().ravel()
    return math.fsum((r * r).tolist()) * dx * dy


def _torch_ref_grad(pkg, oracle, rec, U0, dx, dy, bc, ngp=3):
    R = _ref()
    p = oracle.make_params(rec.solver.lf, rec.solver.nf, lx=rec.solver.p.lx, ly=rec.solver.p.ly, bc=bc, ngp=ngp)
    zt, gw = R.weights(oracle.gp_weights(p))
    dev = torch.device("cuda:0")
    orders = [[torch.from_numpy(rec.orders(s, k)).to(dev) for k in range(3)] for s in range(rec.nsteps)]
    _, dts = rec.info()
    I0 = torch.from_numpy(U0[4:-4, 4:-4].copy()).to(dev).requires_grad_(True)
    IN = R.steps(I0, orders, [float(d) for d in dts], dx, dy, zt, gw, ngp, bc)
    J = (IN[..., 0] ** 2).sum() * dx * dy
    J.backward()
    return I0.grad.cpu().numpy(), IN.detach().cpu().numpy()


def test_record_replay_and_autograd_function(pkg):
    from gpmood_gb300.adjoint import FrozenMoodSteps, frozen_replay
    s, U = _vortex(pkg)
    dx, dy = 10.0 / LF, 10.0 / NF
    u0 = torch.from_numpy(U).cuda().requires_grad_(True)
    uN = FrozenMoodSteps.apply(u0, s, NSTEPS, EVERY)
    J = _J(uN, dx, dy)
    J.backward()
    g = u0.grad
    assert torch.isfinite(g).all()
    assert float(g[:4].abs().max()) == 0.0 and float(g[:, :4].abs().max()) == 0.0  # ghosts carry no gradient
    # a new recording from the same u0, replayed with frozen masks, gives the same bits
    s2, _ = _vortex(pkg)
    s2.set_state_dev(u0.detach().data_ptr(), 0.0)
    r2 = s2.adj_record(NSTEPS, EVERY)
    assert r2.nsteps == NSTEPS
    with torch.no_grad():
        assert torch.equal(frozen_replay(r2, u0.detach()), uN.detach())
    # and the gradient through the replay Function is the forward Function's
    u1 = u0.detach().clone().requires_grad_(True)
    _J(frozen_replay(r2, u1), dx, dy).backward()
    assert torch.equal(u1.grad, g)


def test_gradient_matches_fp64_torch_autograd(pkg, oracle):
    s, U = _vortex(pkg)
    dx, dy = 10.0 / LF, 10.0 / NF
    s.set_state(U, 0.0)
    rec = s.adj_record(NSTEPS, EVERY)
    lamN = torch.zeros(s.shape, dtype=torch.float64, device="cuda")
    uN = torch.empty_like(lamN)
    s.get_state_dev(uN.data_ptr())
    lamN[4:-4, 4:-4, 0] = 2.0 * uN[4:-4, 4:-4, 0] * dx * dy
    lam0 = torch.empty_like(lamN)
    rec.backward(lamN.data_ptr(), lam0.data_ptr())
    g_cuda = lam0.cpu().numpy()[4:-4, 4:-4]
    g_ref, IN = _torch_ref_grad(pkg, oracle, rec, U, dx, dy, pkg.PERIODIC)
    # the torch forward of the frozen map agrees with the CUDA forward
    uNh = uN.cpu().numpy()[4:-4, 4:-4]
    assert np.abs(IN - uNh).max() <= 1e-12 * np.abs(uNh).max()
    err = np.abs(g_cuda - g_ref).max() / np.abs(g_ref).max()
    print(f"vortex 128^2, 50 steps: max |g_cuda - g_torch| / max |g_torch| = {err:.3e}")
    assert err <= 1e-10


def test_gradient_matches_central_differences(pkg):
    s, U = _vortex(pkg)
    dx, dy = 10.0 / LF, 10.0 / NF
    s.set_state(U, 0.0)
    rec = s.adj_record(NSTEPS, EVERY)
    u0 = torch.from_numpy(U).cuda()
    uN = torch.empty_like(u0)
    rec.replay(u0.data_ptr(), uN.data_ptr())
    lamN = torch.zeros_like(u0)
    lamN[4:-4, 4:-4, 0] = 2.0 * uN[4:-4, 4:-4, 0] * dx * dy
    lam0 = torch.empty_like(u0)
    rec.backward(lamN.data_ptr(), lam0.data_ptr())
    gen = torch.Generator(device="cuda").manual_seed(1234)
    eps = 1e-6
    worst = 0.0
    up, um = torch.empty_like(u0), torch.empty_like(u0)
    for _ in range(32):
        v = torch.zeros_like(u0)
        v[4:-4, 4:-4] = torch.randn((NF, LF, 4), generator=gen, dtype=torch.float64, device="cuda")
        rec.replay((u0 + eps * v).data_ptr(), up.data_ptr())
        rec.replay((u0 - eps * v).data_ptr(), um.data_ptr())
        fd = (_J_exact(up, dx, dy) - _J_exact(um, dx, dy)) / (2 * eps)
        ad = float((lam0 * v).sum())
        rel = abs(fd - ad) / abs(ad)
        worst = max(worst, rel)
        assert rel <= 2e-6, (fd, ad, rel)
    print(f"central differences, 32 directions: worst relative error {worst:.3e}")


def test_checkpoint_spacing_does_not_change_the_gradient(pkg):
    grads = []
    for every in (1, 10, 50):
        s, U = _vortex(pkg, 64, 64)
        s.set_state(U, 0.0)
        rec = s.adj_record(20, every)
        lamN = torch.zeros(s.shape, dtype=torch.float64, device="cuda")
        lamN[4:-4, 4:-4, 0] = 1.0
        lam0 = torch.empty_like(lamN)
        rec.backward(lamN.data_ptr(), lam0.data_ptr())
        grads.append(lam0.cpu())
    assert torch.equal(grads[0], grads[1]) and torch.equal(grads[1], grads[2])


@pytest.mark.parametrize("ic,bc,kw", [
    ("rp2d3", 17, dict(tmax=0.8)),
    ("sedov", 20, dict(tmax=0.05)),
])
def test_shock_problems_with_lowered_orders(pkg, oracle, ic, bc, kw):
    lf = nf = 64
    p = oracle.make_params(lf, nf, bc=bc, **kw)
    U = oracle.initial_condition(p, ic)
    s = pkg.Solver(lf=lf, nf=nf, bc_type=bc, tmax=kw["tmax"], fp_mode=0)
    s.set_state(U, 0.0)
    rec = s.adj_record(6, 3)
    lowered = sum(int((rec.orders(i, k)[4:-4, 4:-4] < 5).sum()) for i in range(rec.nsteps) for k in range(3))
    assert lowered > 0
    dx, dy = 1.0 / lf, 1.0 / nf
    u0 = torch.from_numpy(U).cuda()
    uN = torch.empty_like(u0)
    rec.replay(u0.data_ptr(), uN.data_ptr())
    lamN = torch.zeros_like(u0)
    lamN[4:-4, 4:-4, 0] = 2.0 * uN[4:-4, 4:-4, 0] * dx * dy
    lam0 = torch.empty_like(u0)
    rec.backward(lamN.data_ptr(), lam0.data_ptr())
    g_ref, _ = _torch_ref_grad(pkg, oracle, rec, U, dx, dy, bc)
    g_cuda = lam0.cpu().numpy()[4:-4, 4:-4]
    err = np.abs(g_cuda - g_ref).max() / np.abs(g_ref).max()
    print(f"{ic}: {lowered} lowered stage orders, relative gradient error {err:.3e}")
    assert err <= 1e-10
