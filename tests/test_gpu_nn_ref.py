"""The reference's own network and NN_DETECTION (gpmood_params.nn_reference = 1;
mod_NN.f90:14-58, mod_subroutine_NN_MOOD.f90).

* decisions and outputs against the FP32 restatement in oracle/nn_oracle.py
  (exp rounds differently on the two sides: outputs to 1e-5, decisions equal
  away from ties);
* a network that never fires: CellGPO stays 3 = Mord, so after the first
  nsteps_with_no_nn steps (full DETECTION) the run equals the oracle with DMP
  off (NN_DETECTION keeps only the NaN/positivity checks), bit for bit;
* a network that always fires on a state without constant stencils: every
  cell starts at order 1, which equals the oracle with order-1 initial masks."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import nan_equal

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _nno():
    import __graft_entry__ as ge
    ge.import_oracle()
    import nn_oracle
    return nn_oracle


def _random_net(L, length=60, seed=0, b2=None):
    rng = np.random.default_rng(seed)
    p = np.concatenate([rng.normal(0, 1 / np.sqrt(L), length * L), rng.normal(0, 0.1, length),
                        rng.normal(0, 1 / np.sqrt(length), length * length), rng.normal(0, 0.1, length),
                        rng.normal(0, 1 / np.sqrt(length), 2 * length), rng.normal(0, 0.1, 2)]).astype(np.float32)
    if b2 is not None:
        p[-2:] = b2
    return p


def _wavy(n):
    """A smooth state with no constant stencil anywhere (periodic box [0,1]^2)."""
    x = (np.arange(-3, n + 5) - 0.5) / n
    X, Y = np.meshgrid(x, x)
    U = np.zeros((n + 8, n + 8, 4))
    r = 1.0 + 0.2 * np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y)
    u, v, p = 0.3 * np.cos(2 * np.pi * Y), 0.2 * np.sin(2 * np.pi * X), 1.0 + 0.1 * np.sin(2 * np.pi * (X + Y))
    U[..., 0], U[..., 1], U[..., 2], U[..., 3] = r, r * u, r * v, p / 0.4 + 0.5 * r * (u * u + v * v)
    return U


def test_reference_network_matches_fp32_restatement(pkg, oracle):
    N = _nno()
    n = 64
    p = oracle.make_params(n, n, bc=17, tmax=0.8, mord=3, ngp=2)
    U = oracle.initial_condition(p, "rp2d3")
    st = oracle.Stepper(p)
    t = 0.0
    for _ in range(20):  # a state with shocks and smooth parts
        dt = oracle.setdt(p, U, p.tmax - t)
        Ur = np.empty_like(U)
        st.time_stepping(U, Ur, t, dt)
        t += dt
        U = Ur
    net = _random_net(52, seed=3)
    x, const = N.ref_features(U, 3)
    r = N.ref_forward(net, x)
    with pkg.Solver(lf=n, nf=n, bc_type=17, tmax=0.8, mord=3, ngp=2, method=pkg.NN_GP_MOOD, nn_reference=1) as s:
        s.set_state(U, t)
        s.set_nn(net)
        d = torch.empty(2 * n * n, dtype=torch.float32, device="cuda")
        s.nn_ref_logits(d.data_ptr())
        rg = d.cpu().numpy().reshape(-1, 2)
        gated, cnt = s.nn_predict()
    live = ~const
    assert const.any() and live.any()
    np.testing.assert_allclose(rg[live], r[live], rtol=1e-5, atol=1e-5)
    assert np.all(rg[const] == 0)
    want = (r[:, 0] > r[:, 1]) & live
    clear = np.abs(r[:, 0] - r[:, 1]) > 1e-4
    g = gated.ravel().astype(bool)
    assert np.array_equal(g[clear], want[clear])
    assert cnt == int(g.sum()) and 0 < cnt < n * n


@pytest.mark.parametrize("fire", [False, True])
def test_reference_network_runs_equal_the_oracle(pkg, oracle, fire):
    n, nsteps, warm = 48, 6, 2
    if fire:
        U0 = _wavy(n)
        bc = 18
    else:
        p0 = oracle.make_params(n, n, bc=17, tmax=0.8, mord=3, ngp=2)
        U0 = oracle.initial_condition(p0, "rp2d3")
        bc = 17
    net = _random_net(52, seed=5, b2=[1e3, -1e3] if fire else [-1e3, 1e3])
    full = oracle.make_params(n, n, bc=bc, tmax=0.8, mord=3, ngp=2)
    nn_det = oracle.make_params(n, n, bc=bc, tmax=0.8, mord=3, ngp=2, dmp=0)
    st_full, st_nn = oracle.Stepper(full), oracle.Stepper(nn_det)
    U = U0.copy()
    oracle.boundary(full, U)
    Ug0 = U.copy()
    t = 0.0
    ones = [np.ones((n, n), np.int8)] * 3
    for k in range(nsteps):
        dt = oracle.setdt(full, U, full.tmax - t)
        Ur = np.empty_like(U)
        if k < warm:
            st_full.time_stepping(U, Ur, t, dt)
        else:
            st_nn.time_stepping(U, Ur, t, dt, init_orders=ones if fire else None)
        t += dt
        U = Ur
    with pkg.Solver(lf=n, nf=n, bc_type=bc, tmax=0.8, mord=3, ngp=2, method=pkg.NN_GP_MOOD, nn_reference=1,
                    nsteps_with_no_nn=warm, fp_mode=pkg.FP_EXACT) as s:
        s.set_nn(net)
        s.set_state(Ug0, 0.0)
        assert s.advance(nsteps) == nsteps
        Ug, tg, _ = s.get_state()
        c = s.counters()
    if fire:
        assert c.a_priori_last_step == 3 * n * n
    else:
        assert c.a_priori_last_step == 0
    assert tg == t
    I = (slice(4, -4), slice(4, -4))
    assert nan_equal(Ug[I], U[I]), np.nanmax(np.abs(Ug[I] - U[I]))


def _constant_net(L, length, b2):
    """A network whose outputs are b2 on every cell (zero weights)."""
    p = np.zeros(length * L + length + length * length + length + 2 * length + 2, np.float32)
    p[-2:] = b2
    return p


@pytest.mark.parametrize("fire", [False, True])
def test_convex_combination_method_equals_the_oracle(pkg, oracle, fire):
    """NN_GP_MOOD_CC (mod_NN_GP_MOOD_CC.f90): softmaxed outputs decide the
    orders; order-3 states of column L = 52 (the reference's values_NN(l, ...)
    with l read as L) are blended v1*U + v2*Uh with the row's last-cell pair,
    order-1 states are the cell values.  Exact mode, bit for bit against the
    oracle's blend with the pair the GPU's network produced."""
    n, nsteps = 64, 4
    U0 = _wavy(n)
    net = _constant_net(52, 5, [0.5, -0.5] if fire else [-0.5, 0.5])
    kw = dict(lf=n, nf=n, bc_type=18, tmax=0.8, mord=3, ngp=2, method=pkg.NN_GP_MOOD_CC, nsteps_with_no_nn=0,
              fp_mode=pkg.FP_EXACT)
    p = oracle.make_params(n, n, bc=18, tmax=0.8, mord=3, ngp=2, dmp=0)
    U = U0.copy()
    oracle.boundary(p, U)
    Ug0 = U.copy()
    with pkg.Solver(**kw) as s:
        s.set_nn(net)
        s.set_state(Ug0, 0.0)
        d = torch.empty(2 * n * n, dtype=torch.float32, device="cuda")
        s.nn_ref_logits(d.data_ptr())
        v = d.cpu().numpy().reshape(n, n, 2)
        assert np.allclose(v.sum(axis=-1), 1.0, atol=1e-6)  # softmax pairs
        assert (v[..., 0] > v[..., 1]).all() == fire
        assert s.advance(nsteps) == nsteps
        Ug, tg, _ = s.get_state()
        c = s.counters()
    assert c.a_priori_last_step == (3 * n * n if fire else 0)
    w = np.zeros((n + 2, 2), np.float32)
    w[:, 1] = 1.0
    w[1:n + 1] = v[:, n - 1]  # the pair of each row's last cell (l = lf)
    st = oracle.Stepper(p)
    st.set_cc(52, w)
    ones = [np.ones((n, n), np.int8)] * 3
    t = 0.0
    for _ in range(nsteps):
        dt = oracle.setdt(p, U, p.tmax - t)
        Ur = np.empty_like(U)
        st.time_stepping(U, Ur, t, dt, init_orders=ones if fire else None)
        t += dt
        U = Ur
    assert tg == t
    I = (slice(4, -4), slice(4, -4))
    assert nan_equal(Ug[I], U[I]), np.nanmax(np.abs(Ug[I] - U[I]))
    if not fire:  # the blend acted: the run differs from the same oracle run without it
        st2 = oracle.Stepper(p)
        U2, t2 = Ug0.copy(), 0.0
        for _ in range(nsteps):
            dt = oracle.setdt(p, U2, p.tmax - t2)
            Ur = np.empty_like(U2)
            st2.time_stepping(U2, Ur, t2, dt)
            t2 += dt
            U2 = Ur
        assert not np.array_equal(U2[I], U[I])
