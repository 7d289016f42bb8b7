"""The a-priori MLP gate on the GPU: features, BF16 tensor-core forward and
backward checked against the CPU oracle (oracle/nn_oracle.py), Adam, the
training-sample harvest, and what a trained gate gains over plain GP-MOOD."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def nno(oracle):
    import nn_oracle
    return nn_oracle


def _state(oracle, ic, lf, nf, bc, tmax, steps):
    p = oracle.make_params(lf, nf, bc=bc, tmax=tmax)
    U = oracle.initial_condition(p, ic)
    if steps:
        oracle.Stepper(p).run(U, 0.0, steps)
    return U


def test_features_match_oracle(pkg, oracle, nno):
    lf = nf = 64
    U = _state(oracle, "rp2d3", lf, nf, 17, 0.8, 3)
    with pkg.Solver(lf=lf, nf=nf, bc_type=17) as s:
        s.set_state(U, 0.0)
        x = torch.empty((lf * nf, 36), dtype=torch.float32, device="cuda")
        c = torch.empty((lf * nf,), dtype=torch.int8, device="cuda")
        s.nn_features(x.data_ptr(), c.data_ptr())
    xr, cr = nno.features(U, lf, nf)
    assert np.array_equal(x.cpu().numpy(), xr)
    assert np.array_equal(c.cpu().numpy().astype(bool), cr)


def _params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    parts = []
    for fi, fo in ((36, 64), (64, 64), (64, 1)):
        b = scale / np.sqrt(fi)
        parts += [rng.uniform(-b, b, fi * fo), rng.uniform(-b, b, fo)]
    return np.concatenate(parts).astype(np.float32)


def test_forward_and_gradient_match_oracle(pkg, nno):
    from gpmood_gb300 import nn_train as T
    rng = np.random.default_rng(5)
    n = 1000  # not a multiple of the 128-row CTA tile
    x = rng.uniform(-1, 1, size=(n, 36)).astype(np.float32)
    y = (rng.uniform(size=n) < 0.25).astype(np.float32)
    p = _params(7, scale=2.0)
    dp, dx, dy = (torch.from_numpy(a).cuda() for a in (p, x, y))
    z = torch.empty(n, dtype=torch.float32, device="cuda")
    T.forward(dp.data_ptr(), dx.data_ptr(), n, z.data_ptr())
    zr, _ = nno.forward(p, x, emulate_bf16=True)
    np.testing.assert_allclose(z.cpu().numpy(), zr, rtol=2e-3, atol=2e-3)
    g = torch.empty_like(dp)
    loss = torch.empty(1, dtype=torch.float32, device="cuda")
    T.loss_grad(dp.data_ptr(), dx.data_ptr(), dy.data_ptr(), n, g.data_ptr(), loss.data_ptr(), pos_weight=3.0)
    lr_, gr = nno.loss_grad(p, x, y, 3.0, emulate_bf16=True)
    gg = g.cpu().numpy().astype(np.float64)
    assert abs(loss.item() - lr_) <= 1e-4 * abs(lr_)
    rel = np.linalg.norm(gg - gr) / np.linalg.norm(gr)
    assert rel < 1e-2, rel
    # and against the exact FP64 gradient of the same network
    _, g64 = nno.loss_grad(p, x, y, 3.0, emulate_bf16=False)
    rel64 = np.linalg.norm(gg - g64) / np.linalg.norm(g64)
    assert rel64 < 5e-2, rel64


def test_adam_step(pkg):
    from gpmood_gb300 import nn_train as T
    rng = np.random.default_rng(2)
    p = rng.normal(size=6593).astype(np.float32)
    g = rng.normal(size=6593).astype(np.float32)
    m = rng.normal(size=6593).astype(np.float32) * 0.1
    v = rng.uniform(size=6593).astype(np.float32) * 0.1
    dp, dg, dm, dv = (torch.from_numpy(a.copy()).cuda() for a in (p, g, m, v))
    T.adam(dp.data_ptr(), dg.data_ptr(), dm.data_ptr(), dv.data_ptr(), 3, 1e-3)
    b1, b2, eps = 0.9, 0.999, 1e-8
    m1 = b1 * m + (1 - b1) * g
    v1 = b2 * v + (1 - b2) * g * g
    lr_t = 1e-3 * np.sqrt(1 - b2 ** 3) / (1 - b1 ** 3)
    p1 = p - lr_t * m1 / (np.sqrt(v1) + eps)
    np.testing.assert_allclose(dp.cpu().numpy(), p1, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(dm.cpu().numpy(), m1, rtol=1e-5, atol=1e-7)


def test_gate_decision_matches_oracle(pkg, oracle, nno):
    lf = nf = 64
    U = _state(oracle, "rp2d3", lf, nf, 17, 0.8, 3)
    p = _params(11, scale=2.0)
    with pkg.Solver(lf=lf, nf=nf, bc_type=17, method=pkg.NN_GP_MOOD) as s:
        s.set_state(U, 0.0)
        s.set_nn(p)
        mask, cnt = s.nn_predict()
    x, cst = nno.features(U, lf, nf)
    z, _ = nno.forward(p, x, emulate_bf16=True)
    ref = (z > 0) & ~cst
    got = mask.ravel().astype(bool)
    assert cnt == int(got.sum())
    diff = got != ref
    assert np.all(np.abs(z[diff]) < 1e-2), z[diff]
    assert ref.sum() > 0 and (~ref & ~cst).sum() > 0


@pytest.mark.parametrize("ic,bc,tmax,steps", [("rp2d3", 17, 0.8, 3), ("sedov", 20, 0.05, 6)])
def test_tensor_core_gate_logits_match_oracle(pkg, oracle, nno, ic, bc, tmax, steps):
    """The tcgen05 gate (TMEM accumulators) against the BF16-emulating numpy
    forward: same roundings of inputs, weights and hidden activations, FP32
    sums in another order (tolerance as the training forward's).  300x200 is
    not a multiple of the 128-cell tile."""
    lf, nf = 300, 200
    U = _state(oracle, ic, lf, nf, bc, tmax, steps)
    p = _params(13, scale=2.0)
    with pkg.Solver(lf=lf, nf=nf, bc_type=bc, method=pkg.NN_GP_MOOD) as s:
        s.set_state(U, 0.0)
        s.set_nn(p)
        z = torch.full((lf * nf,), float("nan"), dtype=torch.float32, device="cuda")
        s.nn_gate_logits(z.data_ptr())
        zg = z.cpu().numpy()
        mask, cnt = s.nn_predict()
    x, cst = nno.features(U, lf, nf)
    zr, _ = nno.forward(p, x, emulate_bf16=True)
    assert np.all(zg[cst] == 0)
    np.testing.assert_allclose(zg[~cst], zr[~cst], rtol=2e-3, atol=2e-3)
    got = mask.ravel().astype(bool)
    assert np.array_equal(got, (zg > 0) & ~cst) and cnt == int(got.sum())


def test_harvest_labels_are_the_stage1_mood_decisions(pkg, oracle, nno):
    lf = nf = 64
    U = _state(oracle, "sedov", lf, nf, 20, 0.05, 4)
    x = torch.zeros((lf * nf, 36), dtype=torch.float32, device="cuda")
    y = torch.zeros((lf * nf,), dtype=torch.float32, device="cuda")
    cnt = torch.zeros((1,), dtype=torch.int32, device="cuda")
    with pkg.Solver(lf=lf, nf=nf, bc_type=20, tmax=0.05) as s:
        s.set_state(U, 0.0)
        s.nn_harvest(x.data_ptr(), y.data_ptr(), lf * nf, 1.0, 3, cnt.data_ptr())
        s.advance(1)
        s.nn_harvest(0, 0, 0, 0.0, 0, 0)
        o1 = s.stage_orders(0)
    xr, cst = nno.features(U, lf, nf)
    n = int(cnt.item())
    assert n == int((~cst).sum())
    lab = (o1.ravel() < 5)[~cst]
    # the harvest appends in arbitrary order: compare as multisets of (features, label)
    got = np.concatenate([x[:n].cpu().numpy(), y[:n].cpu().numpy()[:, None]], axis=1)
    ref = np.concatenate([xr[~cst], lab[:, None].astype(np.float32)], axis=1)
    key = lambda a: a[np.lexsort(a.T[::-1])]
    assert np.array_equal(key(got), key(ref))
    assert lab.sum() > 0


def test_training_on_plain_mood_labels_and_gate_gain(pkg):
    """Harvest stage-1 labels from plain GP-MOOD runs, train the gate with the
    library's BF16 kernels, then run the same problem plain and gated: the
    trained gate must catch troubled cells up front (fewer a-posteriori
    detections than plain) while the solution stays close to plain's."""
    from gpmood_gb300 import ic, nn_train as T
    n = 128
    runs = [(ic.rp2d3(n, n), dict(lf=n, nf=n, bc_type=17, tmax=0.8)),
            (ic.sedov(n, n), dict(lf=n, nf=n, bc_type=20, tmax=0.05))]
    ds = T.harvest(runs, capacity=400_000, keep_negative=0.05, steps_per_run=60, seed=1)
    assert ds.n > 10_000 and 0.05 < ds.positives / ds.n < 0.95, (ds.n, ds.positives)
    p0 = T.init_params(0)
    p, hist = T.train(ds, p0, epochs=6, batch=2048, lr=3e-3, pos_weight=1.0)
    assert hist[-1][1] < 0.6 * hist[0][1], hist[:: max(1, len(hist) // 8)]
    m = T.evaluate(ds, p)
    assert m["recall"] > 0.8 and m["accuracy"] > 0.85, m

    def run(method):
        with pkg.Solver(lf=n, nf=n, bc_type=17, tmax=0.8, method=method, fp_mode=pkg.FP_FAST) as s:
            U = ic.rp2d3(n, n)
            s.Boundary_C(U, 0.0)
            s.set_state(U, 0.0)
            if method == pkg.NN_GP_MOOD:
                s.set_nn(p)
            post, prior = 0, 0
            for _ in range(40):
                s.advance(1)
                c = s.counters()
                post += c.detected_last_step
                prior += c.a_priori_last_step
            U1, t, _ = s.get_state()
        return U1, t, post, prior

    Up, tp, post_p, _ = run(pkg.GP_MOOD)
    Ug, tg, post_g, prior_g = run(pkg.NN_GP_MOOD)
    assert prior_g > 0
    assert post_g < post_p, (post_g, post_p)
    I = (slice(4, -4), slice(4, -4), 0)
    rel = np.abs(Ug[I] - Up[I]).sum() / np.abs(Up[I]).sum()
    assert rel < 1e-2, rel


def test_gate_extras_repair_gives_orders_back(pkg):
    """gpmood_set_nn_repair: a gated cell whose uniform-order update passes
    DETECTION gets Mord back, so fewer cells start lowered; the run stays near
    plain GP-MOOD (how near, against the gated run without the repair, depends
    on the problem: closer on this one over 40 steps)."""
    from gpmood_gb300 import ic, nn_train as T
    from pathlib import Path
    gate = Path(__file__).resolve().parents[1] / "gp-mood_gb300" / "gates" / "gate_sedov_rp2d3.txt"
    import json
    params = T.load_text(str(gate))
    thr = float(json.loads(gate.with_suffix(".json").read_text())["threshold"])
    n = 128
    U0 = ic.rp2d3(n, n)

    def run(method, repair=False):
        with pkg.Solver(lf=n, nf=n, bc_type=17, tmax=0.8, method=method, fp_mode=pkg.FP_FAST) as s:
            s.Boundary_C(U0, 0.0)
            s.set_state(U0, 0.0)
            if method == pkg.NN_GP_MOOD:
                s.set_nn(params)
                s.set_nn_threshold(thr)
                s.set_nn_repair(repair)
            prior = 0
            for _ in range(40):
                s.advance(1)
                prior += s.counters().a_priori_last_step
            U, t, _ = s.get_state()
        return U, prior

    Up, _ = run(pkg.GP_MOOD)
    Ug, prior_g = run(pkg.NN_GP_MOOD)
    Ur, prior_r = run(pkg.NN_GP_MOOD, repair=True)
    assert 0 < prior_r < prior_g, (prior_r, prior_g)
    I = (slice(4, -4), slice(4, -4), 0)
    rel = lambda a: np.abs(a[I] - Up[I]).sum() / np.abs(Up[I]).sum()
    assert rel(Ur) <= rel(Ug), (rel(Ur), rel(Ug))
