"""Parity of the CUDA path against the CPU oracle, through the C ABI.

FP_EXACT: bit-identical states, time steps and MOOD order masks.
FP_FAST : per-field relative L1 <= 1e-12 and identical MOOD order masks after
          10 steps (the tolerance of the design target)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import nan_equal

pytestmark = pytest.mark.gpu

CASES = {
    # name: (ic, lf, nf, knobs)
    "rp2d3": ("rp2d3", 64, 64, dict(bc=17, tmax=0.8)),
    "sedov": ("sedov", 64, 64, dict(bc=20, tmax=0.05)),
    "dmr": ("dmr", 96, 24, dict(bc=35, lx=4.0, ly=1.0, tmax=0.2)),
    "vortex": ("vortex", 48, 48, dict(bc=18, lx=10.0, ly=10.0, tmax=1.0)),
    "rp2d3_r1": ("rp2d3", 64, 64, dict(bc=17, tmax=0.8, mord=3, ngp=2)),
    # ragged sizes: no dimension a multiple of the 32x8 face tile
    "ragged": ("rp2d3", 37, 19, dict(bc=17, tmax=0.8)),
    "ragged_periodic": ("vortex", 33, 41, dict(bc=18, lx=10.0, ly=10.0, tmax=1.0)),
    # smaller than one tile in both directions
    "tiny": ("rp2d3", 8, 6, dict(bc=17, tmax=0.8)),
    # the polynomial reconstruction of pol_presim with and without MOOD (method 200, 201)
    "pol_mood": ("rp2d3", 48, 48, dict(bc=17, tmax=0.8, mord=3, ngp=2, method=200)),
    "unlim_pol": ("vortex", 48, 48, dict(bc=18, lx=10.0, ly=10.0, tmax=1.0, mord=3, ngp=2, method=201)),
}


def _solver(pkg, lf, nf, fp_mode, kn):
    kw = dict(lf=lf, nf=nf, fp_mode=fp_mode, tmax=kn.get("tmax", 0.8), bc_type=kn.get("bc", 17),
              lx=kn.get("lx", 1.0), ly=kn.get("ly", 1.0), mord=kn.get("mord", 5), ngp=kn.get("ngp", 3))
    for k in ("method", "dmp", "u2", "u2_tol", "max_mood_iters"):
        if k in kn:
            kw[k] = kn[k]
    return pkg.Solver(**kw)


def _oracle_params(oracle, lf, nf, kn):
    kw = dict(kn)
    bc = kw.pop("bc", 17)
    kw.pop("max_mood_iters", None)
    return oracle.make_params(lf, nf, bc=bc, **kw)


def _run_pair(pkg, oracle, case, nsteps, fp_mode):
    ic, lf, nf, kn = CASES[case]
    p = _oracle_params(oracle, lf, nf, kn)
    U = oracle.initial_condition(p, ic)
    st = oracle.Stepper(p)
    Ug = U.copy()
    t = 0.0
    with _solver(pkg, lf, nf, fp_mode, kn) as s:
        for step in range(nsteps):
            dt = oracle.setdt(p, U, p.tmax - t)
            dtg = s.Setdt(Ug, p.tmax - t)
            Ur = np.empty_like(U)
            masks = st.time_stepping(U, Ur, t, dt, want_orders=True)
            Ugr = np.empty_like(Ug)
            s.time_stepping(Ug, Ugr, t, dtg)
            yield step, (U, Ur, dt, masks[2]), (Ugr, dtg, s.orders(), s.counters()), st
            t += dt
            U, Ug = Ur, Ugr


@pytest.mark.parametrize("case", list(CASES))
def test_exact_mode_bitwise(pkg, oracle, case):
    nsteps = 10 if case != "dmr" else 6
    for step, (U, Ur, dt, mask), (Ugr, dtg, mask_g, ctr), st in _run_pair(pkg, oracle, case, nsteps, pkg.FP_EXACT):
        assert dtg == dt, (step, dtg, dt)
        assert np.array_equal(mask_g, mask), f"order mask differs at step {step}"
        assert nan_equal(Ugr, Ur), f"state differs at step {step}: max |d| = {np.nanmax(np.abs(Ugr - Ur))}"


@pytest.mark.parametrize("case", ["rp2d3", "sedov", "vortex", "dmr", "ragged", "tiny"])
def test_fast_mode_tolerance(pkg, oracle, case):
    ic, lf, nf, kn = CASES[case]
    p = _oracle_params(oracle, lf, nf, kn)
    U = oracle.initial_condition(p, ic)
    st = oracle.Stepper(p)
    t = 0.0
    masks = []
    for _ in range(10):
        dt = oracle.setdt(p, U, p.tmax - t)
        Ur = np.empty_like(U)
        masks.append(st.time_stepping(U, Ur, t, dt, want_orders=True)[2])
        t += dt
        U = Ur
    U0 = oracle.initial_condition(p, ic)
    with _solver(pkg, lf, nf, pkg.FP_FAST, kn) as s:
        s.set_state(U0, 0.0)
        assert s.advance(10) == 10
        Ug, tg, n = s.get_state()
        mask_g = s.orders()
    assert n == 10
    assert abs(tg - t) <= 1e-12 * t
    interior = (slice(4, -4), slice(4, -4))
    for k in range(4):
        ref = U[interior + (k,)]
        num = np.abs(Ug[interior + (k,)] - ref).sum()
        den = np.abs(ref).sum()
        assert num <= 1e-12 * den, (k, num / den)
    assert np.array_equal(mask_g, masks[-1])


def test_device_resident_advance_matches_oracle_run(pkg, oracle):
    """gpmood_advance (Setdt fused into the last RK combination) == the main.f90 loop."""
    ic, lf, nf, kn = CASES["sedov"]
    p = _oracle_params(oracle, lf, nf, kn)
    U = oracle.initial_condition(p, ic)
    U0 = U.copy()
    t, n = oracle.Stepper(p).run(U, 0.0, 12)
    with _solver(pkg, lf, nf, pkg.FP_EXACT, kn) as s:
        s.set_state(U0, 0.0)
        assert s.advance(12) == 12
        Ug, tg, ng = s.get_state()
    assert (ng, tg) == (n, t)
    assert nan_equal(Ug, U)


def test_run_stops_at_tmax(pkg, oracle):
    ic, lf, nf, kn = CASES["sedov"]
    kn = dict(kn, tmax=2e-5)
    p = _oracle_params(oracle, lf, nf, kn)
    U = oracle.initial_condition(p, ic)
    U0 = U.copy()
    t, n = oracle.Stepper(p).run(U, 0.0, 1000)
    with _solver(pkg, lf, nf, pkg.FP_EXACT, kn) as s:
        s.set_state(U0, 0.0)
        assert s.advance(1000) == n
        Ug, tg, _ = s.get_state()
    assert tg == t == 2e-5
    assert nan_equal(Ug, U)


def test_boundary_c_matches_oracle(pkg, oracle):
    rng = np.random.default_rng(0)
    for bc, lx, ly in ((17, 1., 1.), (18, 1., 1.), (20, 1., 1.), (35, 4., 1.), (19, 9., 1.), (201, 1.5, 1.5),
                       (301, 1.5, 1.5), (401, 6., 1.), (402, 0.25, 1.), (403, 1., 1.)):
        p = oracle.make_params(40, 24, bc=bc, lx=lx, ly=ly)
        U = rng.uniform(0.5, 2.0, size=oracle.padded(40, 24).shape)
        Ug = U.copy()
        oracle.boundary(p, U, 0.013)
        with pkg.Solver(lf=40, nf=24, bc_type=bc, lx=lx, ly=ly) as s:
            s.Boundary_C(Ug, 0.013)
        assert np.array_equal(U, Ug), bc


def test_gp_se_mode(pkg, oracle):
    """method GP_SE (MOOD off): unlimited R2 reconstruction, same bits."""
    ic, lf, nf, kn = CASES["vortex"]
    kn = dict(kn, method=202)
    p = _oracle_params(oracle, lf, nf, kn)
    U = oracle.initial_condition(p, ic)
    dt = oracle.setdt(p, U, p.tmax)
    Ur = np.empty_like(U)
    oracle.Stepper(p).time_stepping(U.copy(), Ur, 0.0, dt)
    with _solver(pkg, lf, nf, pkg.FP_EXACT, kn) as s:
        Ug = np.empty_like(U)
        s.time_stepping(U, Ug, 0.0, dt)
    assert nan_equal(Ug, Ur)


def test_mood_cap_is_an_error_and_the_context_survives(pkg, oracle):
    """A MOOD loop stopped by max_mood_iters returns GPMOOD_E_MOOD_CAP (no hang,
    no fault); the same problem then steps normally with the default cap."""
    ic, lf, nf, kn = CASES["rp2d3"]
    p = _oracle_params(oracle, lf, nf, kn)
    U = oracle.initial_condition(p, ic)
    dt = oracle.setdt(p, U, p.tmax)
    with _solver(pkg, lf, nf, pkg.FP_EXACT, dict(kn, max_mood_iters=1)) as s:
        out = np.empty_like(U)
        with pytest.raises(pkg.GpmoodError) as e:
            s.time_stepping(U, out, 0.0, dt)
        assert e.value.code == -3
        assert s.counters().status_flags & 2
    ref = np.empty_like(U)
    oracle.Stepper(p).time_stepping(U.copy(), ref, 0.0, dt)
    with _solver(pkg, lf, nf, pkg.FP_EXACT, kn) as s:
        out = np.empty_like(U)
        s.time_stepping(U, out, 0.0, dt)
        assert s.counters().max_passes_stage > 1
    assert nan_equal(out, ref)


def test_one_call_step_equals_the_two_calls(pkg, oracle):
    """gpmood_setdt_time_stepping = gpmood_setdt + gpmood_time_stepping, bit for bit."""
    p = oracle.make_params(48, 40, bc=17, tmax=0.8)
    U = oracle.initial_condition(p, "rp2d3")
    kw = dict(lf=48, nf=40, bc_type=17, tmax=0.8, fp_mode=pkg.FP_EXACT)
    with pkg.Solver(**kw) as a, pkg.Solver(**kw) as b:
        Ua, Ub, ta, tb = U.copy(), U.copy(), 0.0, 0.0
        for _ in range(4):
            dta = a.Setdt(Ua, 0.8 - ta)
            Ura = np.empty_like(Ua)
            a.time_stepping(Ua, Ura, ta, dta)
            Urb = np.empty_like(Ub)
            dtb = b.setdt_time_stepping_ptr(Ub.ctypes.data, Urb.ctypes.data, tb, 0.8 - tb)
            assert dtb == dta
            assert nan_equal(Urb, Ura)
            ta += dta
            tb += dtb
            Ua, Ub = Ura, Urb


@pytest.mark.parametrize("bad", ["negative_pressure", "nan_density"])
def test_inadmissible_state_is_caught_and_reported(pkg, oracle, bad):
    """An inadmissible cell planted in the initial array (fault injection on
    the host, no GPU fault): MOOD lowers the cells around it to first order,
    the bad values stay in order-1 cells, the step equals the oracle bit for
    bit, and status bit 0 reports the state left in an order-1 cell without
    failing the call."""
    ic, lf, nf, kn = CASES["rp2d3"]
    p = _oracle_params(oracle, lf, nf, kn)
    U = oracle.initial_condition(p, ic)
    dt = oracle.setdt(p, U, p.tmax)
    j, i = 4 + 20, 4 + 30  # interior cell (l, n) = (31, 21)
    if bad == "negative_pressure":
        U[j, i, 3] = 0.5 * (U[j, i, 1] ** 2 + U[j, i, 2] ** 2) / U[j, i, 0] - 1.0
    else:
        U[j, i, 0] = np.nan
    ref = np.empty_like(U)
    oracle.Stepper(p).time_stepping(U.copy(), ref, 0.0, dt)
    with _solver(pkg, lf, nf, pkg.FP_EXACT, kn) as s:
        out = np.empty_like(U)
        s.time_stepping(U, out, 0.0, dt)
        flags = s.counters().status_flags
        orders = s.orders()
    assert nan_equal(out, ref)
    assert flags & 1
    assert orders[j - 4, i - 4] == 1
    interior = out[4:-4, 4:-4]
    bad_cells = ~np.isfinite(interior).all(axis=-1)
    assert bad_cells.any() and bad_cells.sum() < 50  # local, not spread over the grid


@pytest.mark.parametrize("bad", ["negative_pressure", "nan_density"])
def test_fast_mode_inadmissible_state_stays_local(pkg, oracle, bad):
    """The fast first pass solves HLLC with selects and gives an inadmissible
    Gauss point a NaN flux (not the reference's 1/(vx-vx)): the planted cell
    still ends at order 1, status bit 0 reports it, the non-finite cells are
    the exact mode's, and every other cell agrees with the exact mode to
    1e-12."""
    ic, lf, nf, kn = CASES["rp2d3"]
    p = _oracle_params(oracle, lf, nf, kn)
    U = oracle.initial_condition(p, ic)
    dt = oracle.setdt(p, U, p.tmax)
    j, i = 4 + 20, 4 + 30
    if bad == "negative_pressure":
        U[j, i, 3] = 0.5 * (U[j, i, 1] ** 2 + U[j, i, 2] ** 2) / U[j, i, 0] - 1.0
    else:
        U[j, i, 0] = np.nan
    res = {}
    for name, mode in (("exact", pkg.FP_EXACT), ("fast", pkg.FP_FAST)):
        with _solver(pkg, lf, nf, mode, kn) as s:
            out = np.empty_like(U)
            s.time_stepping(U, out, 0.0, dt)
            res[name] = (out, s.counters().status_flags, s.orders())
    (ue, fe, oe), (uf, ff, of) = res["exact"], res["fast"]
    assert ff & 1 and of[j - 4, i - 4] == 1
    bad_e = ~np.isfinite(ue[4:-4, 4:-4]).all(axis=-1)
    bad_f = ~np.isfinite(uf[4:-4, 4:-4]).all(axis=-1)
    assert np.array_equal(bad_e, bad_f) and bad_f.sum() < 50
    good = ~bad_f
    a, b = ue[4:-4, 4:-4][good], uf[4:-4, 4:-4][good]
    assert np.abs(a - b).sum() <= 1e-12 * np.abs(a).sum()


@pytest.mark.parametrize("bc,lx,ly", [(19, 9., 1.), (201, 1.5, 1.5), (301, 1.5, 1.5), (401, 6., 1.), (402, 0.25, 1.),
                                      (403, 1., 1.)])
def test_other_boundary_types_step_like_the_oracle(pkg, oracle, bc, lx, ly):
    """Dirichlet, Mach800, DoubleMach800, RMI, RT and KH boundaries (BC.f90)
    through whole steps: time steps and states bit-identical to the oracle."""
    lf, nf = 48, 32
    p = oracle.make_params(lf, nf, bc=bc, lx=lx, ly=ly, tmax=1.0)
    U = oracle.initial_condition(p, "rp2d3")
    st = oracle.Stepper(p)
    Ug = U.copy()
    t = 0.0
    with pkg.Solver(lf=lf, nf=nf, bc_type=bc, lx=lx, ly=ly, tmax=1.0, fp_mode=pkg.FP_EXACT) as s:
        for step in range(3):
            dt = oracle.setdt(p, U, p.tmax - t)
            dtg = s.Setdt(Ug, p.tmax - t)
            assert dtg == dt, (step, dtg, dt)
            Ur = np.empty_like(U)
            st.time_stepping(U, Ur, t, dt)
            Ugr = np.empty_like(Ug)
            s.time_stepping(Ug, Ugr, t, dtg)
            assert nan_equal(Ugr, Ur), (step, np.nanmax(np.abs(Ugr - Ur)))
            t += dt
            U, Ug = Ur, Ugr


@pytest.mark.parametrize("case", ["sedov", "ragged", "tiny"])
def test_fast_first_pass_tma_and_load_staging_agree(pkg, oracle, case, monkeypatch):
    """The fast two-direction face kernel stages its halo tile with a TMA bulk
    tensor copy (default) or with plain loads (GPMOOD_FLUX_TMA=0): the staged
    tile is the same, so the runs agree bit for bit, including grids whose
    edge tiles reach past the padded grid (zero-filled box)."""
    ic, lf, nf, kn = CASES[case]
    p = _oracle_params(oracle, lf, nf, kn)
    U0 = oracle.initial_condition(p, ic)
    out = []
    for tma in ("1", "0"):
        monkeypatch.setenv("GPMOOD_FLUX_TMA", tma)
        with _solver(pkg, lf, nf, pkg.FP_FAST, kn) as s:
            s.set_state(U0, 0.0)
            assert s.advance(6) == 6
            U, t, _ = s.get_state()
            out.append((U, t, s.orders(), s.counters().status_flags))
    (Ua, ta, ma, sa), (Ub, tb, mb, sb) = out
    assert sa == sb == 0
    assert ta == tb and np.array_equal(ma, mb)
    assert nan_equal(Ua, Ub)


@pytest.mark.parametrize("fp", ["exact", "fast"])
def test_solo_mood_passes_split_detection_agrees(pkg, oracle, fp, monkeypatch):
    """One-CTA MOOD passes split DETECTION over warp roles (default) or keep
    it on one thread per cross cell (GPMOOD_SOLO_SPLIT=0): the decisions and
    so the runs are the same, bit for bit, on the DMR crawl."""
    ic, lf, nf, kn = CASES["dmr"]
    p = _oracle_params(oracle, lf, nf, kn)
    U0 = oracle.initial_condition(p, ic)
    mode = pkg.FP_EXACT if fp == "exact" else pkg.FP_FAST
    out = []
    for split in ("1", "0"):
        monkeypatch.setenv("GPMOOD_SOLO_SPLIT", split)
        with _solver(pkg, lf, nf, mode, kn) as s:
            s.set_state(U0, 0.0)
            assert s.advance(8) == 8
            U, t, _ = s.get_state()
            c = s.counters()
            out.append((U, t, s.orders(), c.detected_total, c.max_passes_stage))
    (Ua, ta, ma, da, pa), (Ub, tb, mb, db, pb) = out
    assert (ta, da, pa) == (tb, db, pb) and pa > 2
    assert np.array_equal(ma, mb)
    assert nan_equal(Ua, Ub)
