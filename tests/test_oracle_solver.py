"""Invariants of the CPU oracle's solver and the reference's GP inversion
self-check; the reference's recorded runs are reproduced in
tests/test_reference_pins.py."""
from __future__ import annotations

import numpy as np
import pytest

I = (slice(4, -4), slice(4, -4))


def run(oracle, p, ic, nsteps):
    U = oracle.initial_condition(p, ic)
    st = oracle.Stepper(p)
    t, n = st.run(U, 0.0, nsteps)
    return U, t, n, st


def test_rp2d3_diagonal_symmetry(oracle):
    """plot/plotter_hdf5.py:43: sum|q - q^T| / (nx*ny) of the 2DRP3 solution;
    the IC is symmetric under x<->y with u<->v."""
    p = oracle.make_params(64, 64, bc=17, tmax=0.8)
    U, t, n, _ = run(oracle, p, "rp2d3", 25)
    rho = U[I + (0,)]
    err = np.abs(rho - rho.T).sum() / rho.size
    assert err < 1e-12, err
    mx, my = U[I + (1,)], U[I + (2,)]
    assert np.abs(mx - my.T).max() < 1e-10


def test_sedov_fourfold_symmetry(oracle):
    p = oracle.make_params(64, 64, bc=20, tmax=0.05)
    U, t, n, st = run(oracle, p, "sedov", 20)
    rho = U[I + (0,)]
    assert np.abs(rho - rho.T).max() < 1e-12
    assert np.abs(rho - rho[::-1, :]).max() < 1e-12
    assert st.counters[0] > 0  # the blast triggers MOOD


def test_periodic_conservation(oracle):
    p = oracle.make_params(48, 48, bc=18, lx=10.0, ly=10.0, tmax=1.0)
    U0 = oracle.initial_condition(p, "vortex")
    m0 = U0[I].sum(axis=(0, 1))
    U, t, n, _ = run(oracle, p, "vortex", 15)
    m1 = U[I].sum(axis=(0, 1))
    np.testing.assert_allclose(m1, m0, rtol=1e-13)


def test_vortex_convergence_order(oracle):
    """R2 GP on the smooth vortex: the L1 error falls at high order."""
    errs = []
    for n in (40, 80):
        dx = 10.0 / n
        p = oracle.make_params(n, n, bc=18, lx=10.0, ly=10.0, tmax=1.0)
        U0 = oracle.initial_condition(p, "vortex")
        U, t, k, _ = run(oracle, p, "vortex", 10 ** 6)
        # exact solution at t = 1: the IC advected by (1, 1)
        shift = int(round(1.0 / dx))
        assert abs(shift * dx - 1.0) < 1e-12
        ref = np.roll(np.roll(U0[I + (0,)], shift, axis=0), shift, axis=1)
        errs.append(np.abs(U[I + (0,)] - ref).sum() * dx * dx)
    order = np.log2(errs[0] / errs[1])
    assert order > 3.0, (errs, order)


def test_shock_detector_cases(oracle):
    import ctypes as C
    p = oracle.make_params(16, 16)
    U = oracle.padded(16, 16)
    U[..., 0] = 1.0
    U[..., 3] = 2.5
    assert oracle.lib().orc_shock_detector(C.byref(p), U, 8, 8) == 0  # quiescent: no shock
    # strongly converging flow across a pressure jump, Mach > 0.2: a shock
    for n in range(U.shape[0]):
        for l in range(U.shape[1]):
            left = l - 3 <= 8
            r, u, pr = (1.0, 2.0, 1.0) if left else (1.0, -2.0, 10.0)
            U[n, l] = [r, r * u, 0.0, pr / 0.4 + 0.5 * r * u * u]
    assert oracle.lib().orc_shock_detector(C.byref(p), U, 8, 8) == 1
    # the same jump in a diverging flow is not a shock
    U[..., 1] = -U[..., 1]
    assert oracle.lib().orc_shock_detector(C.byref(p), U, 8, 8) == 0


@pytest.mark.parametrize("n,ref", [(50, 1.8488927466117464E-032), (100, 3.9443045261050590E-031),
                                   (200, 2.2088105346188331E-029), (400, 1.5146129380243427E-028)])
def test_deprecated_inversion_error_anchor(oracle, n, ref):
    """Column 4 of the same files: the GP_init.f90:250 inversion error of the
    R1 covariance at ell = 1 (ell/dx = n/20)."""
    p = oracle.make_params(n, n, lx=20.0, ly=20.0, mord=3, ngp=2, ell_o_dx=1.0 / (20.0 / n))
    err = oracle.gp_weights(p).inv_err[1]
    assert ref / 4 <= err <= ref * 4, (err, ref)
    if n == 100:
        assert err == ref  # identical to the last bit


@pytest.mark.parametrize("integ,nflux", [(10, 101), (10, 102), (10, 103), (8, 100), (9, 100), (12, 100)])
def test_variants_conserve_mass_and_symmetry(oracle, integ, nflux):
    """Periodic isentropic vortex: every Riemann solver / integrator conserves
    the totals to rounding; the x<->y symmetric 2DRP3 stays symmetric."""
    p = oracle.make_params(32, 32, bc=18, lx=10.0, ly=10.0, tmax=1.0, integrator=integ, num_flux=nflux)
    U, t, k, _ = run(oracle, p, "vortex", 4)
    U0 = oracle.initial_condition(p, "vortex")
    for v in range(4):
        assert abs(U[I + (v,)].sum() - U0[I + (v,)].sum()) <= 1e-12 * abs(U0[I + (v,)]).sum()
    p = oracle.make_params(32, 32, bc=17, tmax=0.8, integrator=integ, num_flux=nflux)
    U, t, k, _ = run(oracle, p, "rp2d3", 4)
    r = U[I + (0,)]
    assert np.abs(r - r.T).sum() / r.size < 1e-12  # plot/plotter_hdf5.py:43, as above


def test_convex_combination_blend_with_unit_weights_is_plain(oracle):
    """The oracle's NN_GP_MOOD_CC_ blend with values_NN = (0, 1) everywhere
    reproduces plain GP-MOOD at Mord 3 bit for bit; a non-trivial pair in one
    column changes the run."""
    n = 48
    p = oracle.make_params(n, n, bc=17, tmax=0.8, mord=3, ngp=2)
    U0 = oracle.initial_condition(p, "rp2d3")
    w = np.zeros((n + 2, 2), np.float32)
    w[:, 1] = 1.0

    def run(wts):
        st = oracle.Stepper(p)
        if wts is not None:
            st.set_cc(40, wts)
        U, t = U0.copy(), 0.0
        for _ in range(3):
            dt = oracle.setdt(p, U, p.tmax - t)
            Ur = np.empty_like(U)
            st.time_stepping(U, Ur, t, dt)
            t += dt
            U = Ur
        return U

    plain, unit = run(None), run(w)
    assert np.array_equal(plain, unit)
    w2 = w.copy()
    w2[1:n + 1] = [0.25, 0.75]
    assert not np.array_equal(plain, run(w2))
