"""The C ABI library: loads, exports every symbol include/gpmood.h declares,
validates its knobs and fails cleanly without a GPU (no CPU fallback)."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"\b(gpmood_[a-z_0-9]+)\s*\(", h.read_text()))
    return sorted(names)


def test_header_lists_the_reference_boundary():
    syms = declared_symbols()
    for must in ("gpmood_time_stepping", "gpmood_setdt", "gpmood_boundary_c", "gpmood_create", "gpmood_advance"):
        assert must in syms


def test_library_exports_every_declared_symbol(pkg):
    lib = C.CDLL(str(ROOT / "gp-mood_gb300" / "libgpmood.so"))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_the_header(pkg):
    from gpmood_gb300.gpmood import SIGNATURES
    assert sorted(SIGNATURES) == declared_symbols()


def test_default_params_are_the_reference_knobs(pkg):
    p = pkg.default_params()
    assert (p.cfl, p.ell_o_dx, p.mord, p.ngp, p.integrator, p.num_flux) == (0.8, 12.0, 5, 3, 10, 100)
    assert (p.dmp, p.u2, p.u2_tol, p.method) == (1, 1, 1, 2)


@pytest.mark.parametrize("bad", [dict(mord=7), dict(ngp=6), dict(num_flux=104), dict(integrator=11),
                                 dict(bc_type=21), dict(lf=2), dict(method=200), dict(method=204), dict(fp_mode=3),
                                 dict(max_mood_iters=-1), dict(cfl=0.0)])
def test_invalid_knobs_rejected(pkg, bad):
    with pytest.raises(pkg.GpmoodError) as e:
        pkg.Solver(**bad)
    assert e.value.code == -1


def test_weights_on_host_without_gpu(pkg):
    from gpmood_gb300.gpmood import gp_weights
    zt, d2, inv = gp_weights(pkg.default_params(lf=64, nf=64))
    assert zt.shape == (3, 4, 3, 13) and abs(zt[2, 0, 0].sum() - 1) < 1e-14


def test_no_gpu_means_error_not_fallback(pkg):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pkg.GpmoodError) as e:
        pkg.Solver(lf=32, nf=32)
    assert e.value.code == -2


def test_polynomial_weights_match_the_oracle(pkg, oracle):
    """POL_MOOD / Unlim_POL (pol_presim, GP_init.f90:359-419): the host library's
    order-3 weights equal the oracle's, sum to one and mirror L/R, T/B."""
    from gpmood_gb300.gpmood import gp_weights
    for method in (200, 201):
        zt, _, _ = gp_weights(pkg.default_params(lf=32, nf=32, mord=3, ngp=2, method=method))
        st = oracle.Stepper(oracle.make_params(32, 32, mord=3, ngp=2, method=method))
        zo = np.array(st.weights().zt, dtype=np.float64).reshape(3, 4, 5, 13)
        assert np.array_equal(zt[1], zo[1, :, :2, :])
        assert np.all(zt[0, :, :, 0] == 1.0)
        assert np.allclose(zt[1, :, :, :5].sum(axis=-1), 1.0, atol=1e-15)
        iL, iT, iR, iB = 0, 1, 2, 3  # stencil points M, L, T, R, B = 0..4
        assert np.array_equal(zt[1, iL, :, [0, 1, 2, 3, 4]], zt[1, iR, :, [0, 3, 2, 1, 4]])
        assert np.array_equal(zt[1, iT, :, [0, 1, 2, 3, 4]], zt[1, iB, :, [0, 1, 4, 3, 2]])
    with pytest.raises(pkg.GpmoodError):
        gp_weights(pkg.default_params(lf=32, nf=32, mord=5, ngp=2, method=200))
