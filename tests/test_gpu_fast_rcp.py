"""The fast mode's reciprocal (Newton-Raphson from rcp.approx.ftz.f64, two
steps) against IEEE division: within 4 ulp over normal inputs with normal
reciprocals, NaN for zero; its square root against the correctly rounded one."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_fast_reciprocal_within_4_ulp(pkg):
    lib = pkg.load_library()
    rng = np.random.default_rng(7)
    mant = rng.uniform(1.0, 2.0, size=1 << 20)
    expo = rng.integers(-1000, 1000, size=mant.size)
    x = np.ldexp(mant, expo) * rng.choice([-1.0, 1.0], size=mant.size)
    x = np.concatenate([x, [1.0, 3.0, 0.1, 1.4, 1e-300, 1e300, np.nextafter(1.0, 2.0), np.nextafter(2.0, 1.0)]])
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    assert lib.gpmood_fast_rcp(C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), x.size) == 0
    y = yd.cpu().numpy()
    ref = (1.0 / xd).cpu().numpy()  # IEEE division on the GPU
    ulp = np.abs(y - ref) / np.spacing(np.abs(ref))
    assert np.isfinite(y).all()
    assert ulp.max() <= 4.0, (ulp.max(), x[np.argmax(ulp)])
    z = torch.zeros(4, dtype=torch.float64, device="cuda")
    o = torch.empty_like(z)
    assert lib.gpmood_fast_rcp(C.c_void_p(z.data_ptr()), C.c_void_p(o.data_ptr()), 4) == 0
    assert torch.isnan(o).all()


def test_fast_sqrt_within_2_ulp(pkg):
    """The fast mode's square root (rsqrt.approx.ftz.f64, one coupled Newton
    step, one correction) against the correctly rounded sqrt: within 2 ulp for
    positive normal inputs and outputs; NaN for zero, negatives and infinity."""
    lib = pkg.load_library()
    rng = np.random.default_rng(11)
    mant = rng.uniform(1.0, 2.0, size=1 << 20)
    expo = rng.integers(-1000, 1000, size=mant.size)
    x = np.ldexp(mant, expo)
    x = np.concatenate([x, [1.0, 2.0, 4.0, 0.04, 1.4, 1e-300, 1e300, np.nextafter(1.0, 2.0),
                            np.nextafter(4.0, 1.0), np.finfo(np.float64).tiny, np.finfo(np.float64).max]])
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    assert lib.gpmood_fast_sqrt(C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), x.size) == 0
    y = yd.cpu().numpy()
    ref = np.sqrt(x)
    ulp = np.abs(y - ref) / np.spacing(ref)
    assert np.isfinite(y).all()
    assert ulp.max() <= 2.0, (ulp.max(), x[np.argmax(ulp)])
    z = torch.tensor([0.0, -1.0, -0.0, float("inf")], dtype=torch.float64, device="cuda")
    o = torch.empty_like(z)
    assert lib.gpmood_fast_sqrt(C.c_void_p(z.data_ptr()), C.c_void_p(o.data_ptr()), 4) == 0
    assert torch.isnan(o).all()
