"""Shared fixtures.  Tests marked ``gpu`` need a CUDA GPU; every other test runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as ge  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle():
    O = ge.import_oracle()
    O.build()
    return O


@pytest.fixture(scope="session")
def pkg():
    """The product package; builds libgpmood.so once if it is missing."""
    lib = ge.PKG_DIR / "libgpmood.so"
    if not lib.exists():
        ge.build()
    return ge.import_package()


def nan_equal(a, b):
    """Bitwise equality that treats every NaN as equal (GPU NaNs are canonical)."""
    import numpy as np
    a = np.asarray(a)
    b = np.asarray(b)
    both_nan = np.isnan(a) & np.isnan(b)
    return bool(np.all((a.view(np.int64) == b.view(np.int64)) | both_nan))
