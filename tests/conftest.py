"""Shared fixtures.  The golden vectors in tests/golden/reference_fixtures.npz
were extracted from the reference's own test data by tests/golden/make_golden.py
(21 x 11 double-gyre grid on [0,2] x [0,1], checkerboard mask mask[::2, ::2],
as in the reference's tests/conftest.py:9-22)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NX, NY = 21, 11


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "reference_fixtures.npz")))


@pytest.fixture
def coords_dg():
    return np.linspace(0, 2, NX), np.linspace(0, 1, NY)


@pytest.fixture
def mask_dg():
    m = np.zeros((NX, NY), bool)
    m[::2, ::2] = True
    return m


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def nb():
    """The product package with its CUDA library loaded (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import numbacs_gb300
    from numbacs_gb300 import _lib
    _lib.load()
    return numbacs_gb300


def apply_mask(arr, mask):
    out = arr.copy()
    out[mask] = 0.0
    return out


def reconstruct(evals, evecs):
    D = np.zeros_like(evecs)
    D[..., 0, 0] = evals[..., 0]
    D[..., 1, 1] = evals[..., 1]
    return np.einsum("...ij,...jk,...kl->...il", evecs, D, np.swapaxes(evecs, -1, -2))
