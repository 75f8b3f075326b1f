"""The C ABI from a process without torch: tests/ctypes_binding.py (the
reference-side ctypes stub: CUDA runtime for memory, libnbcs for the
integrator) reproduces the reference's double-gyre flow-map fixture
(tests/test_integration.py:55-64)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_ctypes_binding_without_torch(nb, golden):
    r = subprocess.run([sys.executable, os.path.join(HERE, "ctypes_binding.py")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["torch_loaded"] is False
    fm = np.array(out["flowmap"])
    assert fm.shape == golden["fm"].shape
    assert np.allclose(fm.astype(np.float32), golden["fm"])
