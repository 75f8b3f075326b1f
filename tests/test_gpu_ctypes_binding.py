"""The C ABI from a process without torch: tests/ctypes_binding.py (the
reference-side ctypes stub: CUDA runtime for memory, libnbcs for the compute)
reproduces the reference's fixtures through the whole path -- the double-gyre
flow map (tests/test_integration.py:55-64), its FTLE
(tests/test_diagnostics.py:82-96), C_eig eigenvalues
(tests/test_diagnostics.py:133-150) and ridge points
(tests/test_extraction.py:6-12), the spline coefficients and interpolated
velocities (tests/test_flows.py:74-133, :208-229) -- and a spline flow map
bit-identical to the oracle's."""
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
    assert np.allclose(np.array(out["ftle"]).astype(np.float32), golden["ftle"])
    assert np.allclose(np.array(out["evals"]).astype(np.float32), golden["Cevals"])
    assert np.allclose(np.array(out["ridge_pts"]).astype(np.float32), golden["ridge_pts"])
    assert np.allclose(np.array(out["spline_Cu"]), golden["spline_Cu"])
    assert np.allclose(np.array(out["spline_Cv"]), golden["spline_Cv"])
    assert np.allclose(np.array(out["spline_vel"]), golden["spline_vel"])
    import oracle
    ts = np.array([0.0, 0.1, 0.2])
    xs = np.array([0.0, 0.5, 1.0])
    T3, X3, Y3 = np.meshgrid(ts, xs, xs, indexing="ij")
    U = np.sin(X3) * np.cos(Y3) + np.sin(T3)
    V = np.cos(X3) * np.sin(Y3) + np.cos(T3)
    g, cu, cv = oracle.get_interp_arrays_2D(ts, xs, xs, U, V)
    xi = np.array([0.1, 0.4, 0.7])
    ofm = oracle.flowmap_grid_2D(oracle.spline_flow(g, cu, cv), 0.02, 0.15, xi, xi, [1.0])
    assert np.array_equal(np.array(out["spline_flowmap"]), ofm)
