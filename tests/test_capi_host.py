"""C-ABI library and host-side logic (CPU only: no compute calls)."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "nbcs.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nbcs_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from numbacs_gb300 import _lib, build
    build.build()
    L = _lib.load()
    names = _declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    # the Python binding declares a signature for every entry point
    assert set(names) <= set(_lib.SIGNATURES)
    assert L.nbcs_abi_version() == 3


def test_scratch_size_queries():
    from numbacs_gb300 import _lib
    L = _lib.load()
    assert L.nbcs_spline_prefilter_scratch_bytes(121, 217, 101) == 8 * (123 * 217 * 101 + 123 * 219 * 101)
    assert L.nbcs_ridge_scratch_bytes(676, 251) >= 676 * 251
    assert L.nbcs_percentile_scratch_bytes(1000) > 0


def test_invalid_arguments_are_reported_without_a_gpu():
    # argument validation happens before any CUDA call
    from numbacs_gb300 import _lib
    L = _lib.load()
    f = _lib.NbcsFlow()
    f.kind = 7
    rc = L.nbcs_flowmap_grid_2d(f, 0.0, 1.0, None, 1, None, 1, None, 0, 1e-6, 1e-8, None, None,
                                None, None, None)
    assert rc == -1 and b"params" in L.nbcs_last_error()
    p = np.zeros(6)
    rc = L.nbcs_flowmap_grid_2d(f, 0.0, 1.0, None, 1, None, 1, p.ctypes.data_as(_lib._vp), 6,
                                1e-6, 1e-8, None, None, None, None, None)
    assert rc == -1 and b"unknown flow kind" in L.nbcs_last_error()
    f.kind = _lib.FLOW_SPLINE2D
    f.extrap = 3  # 0 constant, 1 nearest, 2 linear
    rc = L.nbcs_flowmap_grid_2d(f, 0.0, 1.0, None, 1, None, 1, p.ctypes.data_as(_lib._vp), 1,
                                1e-6, 1e-8, None, None, None, None, None)
    assert rc == -1 and b"extrap" in L.nbcs_last_error()
    # the mixed path indexes quad entries in 32 bits: 2^32 spline nodes or more are refused
    f.extrap = 0
    f.grid[:] = [0.0, 1.0, 1100.0, 0.0, 1.0, 2000.0, 0.0, 1.0, 2000.0]
    f.coef_uv, f.coef_uv32 = 4096, 8192  # never dereferenced: validation comes first
    opts = _lib.NbcsOpts()
    opts.precision = _lib.PREC_MIXED
    rc = L.nbcs_flowmap_grid_2d(f, 0.0, 1.0, None, 1, None, 1, p.ctypes.data_as(_lib._vp), 1,
                                1e-6, 1e-8, None, None, None, opts, None)
    assert rc == -4 and b"2^32" in L.nbcs_last_error()
    # ... and takes cell indices from float mantissas: at most 2^23 nodes per axis
    f.grid[:] = [0.0, 1.0, 3.0, 0.0, 1.0, 3.0, 0.0, 1.0, 9000000.0]
    rc = L.nbcs_flowmap_grid_2d(f, 0.0, 1.0, None, 1, None, 1, p.ctypes.data_as(_lib._vp), 1,
                                1e-6, 1e-8, None, None, None, opts, None)
    assert rc == -4 and b"2^23" in L.nbcs_last_error()
    assert L.nbcs_percentile(None, 0, 50.0, None, None, 0, None) == -1


def test_predefined_flow_tuples():
    from numbacs_gb300.flows import Flow, get_predefined_flow
    fl, p, dom = get_predefined_flow("double_gyre", int_direction=-1.0)
    assert isinstance(fl, Flow) and p[0] == -1.0 and dom == ((0.0, 2.0), (0.0, 1.0))
    np.testing.assert_allclose(p, [-1.0, 0.1, 0.25, 0.0, 0.2 * np.pi, 0.0])
    assert isinstance(get_predefined_flow("double_gyre", return_default_params=False,
                                          return_domain=False), Flow)
    out = get_predefined_flow("double_gyre", parameter_description=True)
    assert len(out) == 4 and "omega" in out[3]
    # the reference's Bickley defaults always carry int_direction = 1.0
    _, pb, domb = get_predefined_flow("bickley_jet", int_direction=-1.0)
    assert pb[0] == 1.0 and len(pb) == 12
    assert domb[0][1] == pytest.approx(np.pi * 6.371)
    with pytest.raises(ValueError):
        get_predefined_flow("nope")


def test_flowmap_rejects_lsoda_and_foreign_funcptr():
    from numbacs_gb300 import flowmap_grid_2D, get_predefined_flow
    fl, p, _ = get_predefined_flow("double_gyre")
    with pytest.raises(NotImplementedError):
        flowmap_grid_2D(fl, 0.0, 1.0, np.zeros(2), np.zeros(2), p, method="lsoda")
    with pytest.raises(TypeError):
        flowmap_grid_2D(12345, 0.0, 1.0, np.zeros(2), np.zeros(2), p)


def test_oracle_is_not_imported_by_the_product():
    pkg = os.path.join(ROOT, "numbacs_gb300")
    for dp, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".h")):
                txt = open(os.path.join(dp, fn)).read()
                assert "import oracle" not in txt and "from oracle" not in txt, fn
                assert "oracle/" not in txt.replace("CPU oracle", ""), fn


def test_geo_workload_shapes():
    from numbacs_gb300 import workloads as W
    t, lon, lat = W.geo_grid()
    assert (len(t), len(lon), len(lat)) == (121, 217, 101)
    lonf, latf = W.geo_ftle_grid(0.2)
    assert (len(lonf), len(latf)) == (676, 251)
    kx, ky, w, phi, amp = W.geo_modes(0)
    assert len(kx) == 256
    kmag = np.hypot(kx, ky)
    assert kmag.min() >= 2 * np.pi / 5000 and kmag.max() <= 2 * np.pi / 100


def test_fails_loudly_without_library(tmp_path):
    """No CPU fallback: with the CUDA library absent the package raises on load
    and on a compute call (run in a child so the session's loaded handle stays)."""
    import subprocess
    import sys
    code = (
        "import numpy as np\n"
        "import numbacs_gb300 as nb\n"
        "from numbacs_gb300 import _lib\n"
        "try:\n"
        "    _lib.load()\n"
        "    raise SystemExit('load() did not raise')\n"
        "except RuntimeError as e:\n"
        "    assert 'not built' in str(e), e\n"
        "fl, p, _ = nb.get_predefined_flow('double_gyre')\n"
        "try:\n"
        "    nb.flowmap_grid_2D(fl, 0.0, 1.0, np.linspace(0, 2, 5), np.linspace(0, 1, 3), p)\n"
        "    raise SystemExit('flowmap_grid_2D did not raise')\n"
        "except RuntimeError:\n"
        "    pass\n"
        "print('loud')\n")
    env = dict(os.environ, NBCS_LIB=str(tmp_path / "missing" / "libnbcs.so"))
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0 and "loud" in r.stdout, r.stderr[-2000:]
