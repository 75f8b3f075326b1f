"""The bounds-checked debug build (-DNBCS_CHECK): every data-dependent access
of the spline gathers, the composition gathers and the labelling links tests
its index against its buffer and reports a bad one through nbcs_check_bits
instead of faulting.  On valid inputs it must report nothing and compute
exactly what the normal build computes (tests/checked_pipeline.py, run in
fresh interpreters with each library)."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _run(tmp_path, lib):
    out = str(tmp_path / ("res_%s.npz" % ("check" if lib else "main")))
    env = dict(os.environ)
    if lib:
        env["NBCS_LIB"] = lib
    else:
        env.pop("NBCS_LIB", None)
    r = subprocess.run([sys.executable, os.path.join(HERE, "checked_pipeline.py"), out],
                       capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    return dict(np.load(out))


def test_checked_build_reports_nothing_and_matches(nb, tmp_path):
    from numbacs_gb300 import build
    lib = build.build(check=True)
    main = _run(tmp_path, None)
    chk = _run(tmp_path, lib)
    assert int(main["check_enabled"]) == 0 and int(chk["check_enabled"]) == 1
    assert int(main["check_bits"]) == 0
    assert int(chk["check_bits"]) == 0, hex(int(chk["check_bits"]))
    keys = sorted(k for k in main if k not in ("check_enabled", "check_bits"))
    assert keys == sorted(k for k in chk if k not in ("check_enabled", "check_bits"))
    for k in keys:
        assert np.array_equal(main[k], chk[k]), k
