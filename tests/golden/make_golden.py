"""Extract the reference's golden vectors for the flow-map -> FTLE -> ridge path
into ``tests/golden/reference_fixtures.npz``.

Sources (paths within the NumbaCS project; the reference itself cannot be
imported here because numba / numbalsoda / interpolation are absent):

  tests/testing_data/fm.npy         flowmap_grid_2D, double gyre 21x11, t0=0, T=8
                                    (tests/test_integration.py:55-64)
  tests/testing_data/fm_n.npy       flowmap_n / flowmap_n_grid_2D, the same particles at n = 4
                                    times (tests/test_integration.py:45-52, :78-90)
  tests/testing_data/ftle.npy       ftle_grid_2D(fm, 8, 0.1, 0.1)  (tests/test_diagnostics.py:82-96)
  tests/testing_data/Cevals.npy,    C_eig_2D(fm, 0.1, 0.1)           (tests/test_diagnostics.py:133-150)
  tests/testing_data/Cevecs.npy
  tests/testing_data/ridge_pts.npy  ftle_ridge_pts(ftle, Cevecs[...,1], x, y) (tests/test_extraction.py:6-12)
  tests/testing_data/ridges.pkl     ftle_ridges(ftle, Cevecs[...,1], x, y)    (tests/test_extraction.py:14-20)
  tests/testing_data/fm_ci.npy,     flowmap_composition_initial, double gyre 21x11, t0=0, T=8,
  tests/testing_data/fms_ci.npy     h=1 (nT=8)                     (tests/test_integration.py:92-103)
  tests/testing_data/fm_cs.npy,     flowmap_composition_step from fms_ci at t0=8
  tests/testing_data/fms_cs.npy                                    (tests/test_integration.py:105-114)
  tests/testing_data/fm_aux.npy     flowmap_aux_grid_2D, double gyre 21x11, t0=0, T=8, h=1e-5
                                    (tests/test_integration.py:66-75)
  tests/testing_data/C.npy          C_tensor_2D(fm_aux, 0.1, 0.1)    (tests/test_diagnostics.py:99-109)
  tests/testing_data/Cevals_aux.npy, C_eig_aux_2D(fm_aux, 0.1, 0.1)  (tests/test_diagnostics.py:112-131)
  tests/testing_data/Cevecs_aux.npy
  tests/testing_data/ordered_ridges.pkl  ftle_ordered_ridges(ftle, Cevecs[...,1], x, y, 0.1)
                                    (tests/test_extraction.py:22-28)
  tests/test_flows.py literals      spline coefficients Cu/Cv (:74-133), spline values at 27
                                    points (:208-229), double-gyre and Bickley velocities
                                    at the same 27 points (:315-357)
  tests/test_utils.py literals      the deformation-gradient stencils at grid point (5, 5):
                                    gradF_stencil_2D of fm (:74-89), gradF_aux_stencil_2D and
                                    gradF_main_stencil_2D of fm_aux (:91-120), and
                                    eigvalsh_max_2D of B^T B (:190-199)

The ``.npy`` files are read with ``allow_pickle=False``; the ``.pkl`` file is read
with an unpickler that only admits numpy array reconstruction; the test-source
literals are read with ``ast`` (never executed).

Usage:  python tests/golden/make_golden.py REFERENCE_ROOT
        (or NBCS_REFERENCE_ROOT=<NumbaCS checkout> python tests/golden/make_golden.py)
"""
import ast
import io
import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class _NumpyOnlyUnpickler(pickle.Unpickler):
    _ALLOWED = {
        ("numpy.core.multiarray", "_reconstruct"), ("numpy._core.multiarray", "_reconstruct"),
        ("numpy", "ndarray"), ("numpy", "dtype"),
        ("numpy.core.multiarray", "scalar"), ("numpy._core.multiarray", "scalar"),
    }

    def find_class(self, module, name):
        if (module, name) in self._ALLOWED:
            mod = __import__(module, fromlist=[name])
            return getattr(mod, name)
        raise pickle.UnpicklingError("refusing %s.%s" % (module, name))


def _load_pkl(path):
    with open(path, "rb") as fh:
        return _NumpyOnlyUnpickler(io.BytesIO(fh.read())).load()


def _eval_literal(node):
    """Evaluate np.array([...]) / tuples / nested lists without executing code."""
    if isinstance(node, ast.Call):
        fn = node.func
        if isinstance(fn, ast.Attribute) and fn.attr == "array":
            return np.array(_eval_literal(node.args[0]), dtype=np.float64)
        raise ValueError("unexpected call")
    if isinstance(node, ast.Tuple):
        return tuple(_eval_literal(e) for e in node.elts)
    return ast.literal_eval(node)


def _test_literals(path):
    tree = ast.parse(open(path).read())
    out = {}
    for fn in tree.body:
        if not isinstance(fn, ast.FunctionDef):
            continue
        for node in ast.walk(fn):
            if (isinstance(node, ast.Assign) and len(node.targets) == 1
                    and isinstance(node.targets[0], ast.Name)
                    and (node.targets[0].id.endswith("_expected") or node.targets[0].id == "B")):
                try:
                    out[(fn.name, node.targets[0].id)] = _eval_literal(node.value)
                except (ValueError, SyntaxError):
                    pass
    return out


def main(ref_root):
    td = os.path.join(ref_root, "tests", "testing_data")
    arrays = {}
    for name in ("fm", "ftle", "Cevals", "Cevecs", "ridge_pts", "fm_ci", "fms_ci", "fm_cs",
                 "fms_cs", "fm_aux", "Cevals_aux", "Cevecs_aux", "C", "fm_n"):
        arrays[name] = np.load(os.path.join(td, name + ".npy"), allow_pickle=False)
    ridges = _load_pkl(os.path.join(td, "ridges.pkl"))
    arrays["n_ridges"] = np.array(len(ridges))
    for k, r in enumerate(ridges):
        arrays["ridges_%d" % k] = np.asarray(r)
    ordered = _load_pkl(os.path.join(td, "ordered_ridges.pkl"))
    arrays["n_ordered"] = np.array(len(ordered))
    for k, r in enumerate(ordered):
        arrays["ordered_%d" % k] = np.asarray(r)
    lit = _test_literals(os.path.join(ref_root, "tests", "test_flows.py"))
    arrays["spline_Cu"] = lit[("test_get_interp_arrays_2D", "Cu_expected")]
    arrays["spline_Cv"] = lit[("test_get_interp_arrays_2D", "Cv_expected")]
    vu, vv = lit[("test_get_callable_2D", "veli_expected")]
    arrays["spline_vel"] = np.stack([vu, vv], axis=1)
    du, dv = lit[("test_get_predefined_callable_dg", "veli_expected")]
    arrays["dg_vel"] = np.stack([du, dv], axis=1)
    bu, bv = lit[("test_get_predefined_callable_bickley", "veli_expected")]
    arrays["bickley_vel"] = np.stack([bu, bv], axis=1)
    ut = _test_literals(os.path.join(ref_root, "tests", "test_utils.py"))
    arrays["gradF_55"] = np.array(ut[("test_gradF_stencil_2D", "gradF_expected")])
    arrays["gradF_aux_55"] = np.array(ut[("test_gradF_aux_stencil_2D", "gradF_aux_expected")])
    arrays["gradF_main_55"] = np.array(ut[("test_gradF_main_stencil_2D", "gradF_main_expected")])
    arrays["eigvalsh_B"] = np.asarray(ut[("test_eigvalsh_max_2D", "B")], dtype=np.float64)
    arrays["eigvalsh_max"] = np.array(ut[("test_eigvalsh_max_2D", "eigval_expected")])
    out = os.path.join(HERE, "reference_fixtures.npz")
    np.savez_compressed(out, **arrays)
    for k, v in sorted(arrays.items()):
        print("%-14s %s %s" % (k, np.shape(v), np.asarray(v).dtype))
    print("wrote", out)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NBCS_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <NumbaCS checkout>  (or set NBCS_REFERENCE_ROOT)")
    main(root)
