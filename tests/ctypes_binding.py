"""The binding a NumbaCS maintainer would add to call libnbcs without torch:
ctypes for the library, the CUDA runtime for device memory.  It is the stub
shown for the reference side (numbacs/_gpu.py) and is run by
tests/test_gpu_ctypes_binding.py in a fresh interpreter, so that nothing but
this file, numpy and the two shared libraries is loaded.

Run directly, it integrates the double gyre on the 21 x 11 grid of the
reference's fixtures (t0 = 0, T = 8, rtol 1e-6, atol 1e-8,
flows.py:1162-1169 defaults) and prints the flow map as JSON.
"""
import ctypes
import ctypes.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "..", "numbacs_gb300", "_build", "libnbcs.so")


def _cudart():
    names = ["libcudart.so.13", "libcudart.so.12", "libcudart.so"]
    found = ctypes.util.find_library("cudart")
    if found:
        names.append(found)
    for base in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
                 "/usr/local/cuda/targets/x86_64-linux/lib"):
        names.append(os.path.join(base, "libcudart.so"))
    for n in names:
        try:
            return ctypes.CDLL(n)
        except OSError:
            continue
    raise OSError("CUDA runtime library not found")


_rt = _cudart()
_nb = ctypes.CDLL(LIB)
_nb.nbcs_last_error.restype = ctypes.c_char_p
_nb.nbcs_flowmap_grid_2d.argtypes = [
    ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_int32,
    ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_double,
    ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
    ctypes.c_void_p]

NBCS_FLOW_DOUBLE_GYRE = 0


class NbcsFlow(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("spherical", ctypes.c_int32),
                ("extrap", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("r", ctypes.c_double), ("grid", ctypes.c_double * 9),
                ("coef_uv", ctypes.c_void_p), ("coef_uv32", ctypes.c_void_p)]


def _dev(nbytes):
    p = ctypes.c_void_p()
    rc = _rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(nbytes))
    if rc != 0:
        raise RuntimeError("cudaMalloc failed: %d" % rc)
    return p


def _h2d(dst, a):
    rc = _rt.cudaMemcpy(dst, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes), 1)
    if rc != 0:
        raise RuntimeError("cudaMemcpy H2D failed: %d" % rc)


def flowmap_grid_2D_gpu(flow_kind, t0, T, x, y, params, rtol=1e-6, atol=1e-8):
    x, y, p = (np.ascontiguousarray(a, np.float64) for a in (x, y, params))
    nx, ny = len(x), len(y)
    dx, dy, dout = _dev(x.nbytes), _dev(y.nbytes), _dev(16 * nx * ny)
    try:
        _h2d(dx, x)
        _h2d(dy, y)
        fl = NbcsFlow(kind=flow_kind)
        rc = _nb.nbcs_flowmap_grid_2d(
            ctypes.byref(fl), t0, T, dx, nx, dy, ny, p.ctypes.data_as(ctypes.c_void_p), len(p),
            rtol, atol, None, dout, None, None, None)
        if rc != 0:
            raise RuntimeError(_nb.nbcs_last_error().decode())
        out = np.empty((nx, ny, 2))
        rc = _rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), dout,
                            ctypes.c_size_t(out.nbytes), 2)
        if rc != 0:
            raise RuntimeError("cudaMemcpy D2H failed: %d" % rc)
        return out
    finally:
        for d in (dx, dy, dout):
            _rt.cudaFree(d)


if __name__ == "__main__":
    x, y = np.linspace(0, 2, 21), np.linspace(0, 1, 11)
    params = np.array([1.0, 0.1, 0.25, 0.0, 0.2 * np.pi, 0.0])
    fm = flowmap_grid_2D_gpu(NBCS_FLOW_DOUBLE_GYRE, 0.0, 8.0, x, y, params)
    print(json.dumps({"flowmap": fm.tolist(), "torch_loaded": "torch" in sys.modules}))
