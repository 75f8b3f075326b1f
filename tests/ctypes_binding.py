"""The binding a NumbaCS maintainer would add to call libnbcs without torch:
ctypes for the library, the CUDA runtime for device memory.  It is the stub
shown for the reference side (numbacs/_gpu.py) and is run by
tests/test_gpu_ctypes_binding.py in a fresh interpreter, so that nothing but
this file, numpy and the two shared libraries is loaded.

It covers the calls of the path: a predefined flow (get_predefined_flow's
kinds), a spline flow (get_interp_arrays_2D -> nbcs_spline_prefilter_3d,
get_flow_2D -> nbcs_spline_pack_uv), flowmap_grid_2D, ftle_grid_2D,
C_eig_2D and ftle_ridge_pts.  Run directly, it runs them on the 21 x 11
double-gyre grid of the reference's fixtures (t0 = 0, T = 8, rtol 1e-6,
atol 1e-8, flows.py:1162-1169 defaults) and on the 3 x 3 x 3 spline case of
the reference's tests/test_flows.py, and prints the results as JSON.
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

_vp, _i32, _i64, _d, _sz = (ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double,
                            ctypes.c_size_t)
_nb.nbcs_spline_prefilter_scratch_bytes.argtypes = [_i32, _i32, _i32]
_nb.nbcs_spline_prefilter_scratch_bytes.restype = _sz
_nb.nbcs_spline_prefilter_3d.argtypes = [_vp, _i32, _i32, _i32, _vp, _vp, _sz, _vp]
_nb.nbcs_spline_pack_uv.argtypes = [_vp, _vp, _i64, _vp, _vp, _vp]
_nb.nbcs_eval_rhs.argtypes = [_vp, _vp, _i32, _vp, _i64, _vp, _i32, _vp]
_nb.nbcs_ftle_grid_2d.argtypes = [_vp, _i32, _i32, _d, _d, _d, _vp, _vp, _vp]
_nb.nbcs_c_eig_2d.argtypes = [_vp, _i32, _i32, _d, _d, _vp, _vp, _vp, _vp]
_nb.nbcs_ridge_scratch_bytes.argtypes = [_i32, _i32]
_nb.nbcs_ridge_scratch_bytes.restype = _sz
_nb.nbcs_ridge_pts.argtypes = [_vp, _vp, _vp, _i32, _vp, _i32, _d, _d, _vp, _vp, _vp, _vp, _vp,
                               _sz, _vp]

NBCS_FLOW_DOUBLE_GYRE = 0
NBCS_FLOW_SPLINE2D = 2


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


def _d2h(a, src):
    rc = _rt.cudaMemcpy(a.ctypes.data_as(ctypes.c_void_p), src, ctypes.c_size_t(a.nbytes), 2)
    if rc != 0:
        raise RuntimeError("cudaMemcpy D2H failed: %d" % rc)
    return a


def _check(rc):
    if rc != 0:
        raise RuntimeError(_nb.nbcs_last_error().decode())


class DeviceArrays:
    """Device buffers freed together."""

    def __init__(self):
        self.ptrs = []

    def new(self, nbytes):
        p = _dev(max(int(nbytes), 1))
        self.ptrs.append(p)
        return p

    def put(self, a):
        a = np.ascontiguousarray(a)
        p = self.new(a.nbytes)
        _h2d(p, a)
        return p

    def free(self):
        for p in self.ptrs:
            _rt.cudaFree(p)
        self.ptrs = []


class SplineFlowGPU:
    """get_interp_arrays_2D + get_flow_2D (flows.py:9-46, :121-258) on the
    device: prefiltered coefficients, interleaved FP64 and FP32 copies, and
    the nbcs_flow handle that replaces the numba funcptr."""

    def __init__(self, t, x, y, U, V, spherical=0, extrap=0, r=6371.0):
        self.mem = DeviceArrays()
        nt, nx, ny = U.shape
        n = (nt + 2) * (nx + 2) * (ny + 2)
        nbytes = _nb.nbcs_spline_prefilter_scratch_bytes(nt, nx, ny)
        scratch = self.mem.new(nbytes)
        coefs = []
        for F in (U, V):
            c = self.mem.new(8 * n)
            _check(_nb.nbcs_spline_prefilter_3d(self.mem.put(np.asarray(F, np.float64)), nt, nx,
                                                ny, c, scratch, nbytes, None))
            coefs.append(c)
        self.coef_uv = self.mem.new(16 * n)
        self.coef_uv32 = self.mem.new(32 * n)  # "quad" layout: 8 floats per node
        _check(_nb.nbcs_spline_pack_uv(coefs[0], coefs[1], n, self.coef_uv, self.coef_uv32, None))
        self.cu = _d2h(np.empty((nt + 2, nx + 2, ny + 2)), coefs[0])
        self.cv = _d2h(np.empty((nt + 2, nx + 2, ny + 2)), coefs[1])
        g = [t[0], t[-1], nt, x[0], x[-1], nx, y[0], y[-1], ny]
        self.flow = NbcsFlow(kind=NBCS_FLOW_SPLINE2D, spherical=spherical, extrap=extrap, r=r,
                             grid=(ctypes.c_double * 9)(*[float(v) for v in g]),
                             coef_uv=self.coef_uv, coef_uv32=self.coef_uv32)


def eval_rhs_gpu(flow, pts, params):
    """The reference @cfunc funcptr(t, y, dy, p) at rows (t, x, y) -> (n, 2)."""
    mem = DeviceArrays()
    try:
        pts = np.ascontiguousarray(pts, np.float64)
        p = np.ascontiguousarray(params, np.float64)
        out = mem.new(16 * len(pts))
        _check(_nb.nbcs_eval_rhs(ctypes.byref(flow), p.ctypes.data_as(_vp), len(p), mem.put(pts),
                                 len(pts), out, 0, None))
        return _d2h(np.empty((len(pts), 2)), out)
    finally:
        mem.free()


def flowmap_grid_2D_gpu(flow, t0, T, x, y, params, rtol=1e-6, atol=1e-8):
    """flowmap_grid_2D (integration.py:123-182); `flow` is an NbcsFlow or a
    predefined flow kind."""
    if isinstance(flow, int):
        flow = NbcsFlow(kind=flow)
    x, y, p = (np.ascontiguousarray(a, np.float64) for a in (x, y, params))
    nx, ny = len(x), len(y)
    mem = DeviceArrays()
    try:
        dout = mem.new(16 * nx * ny)
        _check(_nb.nbcs_flowmap_grid_2d(
            ctypes.byref(flow), t0, T, mem.put(x), nx, mem.put(y), ny,
            p.ctypes.data_as(ctypes.c_void_p), len(p), rtol, atol, None, dout, None, None, None))
        return _d2h(np.empty((nx, ny, 2)), dout)
    finally:
        mem.free()


def ftle_grid_2D_gpu(flowmap, T, dx, dy):
    """ftle_grid_2D (diagnostics.py:21-65)."""
    nx, ny = flowmap.shape[:2]
    mem = DeviceArrays()
    try:
        out = mem.new(8 * nx * ny)
        _check(_nb.nbcs_ftle_grid_2d(mem.put(np.asarray(flowmap, np.float64)), nx, ny, T, dx, dy,
                                     None, out, None))
        return _d2h(np.empty((nx, ny)), out)
    finally:
        mem.free()


def C_eig_2D_gpu(flowmap, dx, dy):
    """C_eig_2D (diagnostics.py:200-244) -> (evals (nx,ny,2), evecs (nx,ny,2,2))."""
    nx, ny = flowmap.shape[:2]
    mem = DeviceArrays()
    try:
        ev, vec = mem.new(16 * nx * ny), mem.new(32 * nx * ny)
        _check(_nb.nbcs_c_eig_2d(mem.put(np.asarray(flowmap, np.float64)), nx, ny, dx, dy, None,
                                 ev, vec, None))
        return _d2h(np.empty((nx, ny, 2)), ev), _d2h(np.empty((nx, ny, 2, 2)), vec)
    finally:
        mem.free()


def ftle_ridge_pts_gpu(f, eigvec_max, x, y, sdd_thresh=0.0, percentile=0):
    """ftle_ridge_pts (extraction/ridges.py:9-76) -> (k, 2) points."""
    nx, ny = f.shape
    mem = DeviceArrays()
    try:
        nbytes = _nb.nbcs_ridge_scratch_bytes(nx, ny)
        pts, n = mem.new(16 * nx * ny), mem.new(8)
        _check(_nb.nbcs_ridge_pts(
            mem.put(np.asarray(f, np.float64)), mem.put(np.asarray(eigvec_max, np.float64)),
            mem.put(np.asarray(x, np.float64)), nx, mem.put(np.asarray(y, np.float64)), ny,
            sdd_thresh, percentile, None, None, pts, n, mem.new(nbytes), nbytes, None))
        k = int(_d2h(np.empty(1, np.int64), n)[0])
        return _d2h(np.empty((k, 2)), pts) if k else np.empty((0, 2))
    finally:
        mem.free()


if __name__ == "__main__":
    x, y = np.linspace(0, 2, 21), np.linspace(0, 1, 11)
    params = np.array([1.0, 0.1, 0.25, 0.0, 0.2 * np.pi, 0.0])
    fm = flowmap_grid_2D_gpu(NBCS_FLOW_DOUBLE_GYRE, 0.0, 8.0, x, y, params)
    ftle = ftle_grid_2D_gpu(fm, 8.0, 0.1, 0.1)
    evals, evecs = C_eig_2D_gpu(fm, 0.1, 0.1)
    pts = ftle_ridge_pts_gpu(ftle, np.ascontiguousarray(evecs[..., :, 1]), x, y)
    # the 3 x 3 x 3 spline case of the reference's tests/test_flows.py
    ts = np.array([0.0, 0.1, 0.2])
    xs = np.array([0.0, 0.5, 1.0])
    T3, X3, Y3 = np.meshgrid(ts, xs, xs, indexing="ij")
    U = np.sin(X3) * np.cos(Y3) + np.sin(T3)
    V = np.cos(X3) * np.sin(Y3) + np.cos(T3)
    sf = SplineFlowGPU(ts, xs, xs, U, V)
    ti, xi = np.array([0.05, 0.12, 0.18]), np.array([0.1, 0.4, 0.7])
    Ti, Xi, Yi = np.meshgrid(ti, xi, xi, indexing="ij")
    vel = eval_rhs_gpu(sf.flow, np.column_stack((Ti.ravel(), Xi.ravel(), Yi.ravel())), [1.0])
    sfm = flowmap_grid_2D_gpu(sf.flow, 0.02, 0.15, xi, xi, [1.0])
    sf.mem.free()
    print(json.dumps({"flowmap": fm.tolist(), "ftle": ftle.tolist(), "evals": evals.tolist(),
                      "ridge_pts": pts.tolist(), "spline_Cu": sf.cu.tolist(),
                      "spline_Cv": sf.cv.tolist(), "spline_vel": vel.tolist(),
                      "spline_flowmap": sfm.tolist(), "torch_loaded": "torch" in sys.modules}))
