"""ctypes bindings for the C oracle (TEST INFRASTRUCTURE ONLY).

Every function mirrors one reference NumbaCS function on numpy arrays:

  flowmap           src/numbacs/integration.py:8-62
  flowmap_n         src/numbacs/integration.py:65-121 (and flowmap_n_grid_2D :468-534)
  flowmap_grid_2D   src/numbacs/integration.py:123-182
  ftle_grid_2D      src/numbacs/diagnostics.py:21-65
  C_tensor_2D       src/numbacs/diagnostics.py:69-111
  C_eig_2D          src/numbacs/diagnostics.py:200-244
  ftle_from_eig     src/numbacs/diagnostics.py:247-269
  ftle_ridge_pts    src/numbacs/extraction/ridges.py:9-76
  _ftle_ridges      src/numbacs/extraction/ridges.py:79-154
  ftle_ridges       src/numbacs/extraction/ridges.py:186-229 (labelling restated
                    as 8-connected components numbered in raster order of their
                    first pixel, the scipy.ndimage.label convention)
  prefilter_3d      src/numbacs/flows.py:9-46 (interpolation.splines.prefilter, k=3)
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "liboracle.so")

FLOW_DOUBLE_GYRE = 0
FLOW_BICKLEY = 1
FLOW_SPLINE2D = 2

OK, MASKED, MAX_STEPS, STEP_UNDERFLOW, NONFINITE = 0, 1, -2, -3, -4


def build(force=False):
    """Compile oracle.c into _build/liboracle.so with gcc (-O2 -ffp-contract=off)."""
    src = os.path.join(_HERE, "oracle.c")
    hdr = os.path.join(_HERE, "oracle.h")
    tab = os.path.join(_HERE, "..", "numbacs_gb300", "csrc", "dop853_tableau.h")
    if not force and os.path.exists(_LIB_PATH):
        mt = os.path.getmtime(_LIB_PATH)
        if all(os.path.getmtime(p) <= mt for p in (src, hdr, tab)):
            return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
           "-shared", "-std=c11", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


_lib = None


class _Flow(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("spherical", ctypes.c_int), ("extrap", ctypes.c_int),
                ("r", ctypes.c_double), ("grid", ctypes.c_double * 9),
                ("cu", ctypes.c_void_p), ("cv", ctypes.c_void_p), ("libm", ctypes.c_int)]


def _dp(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, d, i, i64 = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int64
        L.orc_rhs.argtypes = [vp, d, vp, vp, vp]
        L.orc_prefilter_3d.argtypes = [vp, i, i, i, vp]
        L.orc_eval_spline_3d.argtypes = [vp, vp, i, d, d, d]
        L.orc_eval_spline_3d.restype = d
        L.orc_flowmap_grid_2d.argtypes = [vp, d, d, vp, i, vp, i, vp, i, d, d, vp, vp, vp, vp, i, i]
        L.orc_flowmap_pts.argtypes = [vp, d, d, vp, ctypes.c_long, vp, d, d, vp, vp, vp, i, i]
        L.orc_flowmap_n_pts.argtypes = [vp, vp, ctypes.c_long, vp, i, vp, d, d, vp, vp, vp, i, i]
        L.orc_ftle_grid_2d.argtypes = [vp, i, i, d, d, d, vp, vp]
        L.orc_c_eig_2d.argtypes = [vp, i, i, d, d, vp, vp, vp]
        L.orc_ftle_from_eig.argtypes = [vp, i64, d, vp]
        L.orc_percentile.argtypes = [vp, i64, d]
        L.orc_percentile.restype = d
        L.orc_ridge_field.argtypes = [vp, vp, vp, i, vp, i, d, d, vp, vp]
        L.orc_ridge_field_d.argtypes = [vp, vp, vp, i, vp, i, d, d, d, d, vp, vp]
        L.orc_flowmap_aux_grid_2d.argtypes = [vp, d, d, vp, i, vp, i, vp, d, i, i, d, d, vp, vp,
                                              vp, vp, i, i]
        L.orc_c_eig_aux_2d.argtypes = [vp, i, i, d, d, d, i, vp, vp, vp]
        L.orc_c_tensor_2d.argtypes = [vp, i, i, i, d, vp, vp]
        L.orc_flowmap_compose.argtypes = [vp, i, i, i, i, vp, vp]
        for fn in (L.orc_cos_deg, L.orc_root8):
            fn.argtypes = [d]
            fn.restype = d
        _lib = L
    return _lib


class Flow:
    """Oracle-side flow description (analytic kind, or spline coefficients)."""

    def __init__(self, kind, grid=None, cu=None, cv=None, spherical=0, extrap=0, r=6371.0,
                 libm=False):
        self.kind = kind
        self.cu = None if cu is None else np.ascontiguousarray(cu, dtype=np.float64)
        self.cv = None if cv is None else np.ascontiguousarray(cv, dtype=np.float64)
        self.s = _Flow()
        self.s.kind = kind
        self.s.spherical = spherical
        self.s.extrap = extrap
        self.s.r = r
        if grid is not None:
            flat = [float(v) for g in grid for v in g]
            for k in range(9):
                self.s.grid[k] = flat[k]
        self.s.cu = _dp(self.cu)
        self.s.cv = _dp(self.cv)
        # libm=True: the reference's literal pow / cos calls instead of the
        # deterministic helpers shared with the GPU library (oracle.h)
        self.s.libm = int(bool(libm))

    @property
    def ptr(self):
        return ctypes.byref(self.s)


def double_gyre(libm=False):
    return Flow(FLOW_DOUBLE_GYRE, libm=libm)


def bickley_jet(libm=False):
    return Flow(FLOW_BICKLEY, libm=libm)


def spline_flow(grid, cu, cv, spherical=0, extrap=0, r=6371.0, libm=False):
    return Flow(FLOW_SPLINE2D, grid, cu, cv, spherical, extrap, r, libm)


def rhs(flow, t, y, params):
    y = np.ascontiguousarray(y, np.float64)
    p = np.ascontiguousarray(params, np.float64)
    dy = np.zeros(2)
    lib().orc_rhs(flow.ptr, float(t), _dp(y), _dp(dy), _dp(p))
    return dy


def prefilter_3d(f):
    f = np.ascontiguousarray(f, np.float64)
    nt, nx, ny = f.shape
    c = np.zeros((nt + 2, nx + 2, ny + 2))
    rc = lib().orc_prefilter_3d(_dp(f), nt, nx, ny, _dp(c))
    if rc != 0:
        raise RuntimeError("oracle prefilter failed (%d)" % rc)
    return c


def get_interp_arrays_2D(tvals, xvals, yvals, U, V):
    nt, nx, ny = U.shape
    grid = ((tvals[0], tvals[-1], nt), (xvals[0], xvals[-1], nx), (yvals[0], yvals[-1], ny))
    return grid, prefilter_3d(U), prefilter_3d(V)


def eval_spline_3d(grid, c, t, x, y, extrap=0):
    g = np.array([float(v) for gg in grid for v in gg])
    c = np.ascontiguousarray(c, np.float64)
    return lib().orc_eval_spline_3d(_dp(g), _dp(c), extrap, float(t), float(x), float(y))


def flowmap_grid_2D(flow, t0, T, x, y, params, rtol=1e-6, atol=1e-8, mask=None,
                    nmax=100000, nthreads=0, return_status=False):
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    p = np.ascontiguousarray(params, np.float64)
    nx, ny = len(x), len(y)
    out = np.zeros((nx, ny, 2))
    status = np.zeros((nx, ny), np.int32)
    stats = np.zeros((nx, ny, 3), np.int32)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib().orc_flowmap_grid_2d(flow.ptr, float(t0), float(T), _dp(x), nx, _dp(y), ny, _dp(p),
                              len(p), float(rtol), float(atol), _dp(m), _dp(out), _dp(status),
                              _dp(stats), int(nmax), int(nthreads))
    if return_status:
        return out, status, stats
    return out


def flowmap(flow, t0, T, pts, params, rtol=1e-6, atol=1e-8, mask=None, nmax=100000, nthreads=0,
            return_status=False):
    """integration.py:8-62 (method dop853): pts (npts, 2) -> (npts, 2)."""
    pts = np.ascontiguousarray(pts, np.float64)
    p = np.ascontiguousarray(params, np.float64)
    npts = pts.shape[0]
    out = np.zeros((npts, 2))
    status = np.zeros(npts, np.int32)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib().orc_flowmap_pts(flow.ptr, float(t0), float(T), _dp(pts), npts, _dp(p), float(rtol),
                          float(atol), _dp(m), _dp(out), _dp(status), int(nmax), int(nthreads))
    return (out, status) if return_status else out


def flowmap_n(flow, t0, T, pts, params, n=2, rtol=1e-6, atol=1e-8, mask=None, nmax=100000,
              nthreads=0, return_status=False):
    """integration.py:65-121 (method dop853): pts (npts, 2) -> ((npts, n, 2), t_eval), the
    positions at t_eval = params[0] * linspace(t0, t0 + T, n) by dense output of one run."""
    pts = np.ascontiguousarray(pts, np.float64)
    p = np.ascontiguousarray(params, np.float64)
    te = np.ascontiguousarray(p[0] * np.linspace(t0, t0 + T, n))
    npts = pts.shape[0]
    out = np.zeros((npts, n, 2))
    status = np.zeros(npts, np.int32)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib().orc_flowmap_n_pts(flow.ptr, _dp(pts), npts, _dp(te), int(n), _dp(p), float(rtol),
                            float(atol), _dp(m), _dp(out), _dp(status), int(nmax), int(nthreads))
    res = (out, p[0] * te)
    return res + (status,) if return_status else res


def flowmap_n_grid_2D(flow, t0, T, x, y, params, n=50, rtol=1e-6, atol=1e-8, mask=None,
                      nmax=100000, nthreads=0, return_status=False):
    """integration.py:468-534: the grid's points through flowmap_n -> ((nx, ny, n, 2), t_eval)."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    X, Y = np.meshgrid(x, y, indexing="ij")
    m = None if mask is None else np.asarray(mask).ravel()
    r = flowmap_n(flow, t0, T, np.column_stack((X.ravel(), Y.ravel())), params, n, rtol, atol, m,
                  nmax, nthreads, return_status)
    out = (r[0].reshape(len(x), len(y), n, 2), r[1])
    return out + (r[2].reshape(len(x), len(y)),) if return_status else out


def flowmap_aux_grid_2D(flow, t0, T, x, y, params, h=1e-5, eig_main=True, compute_edge=True,
                        rtol=1e-6, atol=1e-8, mask=None, nmax=100000, nthreads=0,
                        return_status=False):
    """integration.py:249-464 (method dop853)."""
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    p = np.ascontiguousarray(params, np.float64)
    nx, ny = len(x), len(y)
    na = 5 if eig_main else 4
    out = np.zeros((nx, ny, na, 2))
    status = np.zeros((nx, ny, na), np.int32)
    stats = np.zeros((nx, ny, na, 3), np.int32)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib().orc_flowmap_aux_grid_2d(flow.ptr, float(t0), float(T), _dp(x), nx, _dp(y), ny, _dp(p),
                                  float(h), int(bool(eig_main)), int(bool(compute_edge)),
                                  float(rtol), float(atol), _dp(m), _dp(out), _dp(status),
                                  _dp(stats), int(nmax), int(nthreads))
    if return_status:
        return out, status, stats
    return out


def C_tensor_2D(flowmap_aux, dx, dy, h=1e-5, mask=None):
    """diagnostics.py:69-111: (nx, ny, 3) C11, C12, C22 from the +-h particles."""
    F = np.ascontiguousarray(flowmap_aux, np.float64)
    nx, ny, na = F.shape[:3]
    C = np.zeros((nx, ny, 3))
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib().orc_c_tensor_2d(_dp(F), nx, ny, na, float(h), _dp(m), _dp(C))
    return C


def C_eig_aux_2D(flowmap_aux, dx, dy, h=1e-5, eig_main=True, mask=None):
    """diagnostics.py:113-197."""
    F = np.ascontiguousarray(flowmap_aux, np.float64)
    nx, ny = F.shape[:2]
    if F.shape[2] != (5 if eig_main else 4):
        raise ValueError("flowmap_aux has %d aux particles" % F.shape[2])
    ev = np.zeros((nx, ny, 2))
    vec = np.zeros((nx, ny, 2, 2))
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib().orc_c_eig_aux_2d(_dp(F), nx, ny, float(dx), float(dy), float(h), int(bool(eig_main)),
                           _dp(m), _dp(ev), _dp(vec))
    return ev, vec


def flowmap_composition(flowmaps, grid, nT, first=0):
    """integration.py:609-641; grid = ((x0, x1, nx), (y0, y1, ny))."""
    F = np.ascontiguousarray(flowmaps, np.float64)
    (x0, x1, nx), (y0, y1, ny) = grid
    g = np.array([x0, x1, nx, y0, y1, ny], np.float64)
    out = np.zeros((int(nx), int(ny), 2))
    lib().orc_flowmap_compose(_dp(F), int(nT), int(first), int(nx), int(ny), _dp(g), _dp(out))
    return out


def flowmap_composition_initial(flow, t0, T, h, x, y, grid, params, **kw):
    """integration.py:644-685."""
    nT = abs(round(T / h))
    fms = np.zeros((nT, len(x), len(y), 2))
    for k in range(nT):
        fms[k] = flowmap_grid_2D(flow, t0, h, x, y, params, **kw)
        t0 += h
    return flowmap_composition(fms, grid, nT), fms, nT


def flowmap_composition_step(flowmaps, flow, t0, h, nT, x, y, grid, params, **kw):
    """integration.py:688-737 (shifts flowmaps in place, as the reference does)."""
    flowmaps[:-1] = flowmaps[1:].copy()
    flowmaps[-1] = flowmap_grid_2D(flow, t0, h, x, y, params, **kw)
    return flowmap_composition(flowmaps, grid, nT), flowmaps


def ftle_grid_2D(flowmap, T, dx, dy, mask=None):
    F = np.ascontiguousarray(flowmap, np.float64)
    nx, ny = F.shape[:2]
    out = np.zeros((nx, ny))
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib().orc_ftle_grid_2d(_dp(F), nx, ny, float(T), float(dx), float(dy), _dp(m), _dp(out))
    return out


def C_eig_2D(flowmap, dx, dy, mask=None):
    F = np.ascontiguousarray(flowmap, np.float64)
    nx, ny = F.shape[:2]
    ev = np.zeros((nx, ny, 2))
    vec = np.zeros((nx, ny, 2, 2))
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib().orc_c_eig_2d(_dp(F), nx, ny, float(dx), float(dy), _dp(m), _dp(ev), _dp(vec))
    return ev, vec


def ftle_from_eig(eigval_max, T):
    e = np.ascontiguousarray(eigval_max, np.float64)
    out = np.zeros(e.shape)
    lib().orc_ftle_from_eig(_dp(e), e.size, float(T), _dp(out))
    return out


def percentile(f, q):
    f = np.ascontiguousarray(f, np.float64).ravel()
    return lib().orc_percentile(_dp(f), f.size, float(q))


def cos_deg(d):
    return lib().orc_cos_deg(float(d))


def root8(x):
    return lib().orc_root8(float(x))


def ridge_field(f, eigvec_max, x, y, sdd_thresh=0.0, percentile_=0):
    """(r_pts (nx*ny, 2), ridge mask (nx, ny) bool, threshold) -- _ftle_ridges."""
    return _ridge_field(f, eigvec_max, x, y, sdd_thresh, percentile_)


def _ridge_field(f, eigvec_max, x, y, sdd_thresh=0.0, percentile_=0, f_min=None, dxdy=None):
    f = np.ascontiguousarray(f, np.float64)
    ev = np.ascontiguousarray(eigvec_max, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    nx, ny = f.shape
    if f_min is None:
        f_min = 0.0 if percentile_ == 0 else percentile(f, percentile_)
    mask = np.zeros((nx, ny), np.uint8)
    rpts = np.zeros((nx * ny, 2))
    if dxdy is None:
        lib().orc_ridge_field(_dp(f), _dp(ev), _dp(x), nx, _dp(y), ny, float(sdd_thresh),
                              float(f_min), _dp(mask), _dp(rpts))
    else:
        lib().orc_ridge_field_d(_dp(f), _dp(ev), _dp(x), nx, _dp(y), ny, float(dxdy[0]),
                                float(dxdy[1]), float(sdd_thresh), float(f_min), _dp(mask),
                                _dp(rpts))
    return rpts, mask.astype(bool), f_min


def ftle_ridge_pts(f, eigvec_max, x, y, sdd_thresh=0.0, percentile=0):
    rpts, mask, _ = _ridge_field(f, eigvec_max, x, y, sdd_thresh, percentile)
    return rpts[mask.ravel()]


def ridge_field_fmin(f, eigvec_max, x, y, dx, dy, sdd_thresh, f_min):
    """(r_pts (nx*ny, 2), ridge mask (nx, ny) bool) with the threshold and the
    grid spacing given (a row block of a sharded field)."""
    rpts, mask, _ = _ridge_field(f, eigvec_max, x, y, sdd_thresh, f_min=f_min, dxdy=(dx, dy))
    return rpts, mask


def ridge_pts_fmin(f, eigvec_max, x, y, dx, dy, sdd_thresh, f_min):
    """ftle_ridge_pts with the threshold and the grid spacing given."""
    rpts, mask, _ = _ridge_field(f, eigvec_max, x, y, sdd_thresh, f_min=f_min, dxdy=(dx, dy))
    return rpts[mask.ravel()]


def _ftle_ridges(f, eigvec_max, x, y, sdd_thresh=0.0, percentile=0):
    rpts, mask, _ = _ridge_field(f, eigvec_max, x, y, sdd_thresh, percentile)
    return rpts, mask, f.shape[0], f.shape[1]


def label8(mask):
    """8-connected component labels numbered in raster order of first pixel
    (pure Python flood fill; small inputs only)."""
    mask = np.asarray(mask, bool)
    nx, ny = mask.shape
    lab = np.zeros((nx, ny), np.int64)
    n = 0
    for i in range(nx):
        for j in range(ny):
            if mask[i, j] and lab[i, j] == 0:
                n += 1
                stack = [(i, j)]
                lab[i, j] = n
                while stack:
                    a, b = stack.pop()
                    for da in (-1, 0, 1):
                        for db in (-1, 0, 1):
                            u, v = a + da, b + db
                            if 0 <= u < nx and 0 <= v < ny and mask[u, v] and lab[u, v] == 0:
                                lab[u, v] = n
                                stack.append((u, v))
    return lab, n


def ftle_ridges(f, eigvec_max, x, y, sdd_thresh=0.0, percentile=0, min_ridge_pts=3):
    rpts, mask, nx, ny = _ftle_ridges(f, eigvec_max, x, y, sdd_thresh, percentile)
    lab, n = label8(mask)
    ind = np.arange(nx * ny).reshape(nx, ny)
    out = []
    for k in range(1, n + 1):
        inds = ind[lab == k]
        if len(inds) >= min_ridge_pts:
            out.append(rpts[inds])
    return out


# reference default parameters (flows.py:1162-1169 and :1217-1235)
def double_gyre_params(int_direction=1.0):
    return np.array([int_direction, 0.1, 0.25, 0.0, 0.2 * np.pi, 0.0])


def bickley_params():
    r_e = 6371.0e-3
    U0 = 86400 * 62.66e-6
    L = 1770.0e-3
    c2 = 0.205 * U0
    c3 = 0.461 * U0
    c1 = c3 + (np.sqrt(5) - 1) * (c2 - c3)
    return np.array([1.0, U0, L, 0.0075, 0.15, 0.3, 2.0 / r_e, 4.0 / r_e, 6.0 / r_e, c1, c2, c3])
