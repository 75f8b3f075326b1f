"""FTLE ridges as ordered curves: the drop-in for ftle_ordered_ridges
(src/numbacs/extraction/ridges.py:720-1054).

The ridge test of every grid point (ridges.py:232-318: FTLE above the
threshold, negative second directional derivative along eigvec_max, sub-pixel
point inside the cell) runs on the GPU -- the same kernel as ftle_ridge_pts.
What follows is serial by nature and runs on the host over the ridge points
only, in native code (nbcs_order_ridges, csrc/ordered.cu): the points are
visited in increasing second directional derivative and each unvisited one
grows a curve in both directions; curves whose endpoints lie within
`dist_tol` with tangents within `ep_tan_ang` are joined, and joined curves
shorter than `min_ridge_pts` points are dropped.  The order of every decision
follows the reference, so the curves and their point order are the
reference's.
"""
import ctypes
import math

import numpy as np

from .. import _lib


def ordered_from_ridge_field(f, eigvec_max, x, y, ridge_mask, r_pts, dist_tol,
                             ep_tan_ang=math.pi / 4, min_ridge_pts=5, sdd_thresh=0.0, c=1.0):
    """ftle_ordered_ridges from the ridge mask (nx, ny) and the full ridge-point
    array (nx * ny, 2) of the ridge test (host arrays) -> list of (m, 2)."""
    f = np.ascontiguousarray(f, np.float64)
    ev = np.ascontiguousarray(eigvec_max, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    nx, ny = f.shape
    mask = np.ascontiguousarray(ridge_mask, np.uint8).reshape(nx, ny)
    rp = np.ascontiguousarray(r_pts, np.float64).reshape(nx * ny, 2)
    cap = max(1, int(mask.sum()))
    pts = np.empty((cap, 2))
    lens = np.empty(cap, np.int64)
    n_pts, n_ridges = ctypes.c_int64(0), ctypes.c_int64(0)
    vp = _lib._vp
    _lib.check(_lib.load().nbcs_order_ridges(
        f.ctypes.data_as(vp), ev.ctypes.data_as(vp), x.ctypes.data_as(vp), nx,
        y.ctypes.data_as(vp), ny, mask.ctypes.data_as(vp), rp.ctypes.data_as(vp),
        float(dist_tol), float(ep_tan_ang), int(min_ridge_pts), float(sdd_thresh), float(c),
        pts.ctypes.data_as(vp), cap, lens.ctypes.data_as(vp), cap, ctypes.byref(n_pts),
        ctypes.byref(n_ridges)))
    out, p = [], 0
    for n in lens[:n_ridges.value]:
        out.append(pts[p:p + n].copy())
        p += n
    return out


def ftle_ordered_ridges(f, eigvec_max, x, y, dist_tol, ep_tan_ang=math.pi / 4, min_ridge_pts=5,
                        sdd_thresh=0.0, percentile=0, c=1.0):
    """Ordered FTLE ridge curves (a list of (m, 2) arrays), same signature and
    defaults as the reference; the ridge test runs on the GPU."""
    from .ridges import _ftle_ridges
    r_full, mask, _, _ = _ftle_ridges(f, eigvec_max, x, y, sdd_thresh, percentile)
    if hasattr(mask, "cpu"):
        mask, r_full = mask.cpu().numpy(), r_full.cpu().numpy()
    fh = f.cpu().numpy() if hasattr(f, "cpu") else f
    eh = eigvec_max.cpu().numpy() if hasattr(eigvec_max, "cpu") else eigvec_max
    xh = x.cpu().numpy() if hasattr(x, "cpu") else x
    yh = y.cpu().numpy() if hasattr(y, "cpu") else y
    return ordered_from_ridge_field(fh, eh, xh, yh, mask, r_full, dist_tol, ep_tan_ang,
                                    min_ridge_pts, sdd_thresh, c)
