"""FTLE ridge extraction: drop-in for src/numbacs/extraction/ridges.py.

``ftle_ridge_pts`` (ridges.py:9-76) and the ``_ftle_ridges`` mask
(ridges.py:79-154) run as one percentile-selection + stencil + order-preserving
compaction pipeline on the GPU (csrc/ridges.cu).  The threshold is the
reference's ``np.percentile(f, percentile)`` as numba evaluates it, or 0 when
``percentile == 0``.
"""
import numpy as np
import torch

from .. import _device as D
from .. import _lib


def _run(f, eigvec_max, x, y, sdd_thresh, percentile, want_mask, want_full):
    D.require_cuda()
    fd = D.to_dev(f)
    ev = D.to_dev(eigvec_max)
    xd, yd = D.to_dev(x), D.to_dev(y)
    if fd.dim() != 2:
        raise ValueError("f must have shape (nx, ny)")
    nx, ny = fd.shape
    if tuple(ev.shape) != (nx, ny, 2):
        raise ValueError("eigvec_max must have shape (nx, ny, 2)")
    L = _lib.load()
    nbytes = L.nbcs_ridge_scratch_bytes(nx, ny)
    scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=fd.device)
    mask = D.empty((nx, ny), torch.uint8) if want_mask else None
    full = D.empty((nx * ny, 2)) if want_full else None
    pts = D.empty((nx * ny, 2))
    n_out = D.empty((1,), torch.int64)
    _lib.check(L.nbcs_ridge_pts(D.ptr(fd), D.ptr(ev), D.ptr(xd), nx, D.ptr(yd), ny,
                                float(sdd_thresh), float(percentile), D.ptr(mask), D.ptr(full),
                                D.ptr(pts), D.ptr(n_out), D.ptr(scratch), nbytes, D.stream_ptr()))
    return pts, n_out, mask, full


def ftle_ridge_pts(f, eigvec_max, x, y, sdd_thresh=0.0, percentile=0):
    """Sub-pixel ridge points (k, 2), in row-major grid order."""
    as_torch = D.is_torch(f, eigvec_max)
    pts, n_out, _, _ = _run(f, eigvec_max, x, y, sdd_thresh, percentile, False, False)
    k = int(n_out.item())
    return D.finish(pts[:k], as_torch)


def _ftle_ridges(f, eigvec_max, x, y, sdd_thresh=0.0, percentile=0):
    """(r_pts (nx*ny, 2) zero off the ridge, ridge_bool (nx, ny), nx, ny)."""
    as_torch = D.is_torch(f, eigvec_max)
    _, _, mask, full = _run(f, eigvec_max, x, y, sdd_thresh, percentile, True, True)
    nx, ny = mask.shape
    return D.finish(full, as_torch), D.finish(mask.to(torch.bool), as_torch), nx, ny


def ftle_ridges(f, eigvec_max, x, y, sdd_thresh=0.0, percentile=0, min_ridge_pts=3):
    """Connected ridges: list of (m, 2) point arrays, one per 8-connected
    component of the ridge mask with at least ``min_ridge_pts`` points,
    components ordered by their first grid point in row-major order
    (ridges.py:186-229; scipy.ndimage.label with a full 3x3 structure).

    The mask and ridge points come from the GPU; the component labelling of
    the (small, sparse) mask is done with scipy.ndimage.label on the host, as
    in the reference.
    """
    from scipy.ndimage import generate_binary_structure, label

    as_torch = D.is_torch(f, eigvec_max)
    r_pts, ridge_bool, nx, ny = _ftle_ridges(f, eigvec_max, x, y, sdd_thresh, percentile)
    rb = ridge_bool.cpu().numpy() if isinstance(ridge_bool, torch.Tensor) else ridge_bool
    rp = r_pts.cpu().numpy() if isinstance(r_pts, torch.Tensor) else r_pts
    labels, nlabels = label(rb, structure=generate_binary_structure(2, 2))
    ind_arr = np.arange(nx * ny).reshape(nx, ny)
    ridges = []
    for i in range(1, nlabels + 1):
        inds = ind_arr[labels == i]
        if len(inds) >= min_ridge_pts:
            r = rp[inds, :]
            ridges.append(torch.from_numpy(r).to(D.device()) if as_torch else r)
    return ridges
