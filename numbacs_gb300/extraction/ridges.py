"""FTLE ridge extraction: drop-in for src/numbacs/extraction/ridges.py.

``ftle_ridge_pts`` (ridges.py:9-76) and the ``_ftle_ridges`` mask
(ridges.py:79-154) run as one percentile-selection + stencil + order-preserving
compaction pipeline on the GPU (csrc/ridges.cu).  The threshold is the
reference's ``np.percentile(f, percentile)`` as numba evaluates it, or 0 when
``percentile == 0``.
"""
import torch

from .. import _device as D
from .. import _lib


def _run(f, eigvec_max, x, y, sdd_thresh, percentile, want_mask, want_full, f_min=None,
         dxdy=None):
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
    if f_min is None:
        _lib.check(L.nbcs_ridge_pts(D.ptr(fd), D.ptr(ev), D.ptr(xd), nx, D.ptr(yd), ny,
                                    float(sdd_thresh), float(percentile), D.ptr(mask),
                                    D.ptr(full), D.ptr(pts), D.ptr(n_out), D.ptr(scratch), nbytes,
                                    D.stream_ptr()))
    else:
        _lib.check(L.nbcs_ridge_pts_fmin(D.ptr(fd), D.ptr(ev), D.ptr(xd), nx, D.ptr(yd), ny,
                                         float(dxdy[0]), float(dxdy[1]), float(sdd_thresh),
                                         float(f_min), D.ptr(mask),
                                         D.ptr(full), D.ptr(pts), D.ptr(n_out), D.ptr(scratch),
                                         nbytes, D.stream_ptr()))
    return pts, n_out, mask, full


def ridge_pts_fmin(f, eigvec_max, x, y, dx, dy, sdd_thresh, f_min):
    """ftle_ridge_pts with the threshold f_min and the spacing dx, dy given (a
    row block of a field sharded over several GPUs: the global threshold and
    spacing) -> ridge points (k, 2), row-major."""
    as_torch = D.is_torch(f, eigvec_max)
    pts, n_out, _, _ = _run(f, eigvec_max, x, y, sdd_thresh, 0, False, False, f_min=f_min,
                            dxdy=(dx, dy))
    return D.finish(pts[:int(n_out.item())], as_torch)


def percentile(f, q):
    """np.percentile(f, q) as the reference's numba code evaluates it (float)."""
    D.require_cuda()
    fd = D.to_dev(f).reshape(-1)
    L = _lib.load()
    nbytes = L.nbcs_percentile_scratch_bytes(fd.numel())
    scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=fd.device)
    out = D.empty((1,))
    _lib.check(L.nbcs_percentile(D.ptr(fd), fd.numel(), float(q), D.ptr(out), D.ptr(scratch),
                                 nbytes, D.stream_ptr()))
    return float(out.item())


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


def label8(mask):
    """8-connected component labels of a (nx, ny) mask on the GPU, numbered
    1..n by first pixel in row-major order (scipy.ndimage.label with a 3x3
    structure).  Returns (labels int32 CUDA tensor, n)."""
    D.require_cuda()
    m = D.mask_to_dev(mask)
    nx, ny = m.shape
    L = _lib.load()
    nbytes = L.nbcs_label8_scratch_bytes(nx, ny)
    scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=m.device)
    labels = D.empty((nx, ny), torch.int32)
    n = D.empty((1,), torch.int32)
    _lib.check(L.nbcs_label8(D.ptr(m), nx, ny, D.ptr(labels), D.ptr(n), D.ptr(scratch), nbytes,
                             D.stream_ptr()))
    k = int(n.item())
    if k < 0:
        raise RuntimeError("label8: union-find did not converge")
    return labels, k


def ftle_ridges(f, eigvec_max, x, y, sdd_thresh=0.0, percentile=0, min_ridge_pts=3):
    """Connected ridges: list of (m, 2) point arrays, one per 8-connected
    component of the ridge mask with at least ``min_ridge_pts`` points,
    components ordered by their first grid point in row-major order and
    points within a ridge in row-major order (ridges.py:186-229).

    Mask, ridge points and component labels are computed on the GPU
    (csrc/ridges.cu, csrc/label.cu); the per-ridge split of the labelled
    points is a stable sort by label of the (few) ridge pixels.
    """
    as_torch = D.is_torch(f, eigvec_max)
    _, _, mask, full = _run(f, eigvec_max, x, y, sdd_thresh, percentile, True, True)
    labels, n = label8(mask)
    lab = labels.view(-1)
    idx = torch.nonzero(lab, as_tuple=True)[0]  # ascending: row-major
    labs = lab.index_select(0, idx).long()
    order = torch.sort(labs, stable=True).indices
    pts = full.index_select(0, idx.index_select(0, order))
    counts = torch.bincount(labs, minlength=n + 1)[1:].tolist()
    ridges, start = [], 0
    for c in counts:
        if c >= min_ridge_pts:
            r = pts[start:start + c]
            ridges.append(r if as_torch else r.cpu().numpy())
        start += c
    return ridges
