"""FTLE diagnostics: the drop-in for the FTLE part of numbacs.diagnostics.

Reference: src/numbacs/diagnostics.py:21-65 (ftle_grid_2D), :69-111
(C_tensor_2D), :113-197 (C_eig_aux_2D), :200-244 (C_eig_2D) and :247-269
(ftle_from_eig).  Each is one fused stencil kernel
(csrc/ftle.cu).  ``ftle_evec_2D`` is the fused form of the reference idiom
``C_eig_2D`` -> ``ftle_from_eig(eigvals[...,1], T)`` / ``eigvecs[...,:,1]`` that
feeds ridge extraction.
"""
import torch

from . import _device as D
from . import _lib


def _fm(flowmap):
    F = D.to_dev(flowmap)
    if F.dim() != 3 or F.shape[2] != 2:
        raise ValueError("flowmap must have shape (nx, ny, 2)")
    return F


def ftle_grid_2D(flowmap, T, dx, dy, mask=None):
    """FTLE field (nx, ny) from a flow map; borders and masked points are 0."""
    D.require_cuda()
    as_torch = D.is_torch(flowmap)
    F = _fm(flowmap)
    nx, ny = F.shape[:2]
    md = D.mask_to_dev(mask)
    out = D.empty((nx, ny))
    _lib.check(_lib.load().nbcs_ftle_grid_2d(D.ptr(F), nx, ny, float(T), float(dx), float(dy),
                                             D.ptr(md), D.ptr(out), D.stream_ptr()))
    return D.finish(out, as_torch)


def C_eig_2D(flowmap, dx, dy, mask=None):
    """Eigenvalues (nx, ny, 2) ascending and eigenvectors (nx, ny, 2, 2, in
    columns) of the Cauchy-Green tensor."""
    D.require_cuda()
    as_torch = D.is_torch(flowmap)
    F = _fm(flowmap)
    nx, ny = F.shape[:2]
    md = D.mask_to_dev(mask)
    ev = D.empty((nx, ny, 2))
    vec = D.empty((nx, ny, 2, 2))
    _lib.check(_lib.load().nbcs_c_eig_2d(D.ptr(F), nx, ny, float(dx), float(dy), D.ptr(md),
                                         D.ptr(ev), D.ptr(vec), D.stream_ptr()))
    return D.finish(ev, as_torch), D.finish(vec, as_torch)


def ftle_from_eig(eigval_max, T):
    """log(eigval_max) / (2|T|) where eigval_max > 1, else 0."""
    D.require_cuda()
    as_torch = D.is_torch(eigval_max)
    if isinstance(eigval_max, torch.Tensor) and eigval_max.is_cuda and eigval_max.dtype == torch.float64:
        e = eigval_max
        if not e.is_contiguous():
            e = e.contiguous()
    else:
        e = D.to_dev(eigval_max)
    out = D.empty(tuple(e.shape))
    _lib.check(_lib.load().nbcs_ftle_from_eig(D.ptr(e), e.numel(), 1, float(T), D.ptr(out),
                                              D.stream_ptr()))
    return D.finish(out, as_torch)


def ftle_evec_2D(flowmap, T, dx, dy, mask=None):
    """Fused C_eig_2D + ftle_from_eig: (ftle (nx, ny), eigvec_max (nx, ny, 2))."""
    D.require_cuda()
    as_torch = D.is_torch(flowmap)
    F = _fm(flowmap)
    nx, ny = F.shape[:2]
    md = D.mask_to_dev(mask)
    f = D.empty((nx, ny))
    v = D.empty((nx, ny, 2))
    _lib.check(_lib.load().nbcs_ftle_evec_2d(D.ptr(F), nx, ny, float(T), float(dx), float(dy),
                                             D.ptr(md), D.ptr(f), D.ptr(v), D.stream_ptr()))
    return D.finish(f, as_torch), D.finish(v, as_torch)


def C_eig_aux_2D(flowmap_aux, dx, dy, h=1e-5, eig_main=True, mask=None):
    """Cauchy-Green eigenvalues (nx, ny, 2) and eigenvectors (nx, ny, 2, 2) from
    the auxiliary-grid flow map of flowmap_aux_grid_2D (diagnostics.py:113-197):
    with ``eig_main`` eigenvectors from the +-h particle differences and
    eigenvalues from the centre particles' main-grid differences, else both
    from the +-h differences."""
    D.require_cuda()
    as_torch = D.is_torch(flowmap_aux)
    F = D.to_dev(flowmap_aux)
    na = 5 if eig_main else 4
    if F.dim() != 4 or F.shape[2] != na or F.shape[3] != 2:
        raise ValueError("flowmap_aux must have shape (nx, ny, %d, 2)" % na)
    nx, ny = int(F.shape[0]), int(F.shape[1])
    md = D.mask_to_dev(mask)
    ev = D.empty((nx, ny, 2))
    vec = D.empty((nx, ny, 2, 2))
    _lib.check(_lib.load().nbcs_c_eig_aux_2d(D.ptr(F), nx, ny, int(bool(eig_main)), float(dx),
                                             float(dy), float(h), D.ptr(md), D.ptr(ev),
                                             D.ptr(vec), D.stream_ptr()))
    return D.finish(ev, as_torch), D.finish(vec, as_torch)


def C_tensor_2D(flowmap_aux, dx, dy, h=1e-5, mask=None):
    """C11, C12, C22 (nx, ny, 3) of the Cauchy-Green tensor from the +-h
    particles of flowmap_aux_grid_2D's flow map (diagnostics.py:69-111), for
    2 <= i < nx-2, 2 <= j < ny-2; dx, dy are accepted as the reference does
    (its stencil does not use them)."""
    D.require_cuda()
    as_torch = D.is_torch(flowmap_aux)
    F = D.to_dev(flowmap_aux)
    if F.dim() != 4 or F.shape[2] < 4 or F.shape[3] != 2:
        raise ValueError("flowmap_aux must have shape (nx, ny, 4 or 5, 2)")
    nx, ny, na = int(F.shape[0]), int(F.shape[1]), int(F.shape[2])
    md = D.mask_to_dev(mask)
    C = D.empty((nx, ny, 3))
    _lib.check(_lib.load().nbcs_c_tensor_2d(D.ptr(F), nx, ny, na, float(h), D.ptr(md), D.ptr(C),
                                            D.stream_ptr()))
    return D.finish(C, as_torch)
