"""Device-array plumbing for the drop-in API.

Public functions accept numpy arrays (the reference's types) or torch tensors.
Numpy inputs are copied to the current CUDA device and results come back as
numpy float64 arrays in C order, like the reference returns; torch inputs stay
on the device and results are returned as torch tensors with no host copy.
"""
import numpy as np
import torch

from . import _lib

# bytes moved between host and device by the numpy-in / numpy-out paths
transfer_bytes = {"h2d": 0, "d2h": 0}


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("numbacs_gb300 needs a CUDA device (no CPU fallback)")
    _lib.load()


def is_torch(*arrays):
    return any(isinstance(a, torch.Tensor) for a in arrays if a is not None)


def device():
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr():
    return ctypes_void(torch.cuda.current_stream().cuda_stream)


def ctypes_void(v):
    import ctypes
    return ctypes.c_void_p(int(v)) if v else None


def to_dev(a, dtype=torch.float64):
    """Contiguous CUDA tensor of `dtype` holding `a` (no copy if already so)."""
    if a is None:
        return None
    if isinstance(a, torch.Tensor):
        t = a
        if t.device.type != "cuda":
            t = t.to(device())
        if t.dtype != dtype:
            t = t.to(dtype)
        return t.contiguous()
    arr = np.ascontiguousarray(np.asarray(a), dtype=_np_dtype(dtype))
    transfer_bytes["h2d"] += arr.nbytes
    return torch.from_numpy(arr).to(device(), non_blocking=False)


def mask_to_dev(mask):
    if mask is None:
        return None
    if isinstance(mask, torch.Tensor):
        return to_dev(mask.to(torch.bool), torch.uint8)
    return to_dev(np.asarray(mask, dtype=bool).astype(np.uint8), torch.uint8)


def _np_dtype(dtype):
    return {torch.float64: np.float64, torch.float32: np.float32, torch.uint8: np.uint8,
            torch.int32: np.int32, torch.int64: np.int64}[dtype]


def ptr(t):
    return ctypes_void(t.data_ptr()) if t is not None else None


def empty(shape, dtype=torch.float64):
    return torch.empty(shape, dtype=dtype, device=device())


def finish(t, as_torch):
    """Return a device tensor as-is (torch callers) or as a numpy array."""
    if as_torch:
        return t
    transfer_bytes["d2h"] += t.numel() * t.element_size()
    return t.cpu().numpy()
