"""Flow-map integration: the drop-in for numbacs.integration.flowmap_grid_2D.

Reference: src/numbacs/integration.py:123-182.  The reference loops over the
particle grid with numba ``prange`` and calls numbalsoda's DOP853 per particle;
here one CUDA thread integrates one particle (kernels in csrc/flowmap64.cu and
csrc/flowmap32.cu).  Solver time runs over ``params[0] * [t0, t0 + T]`` and the
right-hand side is evaluated at ``params[0] * t`` and multiplied by
``params[0]``, exactly as in the reference.
"""
import warnings

import numpy as np
import torch

from . import _device as D
from . import _lib
from .flows import _check_callable_flow

_PREC = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}
STATUS_NAMES = {0: "ok", 1: "masked", -2: "max_steps", -3: "step_underflow", -4: "nonfinite"}


def flowmap_grid_2D(funcptr, t0, T, x, y, params, method="dop853", rtol=1e-6, atol=1e-8,
                    mask=None, *, precision="fp64", max_steps=100000, return_status=False,
                    return_stats=False, out=None, lanes_per_particle=0, blocks_per_sm=0,
                    step_model=None, step_model_mode=1):
    """Flow map at t0+T of every particle on the grid x by y -> (nx, ny, 2).

    Same positional signature and defaults as the reference.  Keyword-only
    extras: ``precision`` ("fp64" = the plain path, every operation in IEEE
    double; "mixed" = FP32 stages with compensated FP32-pair positions),
    ``max_steps`` (attempted-step limit), ``return_status`` (also return the
    per-particle int32 status), ``return_stats`` (also return (nx, ny, 3)
    accepted / rejected / RHS-evaluation counts), ``out`` (a preallocated
    (nx, ny, 2) float64 CUDA tensor), and the launch-shape knobs
    ``lanes_per_particle`` (mixed spline path: 1, 2 or 4 lanes share one
    particle's RHS; 0 = automatic) and ``blocks_per_sm`` (0 = one block per
    particle tile).  ``step_model`` (a learned.StepProposer; mixed precision,
    spline flows) proposes each step from local flow features, and
    ``step_model_mode`` combines its proposal h_m with the controller's h_c
    (0: h_m, 1: min(h_m, h_c), 2: sqrt(h_m h_c)).

    ``method="lsoda"`` raises NotImplementedError: only DOP853 runs on the GPU.
    Particles whose integration failed (step limit, step underflow, NaN) keep
    their last position; numpy callers that did not ask for the status get
    a warning with the counts.
    """
    if method.lower() != "dop853":
        raise NotImplementedError("method=%r: only 'dop853' is implemented on the GPU" % method)
    flow = _check_callable_flow(funcptr)
    if precision not in _PREC:
        raise ValueError("precision must be 'fp64' or 'mixed'")
    D.require_cuda()
    as_torch = D.is_torch(x, y, out)
    xd, yd = D.to_dev(x), D.to_dev(y)
    nx, ny = xd.numel(), yd.numel()
    md = D.mask_to_dev(mask)
    if md is not None and tuple(md.shape) != (nx, ny):
        raise ValueError("mask must have shape (nx, ny)")
    prm = np.ascontiguousarray(
        params.cpu().numpy() if isinstance(params, torch.Tensor) else params, dtype=np.float64)
    if out is None:
        out = D.empty((nx, ny, 2))
    elif tuple(out.shape) != (nx, ny, 2) or out.dtype != torch.float64 or not out.is_contiguous():
        raise ValueError("out must be a contiguous float64 (nx, ny, 2) tensor")
    status = D.empty((nx, ny), torch.int32)
    stats = D.empty((nx, ny, 3), torch.int32) if return_stats else None
    opts = _lib.NbcsOpts()
    opts.precision = _PREC[precision]
    opts.max_steps = int(max_steps)
    opts.lanes_per_particle = int(lanes_per_particle)
    opts.blocks_per_sm = int(blocks_per_sm)
    if step_model is not None:
        opts.step_model = step_model.blob.data_ptr()
        opts.step_model_mode = int(step_model_mode)
    opts.stats = stats.data_ptr() if stats is not None else None
    L = _lib.load()
    _lib.check(L.nbcs_flowmap_grid_2d(flow.struct, float(t0), float(T), D.ptr(xd), nx, D.ptr(yd),
                                      ny, prm.ctypes.data_as(_lib._vp), len(prm), float(rtol),
                                      float(atol), D.ptr(md), D.ptr(out), D.ptr(status), opts,
                                      D.stream_ptr()))
    if not return_status and not as_torch:  # torch callers stay asynchronous
        bad = status[(status != 0) & (status != 1)]
        if bad.numel():
            vals, counts = torch.unique(bad, return_counts=True)
            msg = ", ".join("%s: %d" % (STATUS_NAMES.get(int(v), int(v)), int(c))
                            for v, c in zip(vals.tolist(), counts.tolist()))
            warnings.warn("flowmap_grid_2D: %d particles did not finish (%s)" % (bad.numel(), msg),
                          RuntimeWarning, stacklevel=2)
    res = [D.finish(out, as_torch)]
    if return_status:
        res.append(D.finish(status, as_torch))
    if return_stats:
        res.append(D.finish(stats, as_torch))
    return res[0] if len(res) == 1 else tuple(res)
