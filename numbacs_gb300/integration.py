"""Flow-map integration: the drop-in for numbacs.integration.flowmap_grid_2D,
flowmap, flowmap_n, flowmap_n_grid_2D, flowmap_grid_ND, flowmap_aux_grid_2D
and the flow-map composition functions.

Reference: src/numbacs/integration.py:123-182 (flowmap_grid_2D), :8-62
(flowmap), :65-121 (flowmap_n), :468-534 (flowmap_n_grid_2D), :186-247
(flowmap_grid_ND), :249-464
(flowmap_aux_grid_2D), :609-737 (flowmap_composition, _initial, _step).  The
reference loops over the particle grid with numba ``prange`` and calls
numbalsoda's DOP853 per particle; here one CUDA thread (or lane group)
integrates one particle (kernels in csrc/flowmap64.cu and csrc/flowmap32.cu).
Solver time runs over ``params[0] * [t0, t0 + T]`` and the right-hand side is
evaluated at ``params[0] * t`` and multiplied by ``params[0]``, exactly as in
the reference.  Composition is one gather kernel (csrc/compose.cu).
"""
import warnings

import numpy as np
import torch

from . import _device as D
from . import _lib
from .flows import _check_callable_flow

_PREC = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}
STATUS_NAMES = {0: "ok", 1: "masked", -2: "max_steps", -3: "step_underflow", -4: "nonfinite"}


def _warn_unfinished(name, status):
    bad = status[(status != 0) & (status != 1)]
    if bad.numel():
        vals, counts = torch.unique(bad, return_counts=True)
        msg = ", ".join("%s: %d" % (STATUS_NAMES.get(int(v), int(v)), int(c))
                        for v, c in zip(vals.tolist(), counts.tolist()))
        warnings.warn("%s: %d particles did not finish (%s)" % (name, bad.numel(), msg),
                      RuntimeWarning, stacklevel=3)


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
        opts.step_model = step_model.proposal_blob().data_ptr()
        opts.step_model_mode = int(step_model_mode)
    opts.stats = stats.data_ptr() if stats is not None else None
    L = _lib.load()
    _lib.check(L.nbcs_flowmap_grid_2d(flow.struct, float(t0), float(T), D.ptr(xd), nx, D.ptr(yd),
                                      ny, prm.ctypes.data_as(_lib._vp), len(prm), float(rtol),
                                      float(atol), D.ptr(md), D.ptr(out), D.ptr(status), opts,
                                      D.stream_ptr()))
    if not return_status and not as_torch:  # torch callers stay asynchronous
        _warn_unfinished("flowmap_grid_2D", status)
    res = [D.finish(out, as_torch)]
    if return_status:
        res.append(D.finish(status, as_torch))
    if return_stats:
        res.append(D.finish(stats, as_torch))
    return res[0] if len(res) == 1 else tuple(res)


def flowmap(funcptr, t0, T, pts, params, method="dop853", rtol=1e-6, atol=1e-8, mask=None, *,
            precision="fp64", max_steps=100000, return_status=False, return_stats=False):
    """Flow map at t0+T of a list of points pts (npts, 2) -> (npts, 2)
    (integration.py:8-62): the particles of flowmap_grid_2D, taken from a list
    instead of a grid; mask (npts,) leaves entries 0.  Same keyword extras as
    flowmap_grid_2D (no launch-shape knobs, no step_model)."""
    if method.lower() != "dop853":
        raise NotImplementedError("method=%r: only 'dop853' is implemented on the GPU" % method)
    flow = _check_callable_flow(funcptr)
    if precision not in _PREC:
        raise ValueError("precision must be 'fp64' or 'mixed'")
    D.require_cuda()
    as_torch = D.is_torch(pts)
    pd = D.to_dev(pts)
    if pd.dim() != 2 or pd.shape[1] != 2:
        raise ValueError("pts must have shape (npts, 2): the flows are two-dimensional")
    npts = pd.shape[0]
    md = D.mask_to_dev(mask)
    if md is not None and tuple(md.shape) != (npts,):
        raise ValueError("mask must have shape (npts,)")
    prm = np.ascontiguousarray(
        params.cpu().numpy() if isinstance(params, torch.Tensor) else params, dtype=np.float64)
    out = D.empty((npts, 2))
    status = D.empty((npts,), torch.int32)
    stats = D.empty((npts, 3), torch.int32) if return_stats else None
    opts = _lib.NbcsOpts()
    opts.precision = _PREC[precision]
    opts.max_steps = int(max_steps)
    opts.stats = stats.data_ptr() if stats is not None else None
    L = _lib.load()
    _lib.check(L.nbcs_flowmap_pts(flow.struct, float(t0), float(T), D.ptr(pd), npts,
                                  prm.ctypes.data_as(_lib._vp), len(prm), float(rtol), float(atol),
                                  D.ptr(md), D.ptr(out), D.ptr(status), opts, D.stream_ptr()))
    if not return_status and not as_torch:
        _warn_unfinished("flowmap", status)
    res = [D.finish(out, as_torch)]
    if return_status:
        res.append(D.finish(status, as_torch))
    if return_stats:
        res.append(D.finish(stats, as_torch))
    return res[0] if len(res) == 1 else tuple(res)


def flowmap_n(funcptr, t0, T, pts, params, method="dop853", n=2, rtol=1e-6, atol=1e-8,
              mask=None, *, max_steps=100000, return_status=False):
    """Positions of the points pts (npts, 2) at n times -> ((npts, n, 2), t_eval)
    (integration.py:65-121): t_eval = params[0] * linspace(t0, t0 + T, n), one
    DOP853 run per point with dop853's dense output between the steps (as
    numbalsoda.dop853 fills a t_eval grid), FP64; the returned times are
    params[0] * t_eval, as the reference returns them."""
    if method.lower() != "dop853":
        raise NotImplementedError("method=%r: only 'dop853' is implemented on the GPU" % method)
    flow = _check_callable_flow(funcptr)
    if int(n) < 1:
        raise ValueError("n must be >= 1")
    D.require_cuda()
    as_torch = D.is_torch(pts)
    pd = D.to_dev(pts)
    if pd.dim() != 2 or pd.shape[1] != 2:
        raise ValueError("pts must have shape (npts, 2): the flows are two-dimensional")
    npts = pd.shape[0]
    md = D.mask_to_dev(mask)
    if md is not None and tuple(md.shape) != (npts,):
        raise ValueError("mask must have shape (npts,)")
    prm = np.ascontiguousarray(
        params.cpu().numpy() if isinstance(params, torch.Tensor) else params, dtype=np.float64)
    t_eval = prm[0] * np.linspace(t0, t0 + T, int(n))
    ted = D.to_dev(np.ascontiguousarray(t_eval))
    out = D.empty((npts, int(n), 2))
    status = D.empty((npts,), torch.int32)
    opts = _lib.NbcsOpts()
    opts.precision = _lib.PREC_FP64
    opts.max_steps = int(max_steps)
    L = _lib.load()
    _lib.check(L.nbcs_flowmap_n_pts(flow.struct, D.ptr(pd), npts, D.ptr(ted), int(n),
                                    prm.ctypes.data_as(_lib._vp), len(prm), float(rtol),
                                    float(atol), D.ptr(md), D.ptr(out), D.ptr(status), opts,
                                    D.stream_ptr()))
    if not return_status and not as_torch:
        _warn_unfinished("flowmap_n", status)
    res = (D.finish(out, as_torch), prm[0] * t_eval)
    return res + (D.finish(status, as_torch),) if return_status else res


def flowmap_n_grid_2D(funcptr, t0, T, x, y, params, n=50, method="dop853", rtol=1e-6, atol=1e-8,
                      mask=None, *, max_steps=100000, return_status=False):
    """flowmap_n over the grid x by y -> ((nx, ny, n, 2), t_eval)
    (integration.py:468-534), the points in row-major grid order."""
    D.require_cuda()
    as_torch = D.is_torch(x, y)
    xd, yd = D.to_dev(x), D.to_dev(y)
    nx, ny = xd.numel(), yd.numel()
    X, Y = torch.meshgrid(xd, yd, indexing="ij")
    pts = torch.stack([X.reshape(-1), Y.reshape(-1)], dim=1)
    md = D.mask_to_dev(mask)
    if md is not None:
        if tuple(md.shape) != (nx, ny):
            raise ValueError("mask must have shape (nx, ny)")
        md = md.reshape(-1)
    fm, t_eval, st = flowmap_n(funcptr, t0, T, pts, params, method, n, rtol, atol, md,
                               max_steps=max_steps, return_status=True)
    fm, st = fm.reshape(nx, ny, int(n), 2), st.reshape(nx, ny)
    if not return_status and not as_torch:
        _warn_unfinished("flowmap_n_grid_2D", st)
    res = (D.finish(fm, as_torch), t_eval)
    return res + (D.finish(st, as_torch),) if return_status else res


def flowmap_grid_ND(funcptr, t0, T, IC_flat, ndims, params, method="dop853", rtol=1e-6,
                    atol=1e-8, **kwargs):
    """flowmap_grid_ND (integration.py:186-247): the flow map of the initial
    conditions IC_flat (npts * ndims,) -> (npts, ndims); the flows here are
    two-dimensional, so ndims must be 2 (then it is flowmap of the rows)."""
    if int(ndims) != 2:
        raise ValueError("ndims must be 2: the flows are two-dimensional")
    ic = IC_flat if isinstance(IC_flat, torch.Tensor) else np.asarray(IC_flat, dtype=np.float64)
    if ic.shape[0] % 2:
        raise ValueError("IC_flat length must be a multiple of ndims")
    return flowmap(funcptr, t0, T, ic.reshape(-1, 2), params, method, rtol, atol, **kwargs)


def flowmap_aux_grid_2D(funcptr, t0, T, x, y, params, h=1e-5, eig_main=True, compute_edge=True,
                        method="dop853", rtol=1e-6, atol=1e-8, mask=None, *, precision="fp64",
                        max_steps=100000, return_status=False):
    """Flow map of the auxiliary grid (x_i, y_j) + (+-h, 0), (0, +-h) [, (0, 0)]
    -> (nx, ny, 5, 2) with ``eig_main`` (the last particle is the grid point
    itself), else (nx, ny, 4, 2).

    Same positional signature, defaults and skip rules as the reference
    (integration.py:249-464): with ``compute_edge`` the edge points integrate
    only their centre particle (eig_main) or all four; without it they are
    left 0.  Masked points are left 0.  ``precision="mixed"`` is accepted, but
    C_eig_aux_2D divides differences of trajectories 2h apart by 2h, which
    amplifies the FP32 stage rounding about 1/(2h)-fold: the FP64 default is the
    path for this function.
    """
    if method.lower() != "dop853":
        raise NotImplementedError("method=%r: only 'dop853' is implemented on the GPU" % method)
    flow = _check_callable_flow(funcptr)
    if precision not in _PREC:
        raise ValueError("precision must be 'fp64' or 'mixed'")
    D.require_cuda()
    as_torch = D.is_torch(x, y)
    xd, yd = D.to_dev(x), D.to_dev(y)
    nx, ny = xd.numel(), yd.numel()
    na = 5 if eig_main else 4
    md = D.mask_to_dev(mask)
    if md is not None and tuple(md.shape) != (nx, ny):
        raise ValueError("mask must have shape (nx, ny)")
    prm = np.ascontiguousarray(
        params.cpu().numpy() if isinstance(params, torch.Tensor) else params, dtype=np.float64)
    out = D.empty((nx, ny, na, 2))
    status = D.empty((nx, ny, na), torch.int32)
    opts = _lib.NbcsOpts()
    opts.precision = _PREC[precision]
    opts.max_steps = int(max_steps)
    _lib.check(_lib.load().nbcs_flowmap_aux_grid_2d(
        flow.struct, float(t0), float(T), D.ptr(xd), nx, D.ptr(yd), ny,
        prm.ctypes.data_as(_lib._vp), len(prm), float(h), int(bool(eig_main)),
        int(bool(compute_edge)), float(rtol), float(atol), D.ptr(md), D.ptr(out), D.ptr(status),
        opts, D.stream_ptr()))
    if not return_status and not as_torch:
        _warn_unfinished("flowmap_aux_grid_2D", status)
    if return_status:
        return D.finish(out, as_torch), D.finish(status, as_torch)
    return D.finish(out, as_torch)


def UCGrid(*axes):
    """The interpolation package's uniform Cartesian grid: a tuple of
    (a, b, n) per axis, n an int (what the reference's tests build with
    ``interpolation.splines.UCGrid``)."""
    return tuple((float(a), float(b), int(n)) for a, b, n in axes)


def _grid6(grid, nx, ny):
    (x0, x1, gnx), (y0, y1, gny) = grid
    if (int(gnx), int(gny)) != (nx, ny):
        raise ValueError("grid has %s x %s points, the flow maps %d x %d" % (gnx, gny, nx, ny))
    return np.array([x0, x1, gnx, y0, y1, gny], np.float64)


def flowmap_composition(flowmaps, grid, nT, *, first=0):
    """Composed flow map (nx, ny, 2) of the nT maps ``flowmaps`` (nT, nx, ny, 2)
    (integration.py:609-641): the points start at the first map, pass through
    the next ones by bilinear interpolation on ``grid`` (0 outside it, the
    interpolation package's CONSTANT extrapolation) and end at the last.

    Keyword-only extra: ``first`` reads the stack as a ring buffer, map j of
    the sequence being ``flowmaps[(first + j) % nT]``, so a time series can
    overwrite its oldest map instead of shifting the stack.
    """
    D.require_cuda()
    as_torch = D.is_torch(flowmaps)
    F = D.to_dev(flowmaps)
    nT = int(nT)
    if F.dim() != 4 or F.shape[3] != 2 or F.shape[0] != nT:
        raise ValueError("flowmaps must have shape (nT, nx, ny, 2)")
    nx, ny = int(F.shape[1]), int(F.shape[2])
    g = _grid6(grid, nx, ny)
    out = D.empty((nx, ny, 2))
    _lib.check(_lib.load().nbcs_flowmap_compose(D.ptr(F), nT, int(first) % nT,
                                                g.ctypes.data_as(_lib._vp), D.ptr(out),
                                                D.stream_ptr()))
    return D.finish(out, as_torch)


def flowmap_composition_initial(funcptr, t0, T, h, x, y, grid, params, *, streams=8,
                                **kwargs):
    """integration.py:644-685: the nT = |round(T / h)| flow maps over
    [t0 + k h, t0 + (k + 1) h] and their composition -> (flowmap0, flowmaps, nT).
    ``kwargs`` go to flowmap_grid_2D.  The nT integrations are independent:
    they run on ``streams`` parallel streams (forked from and joined back into
    the current stream), so the tail of one short integration overlaps the
    next; the maps are the same whatever the stream count."""
    D.require_cuda()
    as_torch = D.is_torch(x, y)
    xd, yd = D.to_dev(x), D.to_dev(y)
    nT = abs(round(T / h))
    fms = D.empty((nT, xd.numel(), yd.numel(), 2))
    # every per-map call must stay asynchronous for the streams to overlap:
    # device inputs and a device `out` keep flowmap_grid_2D from reading its
    # status back, and a host mask is copied to the device once, here
    if kwargs.get("mask") is not None:
        kwargs["mask"] = D.mask_to_dev(kwargs["mask"])
    main = torch.cuda.current_stream()
    pool = [torch.cuda.Stream() for _ in range(max(1, min(int(streams), nT)))]
    for s in pool:
        s.wait_stream(main)
    for k in range(nT):
        with torch.cuda.stream(pool[k % len(pool)]):
            flowmap_grid_2D(funcptr, t0, h, xd, yd, params, out=fms[k], **kwargs)
        t0 += h
    for s in pool:
        main.wait_stream(s)
    fm0 = flowmap_composition(fms, grid, nT)
    return D.finish(fm0, as_torch), D.finish(fms, as_torch), nT


def flowmap_composition_step(flowmaps, funcptr, t0, h, nT, x, y, grid, params, **kwargs):
    """integration.py:688-737: drop the oldest map, integrate the newest over
    [t0, t0 + h], compose -> (flowmap_k, flowmaps).  ``flowmaps`` is updated in
    place (numpy array or CUDA tensor), as in the reference."""
    D.require_cuda()
    if isinstance(flowmaps, torch.Tensor) and flowmaps.is_cuda:
        flowmaps[:-1] = flowmaps[1:].clone()
        flowmap_grid_2D(funcptr, t0, h, D.to_dev(x), D.to_dev(y), params, out=flowmaps[-1],
                        **kwargs)
        return flowmap_composition(flowmaps, grid, nT), flowmaps
    flowmaps[:-1] = flowmaps[1:]
    flowmaps[-1] = flowmap_grid_2D(funcptr, t0, h, x, y, params, **kwargs)
    return flowmap_composition(flowmaps, grid, nT), flowmaps
