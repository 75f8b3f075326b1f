"""Velocity fields: the drop-in for numbacs.flows on the flow-map path.

Reference: src/numbacs/flows.py.  In the reference a flow is a numba @cfunc
with numbalsoda's ``lsoda_sig`` whose integer address (``funcptr``) is passed
to ``flowmap_grid_2D``.  A host function pointer cannot run on the GPU, so the
factories here return a :class:`Flow` handle in its place: it names a
right-hand side compiled into libnbcs (double gyre, Bickley jet, tricubic
spline) and owns the device copies of any spline coefficients.  Everything
else -- names, argument order, defaults, returned tuples -- follows the
reference.
"""
import math

import numpy as np
import torch

from . import _device as D
from . import _lib


class Flow:
    """Replacement for the ``funcptr`` of a reference flow.

    Attributes mirror ``struct nbcs_flow`` in include/nbcs.h.  Spline flows keep
    their FP64 and FP32 interleaved (u, v) coefficient tensors alive for as long
    as the handle lives.
    """

    def __init__(self, kind, name, spherical=0, extrap=0, r=6371.0, grid=None,
                 coef_uv=None, coef_uv32=None):
        self.kind = kind
        self.name = name
        self.spherical = int(spherical)
        self.extrap = int(extrap)
        self.r = float(r)
        self.grid = grid
        self.coef_uv = coef_uv
        self.coef_uv32 = coef_uv32
        s = _lib.NbcsFlow()
        s.kind = kind
        s.spherical = self.spherical
        s.extrap = self.extrap
        s.r = self.r
        if grid is not None:
            flat = [float(v) for g in grid for v in g]
            for k in range(9):
                s.grid[k] = flat[k]
        s.coef_uv = coef_uv.data_ptr() if coef_uv is not None else None
        s.coef_uv32 = coef_uv32.data_ptr() if coef_uv32 is not None else None
        self._struct = s

    @property
    def struct(self):
        return self._struct

    def __int__(self):
        raise TypeError("numbacs_gb300 flows are device flow handles, not C function pointers")

    def __repr__(self):
        return "Flow(%s)" % self.name


def _check_callable_flow(funcptr):
    if isinstance(funcptr, Flow):
        return funcptr
    raise TypeError(
        "funcptr must be a numbacs_gb300 Flow (from get_predefined_flow or get_flow_2D); "
        "user-defined numba cfuncs cannot run on the GPU")


def get_predefined_flow(flow_str, int_direction=1.0, return_default_params=True,
                        return_domain=True, parameter_description=False):
    """Drop-in for flows.py:1104-1295 (double gyre and Bickley jet).

    Returns the same tuple shapes as the reference, with a :class:`Flow` in
    place of the C callback address.  As in the reference, the Bickley jet's
    default parameters carry ``int_direction = 1.0`` whatever the argument
    (flows.py:1219).
    """
    if flow_str == "double_gyre":
        flow = Flow(_lib.FLOW_DOUBLE_GYRE, "double_gyre")
        A, eps, alpha, omega, psi = 0.1, 0.25, 0.0, 0.2 * math.pi, 0.0
        default_params = np.array([int_direction, A, eps, alpha, omega, psi])
        domain = ((0.0, 2.0), (0.0, 1.0))
        p_str = ("p[0] = int_direction, p[1] = A, p[2] = eps, p[3] = alpha, "
                 + "p[4] = omega, p[5] = psi")
    elif flow_str == "bickley_jet":
        flow = Flow(_lib.FLOW_BICKLEY, "bickley_jet")
        int_direction = 1.0
        r_e = 6371.0e-3
        U0 = 86400 * 62.66e-6
        L = 1770.0e-3
        A1, A2, A3 = 0.0075, 0.15, 0.3
        k1, k2, k3 = 2.0 / r_e, 4.0 / r_e, 6.0 / r_e
        c2 = 0.205 * U0
        c3 = 0.461 * U0
        c1 = c3 + (math.sqrt(5) - 1) * (c2 - c3)
        default_params = np.array([int_direction, U0, L, A1, A2, A3, k1, k2, k3, c1, c2, c3])
        domain = ((0.0, r_e * math.pi), (-3.0, 3.0))
        p_str = ("p[0] = int_direction, p[1] = U0, p[2] = L, p[3] = A1, p[4] = A2, "
                 + "p[5] = A3, p[6] = k1, p[7] = k2, p[8] = k3, p[9] = c1, p[10] = c2, "
                 + "p[11] = c3, units: time - days, length - Mm")
    elif flow_str == "abc":
        raise NotImplementedError("the 3-D ABC flow is not on the 2-D flow-map path")
    else:
        raise ValueError("unknown predefined flow %r" % (flow_str,))
    out = [flow]
    if return_default_params:
        out.append(default_params)
    if return_domain:
        out.append(domain)
    if parameter_description:
        out.append(p_str)
    return out[0] if len(out) == 1 else tuple(out)


def _prefilter(f):
    """natural-BC cubic prefilter of a (nt, nx, ny) device tensor on the GPU"""
    L = _lib.load()
    nt, nx, ny = f.shape
    coef = D.empty((nt + 2, nx + 2, ny + 2))
    nbytes = L.nbcs_spline_prefilter_scratch_bytes(nt, nx, ny)
    scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=f.device)
    _lib.check(L.nbcs_spline_prefilter_3d(D.ptr(f), nt, nx, ny, D.ptr(coef), D.ptr(scratch),
                                          nbytes, D.stream_ptr()))
    return coef


def get_interp_arrays_2D(tvals, xvals, yvals, U, V):
    """Drop-in for flows.py:9-46: grid tuple and cubic spline coefficients.

    The coefficients (nt+2, nx+2, ny+2) are computed on the GPU; numpy in gives
    numpy out, torch in gives CUDA tensors out.
    """
    D.require_cuda()
    as_torch = D.is_torch(U, V)
    Ud, Vd = D.to_dev(U), D.to_dev(V)
    if Ud.dim() != 3 or Vd.shape != Ud.shape:
        raise ValueError("U and V must have the same (nt, nx, ny) shape")
    nt, nx, ny = Ud.shape
    tv = np.asarray(tvals.cpu() if isinstance(tvals, torch.Tensor) else tvals, dtype=np.float64)
    xv = np.asarray(xvals.cpu() if isinstance(xvals, torch.Tensor) else xvals, dtype=np.float64)
    yv = np.asarray(yvals.cpu() if isinstance(yvals, torch.Tensor) else yvals, dtype=np.float64)
    grid_vel = ((float(tv[0]), float(tv[-1]), nt), (float(xv[0]), float(xv[-1]), nx),
                (float(yv[0]), float(yv[-1]), ny))
    Cu = _prefilter(Ud)
    Cv = _prefilter(Vd)
    return grid_vel, D.finish(Cu, as_torch), D.finish(Cv, as_torch)


# extrap_mode -> nbcs_flow.extrap (the interpolation package's option names)
_EXTRAP = {"constant": 0, "nearest": 1, "linear": 2}


def get_flow_2D(grid_vel, C_eval_u, C_eval_v, spherical=0, extrap_mode="constant", r=6371.0):
    """Drop-in for flows.py:121-258: a tricubic-spline flow handle.

    The reference closes a numba cfunc over the coefficient arrays; here the
    coefficients are packed once into interleaved (u, v) FP64 and FP32 device
    arrays owned by the returned :class:`Flow`.

    ``extrap_mode`` decides the velocity at a point (t, x, y) outside the grid
    box, as the reference passes it on to the interpolation package's
    ``eval_spline``:

    * ``"constant"``: zero velocity, so a particle that leaves the box stops;
    * ``"nearest"``: the velocity at the nearest point of the box (each
      coordinate clamped into its axis' range);
    * ``"linear"``: that value continued to first order, plus the spline's
      derivative along each clamped axis times the distance beyond the box.

    "constant" is pinned by the reference's composition fixtures; no fixture
    pins "nearest" or "linear", whose definition here is the CPU oracle's
    (the GPU integrators match it bit for bit in FP64).  The batched kernels
    (:class:`batch.FTLEBatch`) run such flows through the per-field schedule.
    """
    D.require_cuda()
    if extrap_mode not in _EXTRAP:
        raise ValueError("extrap_mode must be one of %s, got %r" % (sorted(_EXTRAP), extrap_mode))
    if spherical not in (0, 1, 2):
        raise ValueError("spherical must be 0, 1 or 2")
    cu, cv = D.to_dev(C_eval_u), D.to_dev(C_eval_v)
    (t0, t1, nt), (x0, x1, nx), (y0, y1, ny) = grid_vel
    if tuple(cu.shape) != (nt + 2, nx + 2, ny + 2) or cv.shape != cu.shape:
        raise ValueError("coefficient arrays must have shape (nt+2, nx+2, ny+2)")
    n = cu.numel()
    uv = D.empty((n, 2))
    uv32 = D.empty((n, 8), torch.float32)  # quad layout (u_j, v_j), j = k .. k+3
    L = _lib.load()
    _lib.check(L.nbcs_spline_pack_uv(D.ptr(cu), D.ptr(cv), n, D.ptr(uv), D.ptr(uv32),
                                     D.stream_ptr()))
    grid = ((float(t0), float(t1), int(nt)), (float(x0), float(x1), int(nx)),
            (float(y0), float(y1), int(ny)))
    return Flow(_lib.FLOW_SPLINE2D, "spline2d", spherical, _EXTRAP[extrap_mode], r, grid, uv, uv32)


def eval_rhs(flow, t, pts, params, precision="fp64"):
    """Evaluate the flow's right-hand side at rows (t, x, y) -> (n, 2) velocities.

    ``t`` may be a scalar or an array matching ``pts`` rows.  This is the
    device counterpart of calling the reference @cfunc ``funcptr(t, y, dy, p)``.
    """
    D.require_cuda()
    flow = _check_callable_flow(flow)
    as_torch = D.is_torch(pts)
    P = D.to_dev(pts)
    if P.dim() == 1:
        P = P.reshape(1, -1)
    n = P.shape[0]
    if P.shape[1] == 2:
        tt = D.to_dev(t) if hasattr(t, "__len__") else torch.full((n,), float(t), dtype=torch.float64,
                                                                     device=P.device)
        P = torch.cat([tt.reshape(n, 1), P], dim=1).contiguous()
    prm = np.ascontiguousarray(params, dtype=np.float64)
    out = D.empty((n, 2))
    L = _lib.load()
    prec = _lib.PREC_MIXED if precision == "mixed" else _lib.PREC_FP64
    _lib.check(L.nbcs_eval_rhs(flow.struct, prm.ctypes.data_as(_lib._vp), len(prm), D.ptr(P), n,
                               D.ptr(out), prec, D.stream_ptr()))
    return D.finish(out, as_torch)
