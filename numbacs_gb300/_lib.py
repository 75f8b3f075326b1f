"""ctypes binding of libnbcs.so (the C ABI declared in include/nbcs.h).

The library is built in-tree by ``numbacs_gb300.build``.  There is no CPU
fallback: if the shared library is missing or no CUDA device is present the
calls raise.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
# NBCS_LIB selects another build of the library (the bounds-checked
# _build_check/libnbcs_check.so, for instance)
LIB_PATH = os.environ.get("NBCS_LIB") or os.path.join(_HERE, "_build", "libnbcs.so")

NBCS_OK = 0
PARTICLE_OK, PARTICLE_MASKED = 0, 1
PARTICLE_MAX_STEPS, PARTICLE_STEP_UNDERFLOW, PARTICLE_NONFINITE = -2, -3, -4
FLOW_DOUBLE_GYRE, FLOW_BICKLEY, FLOW_SPLINE2D = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
MAX_PARAMS = 16


class NbcsFlow(ctypes.Structure):
    """Mirror of ``struct nbcs_flow``."""
    _fields_ = [("kind", ctypes.c_int32), ("spherical", ctypes.c_int32),
                ("extrap", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("r", ctypes.c_double), ("grid", ctypes.c_double * 9),
                ("coef_uv", ctypes.c_void_p), ("coef_uv32", ctypes.c_void_p)]


class NbcsOpts(ctypes.Structure):
    """Mirror of ``struct nbcs_opts``."""
    _fields_ = [("precision", ctypes.c_int32), ("max_steps", ctypes.c_int32),
                ("threads_per_block", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("lanes_per_particle", ctypes.c_int32), ("step_model_mode", ctypes.c_int32),
                ("stats", ctypes.c_void_p), ("step_model", ctypes.c_void_p)]


class NbcsField(ctypes.Structure):
    """Mirror of ``struct nbcs_field``."""
    _fields_ = [("flow", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("np", ctypes.c_int32), ("params", ctypes.c_double * MAX_PARAMS),
                ("t0", ctypes.c_double), ("T", ctypes.c_double), ("rtol", ctypes.c_double),
                ("atol", ctypes.c_double), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("mask", ctypes.c_void_p),
                ("flowmap", ctypes.c_void_p), ("status", ctypes.c_void_p),
                ("ftle", ctypes.c_void_p), ("evec_max", ctypes.c_void_p)]


BATCH_MAX_CLASSES = 8


class NbcsBatchClass(ctypes.Structure):
    """Mirror of ``struct nbcs_batch_class``."""
    _fields_ = [("kind", ctypes.c_int32), ("spherical", ctypes.c_int32),
                ("exact_nodes", ctypes.c_int32), ("lanes", ctypes.c_int32),
                ("field0", ctypes.c_int32), ("nfields", ctypes.c_int32),
                ("tiles", ctypes.c_int64), ("flow", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("r", ctypes.c_double), ("grid", ctypes.c_double * 9),
                ("coef_uv32", ctypes.c_void_p)]


class NbcsBatch(ctypes.Structure):
    """Mirror of ``struct nbcs_batch``."""
    _fields_ = [("scratch", ctypes.c_void_p), ("nflows", ctypes.c_int32),
                ("nfields", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("total_chunks", ctypes.c_int64),
                ("ftle_blocks", ctypes.c_int64), ("tiles", ctypes.c_int64),
                ("nclasses", ctypes.c_int32), ("reserved2", ctypes.c_int32),
                ("classes", NbcsBatchClass * BATCH_MAX_CLASSES)]


# name -> (restype, argtypes)
_vp, _d, _i32, _i64, _sz = ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t
_FP = ctypes.POINTER(NbcsFlow)
SIGNATURES = {
    "nbcs_abi_version": (ctypes.c_int, []),
    "nbcs_last_error": (ctypes.c_char_p, []),
    "nbcs_spline_prefilter_scratch_bytes": (_sz, [_i32, _i32, _i32]),
    "nbcs_spline_prefilter_3d": (ctypes.c_int, [_vp, _i32, _i32, _i32, _vp, _vp, _sz, _vp]),
    "nbcs_spline_pack_uv": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, _vp]),
    "nbcs_eval_rhs": (ctypes.c_int, [_FP, _vp, _i32, _vp, _i64, _vp, _i32, _vp]),
    "nbcs_flowmap_grid_2d": (ctypes.c_int, [_FP, _d, _d, _vp, _i32, _vp, _i32, _vp, _i32, _d, _d,
                                            _vp, _vp, _vp, ctypes.POINTER(NbcsOpts), _vp]),
    "nbcs_flowmap_n_pts": (ctypes.c_int, [_FP, _vp, _i64, _vp, _i32, _vp, _i32, _d, _d, _vp, _vp,
                                          _vp, ctypes.POINTER(NbcsOpts), _vp]),
    "nbcs_flowmap_pts": (ctypes.c_int, [_FP, _d, _d, _vp, _i64, _vp, _i32, _d, _d, _vp, _vp, _vp,
                                        ctypes.POINTER(NbcsOpts), _vp]),
    "nbcs_flowmap_aux_grid_2d": (ctypes.c_int, [_FP, _d, _d, _vp, _i32, _vp, _i32, _vp, _i32, _d,
                                                _i32, _i32, _d, _d, _vp, _vp, _vp,
                                                ctypes.POINTER(NbcsOpts), _vp]),
    "nbcs_flowmap_compose": (ctypes.c_int, [_vp, _i32, _i32, _vp, _vp, _vp]),
    "nbcs_c_eig_aux_2d": (ctypes.c_int, [_vp, _i32, _i32, _i32, _d, _d, _d, _vp, _vp, _vp, _vp]),
    "nbcs_c_tensor_2d": (ctypes.c_int, [_vp, _i32, _i32, _i32, _d, _vp, _vp, _vp]),
    "nbcs_ftle_grid_2d": (ctypes.c_int, [_vp, _i32, _i32, _d, _d, _d, _vp, _vp, _vp]),
    "nbcs_c_eig_2d": (ctypes.c_int, [_vp, _i32, _i32, _d, _d, _vp, _vp, _vp, _vp]),
    "nbcs_ftle_from_eig": (ctypes.c_int, [_vp, _i64, _i64, _d, _vp, _vp]),
    "nbcs_ftle_evec_2d": (ctypes.c_int, [_vp, _i32, _i32, _d, _d, _d, _vp, _vp, _vp, _vp]),
    "nbcs_percentile_scratch_bytes": (_sz, [_i64]),
    "nbcs_percentile": (ctypes.c_int, [_vp, _i64, _d, _vp, _vp, _sz, _vp]),
    "nbcs_ridge_pts_fmin": (ctypes.c_int, [_vp, _vp, _vp, _i32, _vp, _i32, _d, _d, _d, _d, _vp,
                                           _vp, _vp, _vp, _vp, _sz, _vp]),
    "nbcs_ridge_scratch_bytes": (_sz, [_i32, _i32]),
    "nbcs_ridge_pts": (ctypes.c_int, [_vp, _vp, _vp, _i32, _vp, _i32, _d, _d, _vp, _vp, _vp, _vp,
                                      _vp, _sz, _vp]),
    "nbcs_order_ridges": (ctypes.c_int, [_vp, _vp, _vp, _i32, _vp, _i32, _vp, _vp, _d, _d, _i64,
                                         _d, _d, _vp, _i64, _vp, _i64, _vp, _vp]),
    "nbcs_label8_scratch_bytes": (_sz, [_i32, _i32]),
    "nbcs_label8": (ctypes.c_int, [_vp, _i32, _i32, _vp, _vp, _vp, _sz, _vp]),
    "nbcs_mlp_blob_bytes": (_sz, []),
    "nbcs_mlp_param_count": (ctypes.c_int, []),
    "nbcs_mlp_pack": (ctypes.c_int, [_vp, _vp, _vp]),
    "nbcs_mlp_predict": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp]),
    "nbcs_mlp_grad": (ctypes.c_int, [_vp, _vp, _vp, _i64, _vp, _vp, _vp]),
    "nbcs_mlp_adam": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_float, _i32, _vp, _vp]),
    "nbcs_flowmap_log_steps": (ctypes.c_int, [_FP, _d, _d, _vp, _i32, _vp, _i32, _vp, _i32, _d,
                                              _d, ctypes.c_float, ctypes.c_uint32, _vp, _vp, _i64,
                                              _vp, _vp]),
    "nbcs_batch_scratch_bytes": (_sz, [_i32, _i32]),
    "nbcs_batch_prepare": (ctypes.c_int, [_FP, _i32, ctypes.POINTER(NbcsField), _i32, _i32, _vp,
                                          _sz, ctypes.POINTER(NbcsBatch), _vp]),
    "nbcs_batch_run": (ctypes.c_int, [ctypes.POINTER(NbcsBatch), ctypes.POINTER(NbcsOpts), _vp]),
    "nbcs_batch_run_class": (ctypes.c_int, [ctypes.POINTER(NbcsBatch), _i32,
                                            ctypes.POINTER(NbcsOpts), _vp]),
    "nbcs_batch_run_ftle": (ctypes.c_int, [ctypes.POINTER(NbcsBatch), _vp]),
    "nbcs_ridge_noalloc_scratch_bytes": (_sz, []),
    "nbcs_ridge_pts_noalloc": (ctypes.c_int, [_vp, _vp, _vp, _i32, _vp, _i32, _d, _d, _vp, _vp,
                                              _vp, _vp, _vp]),
    "nbcs_launch_count": (ctypes.c_ulonglong, []),
    "nbcs_check_enabled": (ctypes.c_int, []),
    "nbcs_check_bits": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint32), _i32]),
    "nbcs_probe_fma": (ctypes.c_int, [_i32, _i64, _vp, ctypes.POINTER(ctypes.c_double), _vp]),
}

_lib = None


def load(path=LIB_PATH):
    """Load libnbcs.so and declare its signatures (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            "libnbcs.so is not built (%s); run `python -m numbacs_gb300.build`" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc):
    """Raise RuntimeError with the library's message on a non-zero return."""
    if rc != NBCS_OK:
        msg = load().nbcs_last_error()
        raise RuntimeError("libnbcs error %d: %s" % (rc, msg.decode() if msg else ""))
