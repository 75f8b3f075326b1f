"""A small flow-map -> FTLE -> ridges -> labels -> composition pipeline that
tests/test_gpu_checked_build.py runs twice in fresh interpreters: once with
the normal libnbcs.so and once with the bounds-checked build (NBCS_LIB set to
_build_check/libnbcs_check.so).  Writes the results and the library's check
bits to the .npz file named on the command line."""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import numbacs_gb300 as nb  # noqa: E402
from numbacs_gb300 import _lib  # noqa: E402
from numbacs_gb300 import workloads as W  # noqa: E402


def main(out):
    L = _lib.load()
    res = {"check_enabled": np.array(L.nbcs_check_enabled())}
    # double gyre, both integrators, FTLE, ridges, labels
    x, y = np.linspace(0, 2, 101), np.linspace(0, 1, 51)
    dg, p, _ = nb.get_predefined_flow("double_gyre", int_direction=-1.0)
    for prec in ("fp64", "mixed"):
        res["dg_" + prec] = nb.flowmap_grid_2D(dg, 0.0, -10.0, x, y, p, precision=prec)
    f, e = nb.ftle_evec_2D(res["dg_fp64"], -10.0, x[1] - x[0], y[1] - y[0])
    res["ftle"], res["evec"] = f, e
    res["ridge_pts"] = nb.ftle_ridge_pts(f, e, x, y, 0.0, 80)
    ridges = nb.ftle_ridges(f, e, x, y, 0.0, 80)
    res["n_ridges"] = np.array(len(ridges))
    res["ridges_cat"] = np.concatenate(ridges) if ridges else np.zeros((0, 2))
    # spline flow (reduced geophysical field), particles across and beyond the box
    t, lon, lat = W.geo_grid()
    t, lon, lat = t[::4], lon[::4], lat[::4]
    _, _, _, U, V = W.geo_velocity(0, t=t, lon=lon, lat=lat, nmodes=64)
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, lon, lat, U, V)
    xf = np.linspace(lon[0] - 2.0, lon[-1] + 2.0, 45)
    yf = np.linspace(lat[0] - 1.0, lat[-1] + 1.0, 23)
    for mode in ("constant", "linear"):
        fl = nb.get_flow_2D(grid, Cu, Cv, spherical=1, extrap_mode=mode)
        for prec in ("fp64", "mixed"):
            res["geo_%s_%s" % (mode, prec)] = nb.flowmap_grid_2D(
                fl, 180.0, -72.0, xf, yf, np.array([-1.0]), precision=prec)
    # composition of 6 one-hour maps on the double gyre grid
    comp, _, _ = nb.flowmap_composition_initial(dg, 0.0, -6.0, -1.0, x, y,
                                                  nb.UCGrid((0.0, 2.0, 101), (0.0, 1.0, 51)), p)
    res["composition"] = comp
    bits = ctypes.c_uint32(0)
    _lib.check(L.nbcs_check_bits(ctypes.byref(bits), 1))
    res["check_bits"] = np.array(bits.value)
    np.savez(out, **{k: np.asarray(v) for k, v in res.items()})


if __name__ == "__main__":
    main(sys.argv[1])
