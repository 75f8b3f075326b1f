"""Determinism: the same inputs give the same bits on a second run (the
kernels use atomics only where the result does not depend on their order --
the percentile histograms, the ridge counts, the labelling's union-find whose
roots are each component's smallest index, the batch's work counter)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _run(nb, fl, x, y):
    p = np.array([-1.0])
    out = {}
    for prec in ("mixed", "fp64"):
        out[prec] = nb.flowmap_grid_2D(fl, 180.0, -48.0, x, y, p, rtol=1e-7, atol=1e-6,
                                       precision=prec)
    dx, dy = float(x[1] - x[0]), float(y[1] - y[0])
    f, e = nb.ftle_evec_2D(out["mixed"], -48.0, dx, dy)
    out["ftle"], out["evec"] = f, e
    out["pts"] = nb.ftle_ridge_pts(f, e, x, y, 0.0, 85)
    full, mask, _, _ = nb.extraction.ridges._ftle_ridges(f, e, x, y, 0.0, 85)
    out["labels"] = nb.extraction.ridges.label8(mask)[0]
    return out


def test_two_runs_identical(nb):
    from numbacs_gb300 import workloads as W
    from numbacs_gb300.batch import FTLEBatch, Field
    t, lon, lat = W.geo_grid()
    t, lon, lat = t[::2], lon[::2], lat[::2]
    _, _, _, U, V = W.geo_velocity(0, t=t, lon=lon, lat=lat, nmodes=128)
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, lon, lat, U, V)
    fl = nb.get_flow_2D(grid, Cu, Cv, spherical=1)
    x = torch.linspace(lon[0], lon[-1], 301, dtype=torch.float64, device="cuda")
    y = torch.linspace(lat[0], lat[-1], 151, dtype=torch.float64, device="cuda")
    a, b = _run(nb, fl, x, y), _run(nb, fl, x, y)
    for k in a:
        assert torch.equal(a[k], b[k]), k
    fields = [Field(fl, 170.0 + k, -30.0 - 5 * k, x[:: 1 + k % 3], y, np.array([-1.0]),
                    rtol=1e-7, atol=1e-6) for k in range(6)]
    for sched in (-1, -2, 3):
        batch = FTLEBatch(fields, precision="mixed", blocks_per_sm=sched, graph=False)
        batch.run()
        first = [f.flowmap.clone() for f in fields]
        batch.run()
        torch.cuda.synchronize()
        assert all(torch.equal(u, f.flowmap) for u, f in zip(first, fields)), sched
