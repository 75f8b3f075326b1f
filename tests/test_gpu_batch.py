"""Batched persistent integrator: every field of a mixed batch must equal the
single-field path on the same inputs (same solver, same right-hand side, so
bit-identical), also when replayed from a captured CUDA graph."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _flows(nb):
    from numbacs_gb300 import workloads as W
    t, lon, lat = W.geo_grid()
    t, lon, lat = t[::4], lon[::4], lat[::4]
    _, _, _, U, V = W.geo_velocity(0, t=t, lon=lon, lat=lat, nmodes=64)
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, lon, lat, U, V)
    geo = nb.get_flow_2D(grid, Cu, Cv, spherical=1)
    dg, pdg, _ = nb.get_predefined_flow("double_gyre", int_direction=-1.0)
    bj, pbj, dom = nb.get_predefined_flow("bickley_jet")
    return geo, lon, lat, dg, pdg, bj, pbj, dom


def _fields(nb):
    from numbacs_gb300.batch import Field
    geo, lon, lat, dg, pdg, bj, pbj, dom = _flows(nb)
    fs = [
        Field(geo, 180.0, -72.0, np.linspace(lon[0], lon[-1], 67), np.linspace(lat[0], lat[-1], 29),
              np.array([-1.0])),
        Field(dg, 0.0, -10.0, np.linspace(0, 2, 41), np.linspace(0, 1, 21), pdg),
        Field(geo, 170.0, -30.0, np.linspace(lon[0], lon[-1], 13), np.linspace(lat[0], lat[-1], 97),
              np.array([-1.0]), rtol=1e-7, atol=1e-9),
        Field(bj, 0.0, 5.0, np.linspace(0, dom[0][1], 33), np.linspace(-3, 3, 17), pbj, ftle=False),
        Field(dg, 0.0, 8.0, np.linspace(0, 2, 3), np.linspace(0, 1, 3), pdg * np.array([-1, 1, 1, 1, 1, 1])),
    ]
    # a masked spline field (checkerboard, as the reference's tests mask grids)
    m = np.zeros((23, 17), bool)
    m[::2, ::2] = True
    fs.append(Field(geo, 175.0, -40.0, np.linspace(lon[1], lon[-2], 23),
                    np.linspace(lat[1], lat[-2], 17), np.array([-1.0]), mask=m))
    return fs


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("schedule", [3, -1, -2])
def test_batch_equals_single_field(nb, precision, graph, schedule):
    from numbacs_gb300.batch import FTLEBatch
    fields = _fields(nb)
    b = FTLEBatch(fields, precision=precision, blocks_per_sm=schedule, graph=graph)
    b.run()
    b.run()  # a second run (graph replay) recomputes the same values
    torch.cuda.synchronize()
    for f in fields:
        # the batch runs spline fields of the mixed path two lanes per particle
        lp = 2 if (precision == "mixed" and f.flow.kind == 2) else 1
        ref, st = nb.flowmap_grid_2D(f.flow, f.t0, f.T, f.x, f.y, f.params, rtol=f.rtol,
                                     atol=f.atol, mask=f.mask, precision=precision,
                                     return_status=True, lanes_per_particle=lp)
        assert torch.equal(f.status, st)
        assert torch.equal(f.flowmap, ref), (precision, float((f.flowmap - ref).abs().max()))
        if f.ftle is not None:
            ft, ev = nb.ftle_evec_2D(ref, f.T, f.dx, f.dy, mask=f.mask)
            assert torch.equal(f.ftle, ft) and torch.equal(f.evec, ev)


def test_batch_autotune_and_sizes(nb):
    from numbacs_gb300.batch import FTLEBatch
    fields = _fields(nb)
    b = FTLEBatch(fields, precision="mixed", blocks_per_sm=None, graph=True)
    assert b.blocks_per_sm >= 1 or b.blocks_per_sm == -1
    b.run()
    torch.cuda.synchronize()
    assert b.particles == sum(f.x.numel() * f.y.numel() for f in fields)
    def units(f):
        tj = 4 if f.flow.kind == 2 else 8
        return -(-f.x.numel() // 4) * -(-f.y.numel() // tj)
    assert int(b.plan.total_chunks) == sum(units(f) for f in fields)
    def tiles(f):  # one 256-thread block: (32 x 8) particles, (16 x 8) at two lanes each
        ti = 16 if f.flow.kind == 2 else 32
        return -(-f.x.numel() // ti) * -(-f.y.numel() // 8)
    assert int(b.plan.tiles) == sum(tiles(f) for f in fields)
