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
    assert b.blocks_per_sm >= 1 or b.blocks_per_sm in (-1, -2)
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
    # flow classes: spline (spherical), double gyre, Bickley; each a contiguous
    # range of the field table, spline fields at two lanes a particle
    P = b.plan
    cl = [P.classes[k] for k in range(P.nclasses)]
    assert P.nclasses == 3
    assert sorted(c.kind for c in cl) == [0, 1, 2]
    assert sum(c.nfields for c in cl) == len(fields)
    assert sum(int(c.tiles) for c in cl) == int(P.tiles)
    assert sorted((c.field0, c.field0 + c.nfields) for c in cl)[0][0] == 0
    for c in cl:
        assert c.lanes == (2 if c.kind == 2 else 1)
        assert c.flow >= 0  # one flow per class in this batch: the kernel-argument form


def test_batch_extrap_flows_take_the_per_field_schedule(nb):
    from numbacs_gb300.batch import STREAMS, FTLEBatch, Field
    from numbacs_gb300 import workloads as W
    t, lon, lat = W.geo_grid()
    t, lon, lat = t[::4], lon[::4], lat[::4]
    _, _, _, U, V = W.geo_velocity(0, t=t, lon=lon, lat=lat, nmodes=64)
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, lon, lat, U, V)
    geo = nb.get_flow_2D(grid, Cu, Cv, spherical=1, extrap_mode="linear")
    xf = np.linspace(lon[0] - 2, lon[-1] + 2, 37)
    yf = np.linspace(lat[0] - 1, lat[-1] + 1, 19)
    fields = [Field(geo, 100.0, -48.0, xf, yf, np.array([-1.0])),
              Field(geo, 60.0, -72.0, xf[::2], yf, np.array([-1.0]))]
    with pytest.raises(ValueError):
        FTLEBatch(fields, precision="mixed", blocks_per_sm=3)
    for prec in ("mixed", "fp64"):
        b = FTLEBatch(fields, precision=prec, graph=True)
        assert b.blocks_per_sm == STREAMS
        b.run()
        torch.cuda.synchronize()
        for f in fields:
            ref = nb.flowmap_grid_2D(f.flow, f.t0, f.T, f.x, f.y, f.params, rtol=f.rtol,
                                     atol=f.atol, precision=prec, lanes_per_particle=2)
            assert torch.equal(f.flowmap, ref)


def test_batch_c2_fields_against_the_oracle(nb, orc):
    """Fields of the batched time-series workload (full 121 x 217 x 101
    geophysical flow, 256 modes; hourly t0 from 168 h, uneven T, 0.4 deg and
    0.2 deg grids) plus the Bickley jet on 1001 x 301 for 40 days, in one FP64
    batch: the spline fields bit-identical to the oracle (every 4th row), the
    Bickley field as accurate as the oracle against a converged solution
    (40 days of a chaotic jet amplify the last bit of the library sin / cos,
    so the two runs are compared through their error, as in
    test_gpu_configs.py)."""
    from numbacs_gb300.batch import FTLEBatch, Field
    from numbacs_gb300 import workloads as W
    t, lon, lat, U, V = W.geo_velocity(seed=0)
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, lon, lat, U, V)
    geo = nb.get_flow_2D(grid, Cu, Cv, spherical=1)
    og, oCu, oCv = orc.get_interp_arrays_2D(t, lon, lat, U, V)
    ogeo = orc.spline_flow(og, oCu, oCv, spherical=1)
    specs = W.geo_batch_specs()
    picked = [s for s in specs if s[2] == 0.4][:2] + [s for s in specs if s[2] == 0.2][:1]
    fields = []
    for t0, T, sp in picked:
        lx, ly = W.geo_ftle_grid(sp)
        fields.append(Field(geo, t0, T, lx, ly, np.array([-1.0]), rtol=1e-7, atol=1e-9))
    bj, pbj, _ = nb.get_predefined_flow("bickley_jet")
    bx, by = W.bickley_batch_grid()
    fields.append(Field(bj, W.BICKLEY_T0, W.BICKLEY_T, bx, by, pbj))
    b = FTLEBatch(fields, precision="fp64", graph=True)
    b.run()
    torch.cuda.synchronize()
    for (t0, T, sp), f in zip(picked, fields):
        lx, ly = W.geo_ftle_grid(sp)
        ofm, ost, _ = orc.flowmap_grid_2D(ogeo, t0, T, lx[::4], ly, np.array([-1.0]), rtol=1e-7,
                                         atol=1e-9, return_status=True)
        assert np.array_equal(f.flowmap[::4].cpu().numpy(), ofm), (t0, T, sp)
        assert np.array_equal(f.status[::4].cpu().numpy(), ost)
    fb = fields[-1]
    rows = slice(None, None, 25)
    g = fb.flowmap[rows].cpu().numpy()
    o = orc.flowmap_grid_2D(orc.bickley_jet(), 0.0, 40.0, bx[rows], by, pbj)
    tr = orc.flowmap_grid_2D(orc.bickley_jet(), 0.0, 40.0, bx[rows], by, pbj, rtol=1e-11,
                             atol=1e-13)
    eg, eo = np.abs(g - tr).max(-1), np.abs(o - tr).max(-1)
    assert abs(eg.mean() - eo.mean()) <= 0.05 * eo.mean()
    assert abs(np.quantile(eg, 0.99) - np.quantile(eo, 0.99)) <= 0.05 * np.quantile(eo, 0.99)
