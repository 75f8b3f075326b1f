"""CUDA flow-map integration against the golden vectors and the CPU oracle."""
import numpy as np
import pytest
import torch

from conftest import apply_mask

pytestmark = pytest.mark.gpu


def test_rhs_golden(nb, golden, orc):
    from test_oracle_golden import _spline_case
    t, xs, u, v, pts = _spline_case()
    fl, p, _ = nb.get_predefined_flow("double_gyre")
    dg = nb.flows.eval_rhs(fl, pts[:, 0], pts[:, 1:], p)
    assert np.allclose(dg, golden["dg_vel"])
    ref = np.array([orc.rhs(orc.double_gyre(), q[0], q[1:], p) for q in pts])
    np.testing.assert_allclose(dg, ref, rtol=1e-15, atol=1e-16)
    fb, pb, _ = nb.get_predefined_flow("bickley_jet")
    bj = nb.flows.eval_rhs(fb, pts[:, 0], pts[:, 1:], pb)
    assert np.allclose(bj, golden["bickley_vel"])
    np.testing.assert_allclose(
        bj, np.array([orc.rhs(orc.bickley_jet(), q[0], q[1:], pb) for q in pts]), rtol=1e-14,
        atol=1e-15)
    # mixed-precision right-hand sides agree to FP32 accuracy
    dg32 = nb.flows.eval_rhs(fl, pts[:, 0], pts[:, 1:], p, precision="mixed")
    np.testing.assert_allclose(dg32, dg, rtol=0, atol=2e-6)
    bj32 = nb.flows.eval_rhs(fb, pts[:, 0], pts[:, 1:], pb, precision="mixed")
    np.testing.assert_allclose(bj32, bj, rtol=0, atol=2e-5)


def test_spline_prefilter_golden(nb, golden, orc):
    from test_oracle_golden import _spline_case
    t, xs, u, v, pts = _spline_case()
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, xs, xs, u, v)
    assert np.allclose(Cu, golden["spline_Cu"]) and np.allclose(Cv, golden["spline_Cv"])
    fl = nb.get_flow_2D(grid, Cu, Cv)
    vel = nb.flows.eval_rhs(fl, pts[:, 0], pts[:, 1:], np.array([1.0]))
    assert np.allclose(vel, golden["spline_vel"])
    # bit-identical to the oracle's prefilter on a ragged random block
    rng = np.random.default_rng(3)
    f = rng.standard_normal((7, 13, 5))
    c = nb.flows._prefilter(torch.from_numpy(f).cuda()).cpu().numpy()
    assert np.array_equal(c, orc.prefilter_3d(f))
    # degenerate axes (n = 2) and a long axis
    for shape in [(2, 2, 2), (3, 2, 300), (2, 1000, 3)]:
        f = rng.standard_normal(shape)
        c = nb.flows._prefilter(torch.from_numpy(f).cuda()).cpu().numpy()
        assert np.array_equal(c, orc.prefilter_3d(f)), shape


def test_flowmap_golden(nb, golden, coords_dg, mask_dg):
    x, y = coords_dg
    fl, p, _ = nb.get_predefined_flow("double_gyre")
    fm = nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p)
    assert np.allclose(fm.astype(np.float32), golden["fm"])
    fmm = nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p, mask=mask_dg)
    assert np.allclose(fmm.astype(np.float32), apply_mask(golden["fm"], mask_dg))


def _compare(nb_out, orc_out, nb_stats, orc_stats, extent, name):
    """Parity: step sequences identical for (almost) all particles; positions
    within 1e-6 of the domain extent everywhere.  The FP64 arithmetic is the
    same operation for operation; only the last bit of the library sin / cos /
    cosh / tanh of the analytic flows differs between CUDA and the host libm,
    which chaotic trajectories amplify, so rounding-level agreement is asked
    of the median particle."""
    same_steps = np.all(nb_stats == orc_stats, axis=-1)
    err = np.abs(nb_out - orc_out).max(axis=-1)
    frac_same = same_steps.mean()
    assert frac_same >= 0.999, (name, frac_same)
    assert err.max() <= 1e-6 * extent, (name, err.max())
    assert np.median(err) <= 1e-12 * extent, (name, np.median(err))


def _exact(nb_out, orc_out, nb_stats, orc_stats, name):
    """Bit parity: the spline right-hand sides use only + - * / sqrt and the
    shared deterministic cos, so GPU and oracle agree to the last bit."""
    assert np.array_equal(nb_stats, orc_stats), name
    assert np.array_equal(nb_out, orc_out), (name, np.abs(nb_out - orc_out).max())


def test_flowmap_parity_double_gyre(nb, orc):
    x, y = np.linspace(0, 2, 101), np.linspace(0, 1, 51)
    fl, p, _ = nb.get_predefined_flow("double_gyre", int_direction=-1.0)
    fm, st, stats = nb.flowmap_grid_2D(fl, 0.0, -10.0, x, y, p, return_status=True,
                                       return_stats=True)
    ofm, ost, ostats = orc.flowmap_grid_2D(orc.double_gyre(), 0.0, -10.0, x, y, p,
                                           return_status=True)
    assert (st == 0).all() and (ost == 0).all()
    _compare(fm, ofm, stats, ostats, 2.0, "dg")


def test_flowmap_parity_bickley(nb, orc):
    fl, p, dom = nb.get_predefined_flow("bickley_jet")
    x = np.linspace(dom[0][0], dom[0][1], 61)
    y = np.linspace(dom[1][0], dom[1][1], 31)
    fm, stats = nb.flowmap_grid_2D(fl, 0.0, 6.0, x, y, p, return_stats=True)
    ofm, _, ostats = orc.flowmap_grid_2D(orc.bickley_jet(), 0.0, 6.0, x, y, p, return_status=True)
    _compare(fm, ofm, stats, ostats, dom[0][1] - dom[0][0], "bickley")


def _small_geo(orc, seed=0):
    from numbacs_gb300 import workloads as W
    t, lon, lat = W.geo_grid()
    # a reduced sample grid keeps the oracle run to seconds
    t, lon, lat = t[::4], lon[::4], lat[::4]
    _, _, _, U, V = W.geo_velocity(seed, t=t, lon=lon, lat=lat, nmodes=64)
    return t, lon, lat, U, V


@pytest.mark.parametrize("spherical", [0, 1, 2])
def test_flowmap_parity_spline(nb, orc, spherical):
    t, lon, lat, U, V = _small_geo(orc)
    if spherical == 2:
        lon = lon + 180.0  # lon in [80, 215] for the [0, 360) convention
    if spherical == 0:
        U, V = U / 111.0, V / 111.0  # planar: velocities in degrees per hour
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, lon, lat, U, V)
    og, oCu, oCv = orc.get_interp_arrays_2D(t, lon, lat, U, V)
    assert np.array_equal(Cu, oCu) and np.array_equal(Cv, oCv)
    fl = nb.get_flow_2D(grid, Cu, Cv, spherical=spherical)
    of = orc.spline_flow(og, oCu, oCv, spherical=spherical)
    xf = np.linspace(lon[0], lon[-1], 41)
    yf = np.linspace(lat[0], lat[-1], 21)
    p = np.array([-1.0])
    fm, stats = nb.flowmap_grid_2D(fl, 180.0, -72.0, xf, yf, p, return_stats=True)
    ofm, _, ostats = orc.flowmap_grid_2D(of, 180.0, -72.0, xf, yf, p, return_status=True)
    _exact(fm, ofm, stats, ostats, "spline%d" % spherical)


@pytest.mark.parametrize("extrap", ["nearest", "linear"])
@pytest.mark.parametrize("spherical", [0, 1])
def test_flowmap_parity_spline_extrap(nb, orc, extrap, spherical):
    """extrap_mode "nearest" / "linear": particles seeded across and beyond
    the grid box, integrated back past the first time sample, so every mode of
    extrapolation (t, x, y, below and above) is taken.  FP64 bit-identical to
    the oracle; the mixed path's velocities outside the box within FP32
    accuracy of the FP64 path's."""
    t, lon, lat, U, V = _small_geo(orc)
    if spherical == 0:
        U, V = U / 111.0, V / 111.0
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, lon, lat, U, V)
    og, oCu, oCv = orc.get_interp_arrays_2D(t, lon, lat, U, V)
    fl = nb.get_flow_2D(grid, Cu, Cv, spherical=spherical, extrap_mode=extrap)
    of = orc.spline_flow(og, oCu, oCv, spherical=spherical, extrap={"nearest": 1, "linear": 2}[extrap])
    xf = np.linspace(lon[0] - 3.0, lon[-1] + 3.0, 41)
    yf = np.linspace(lat[0] - 2.0, lat[-1] + 2.0, 21)
    p = np.array([-1.0])
    fm, st, stats = nb.flowmap_grid_2D(fl, 30.0, -72.0, xf, yf, p, return_status=True,
                                       return_stats=True)
    ofm, ost, ostats = orc.flowmap_grid_2D(of, 30.0, -72.0, xf, yf, p, return_status=True)
    assert np.array_equal(st, ost)
    _exact(fm, ofm, stats, ostats, "spline%d %s" % (spherical, extrap))
    # the extrapolated velocities differ from "constant" (zero) outside the box;
    # rows are (model time, x, y), the solver time is model time / params[0]
    fl0 = nb.get_flow_2D(grid, Cu, Cv, spherical=spherical)
    out_pts = np.array([[t[0] - 5.0, lon[5], lat[3]], [t[4], lon[-1] + 1.5, lat[2]],
                        [t[3], lon[2], lat[0] - 1.0], [t[-1] + 2.0, lon[-1] + 0.7, lat[-1] + 0.4]])
    ts = out_pts[:, 0] / p[0]
    v64 = nb.flows.eval_rhs(fl, ts, out_pts[:, 1:], p)
    assert np.all(np.abs(v64).max(axis=1) > 0)
    assert np.all(nb.flows.eval_rhs(fl0, ts, out_pts[:, 1:], p) == 0.0)
    ref = np.array([orc.rhs(of, tq, q[1:], p) for tq, q in zip(ts, out_pts)])
    assert np.array_equal(v64, ref)
    v32 = nb.flows.eval_rhs(fl, ts, out_pts[:, 1:], p, precision="mixed")
    np.testing.assert_allclose(v32, v64, rtol=2e-5, atol=2e-5 * np.abs(v64).max())
    # mixed flow maps over 12 h (before chaotic growth) within 1e-4 of the box size
    fm32 = nb.flowmap_grid_2D(fl, 30.0, -12.0, xf, yf, p, rtol=1e-8, atol=1e-10, precision="mixed")
    fm64 = nb.flowmap_grid_2D(fl, 30.0, -12.0, xf, yf, p, rtol=1e-8, atol=1e-10)
    assert np.abs(fm32 - fm64).max() <= 1e-4 * (lon[-1] - lon[0])


def test_flowmap_torch_in_torch_out(nb, coords_dg):
    x, y = coords_dg
    fl, p, _ = nb.get_predefined_flow("double_gyre")
    xt, yt = torch.tensor(x, device="cuda"), torch.tensor(y, device="cuda")
    out = torch.empty((len(x), len(y), 2), dtype=torch.float64, device="cuda")
    fm = nb.flowmap_grid_2D(fl, 0.0, 8.0, xt, yt, p, out=out)
    assert fm is out and fm.is_cuda
    assert np.array_equal(fm.cpu().numpy(), nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p))


def test_flowmap_deterministic(nb):
    x, y = np.linspace(0, 2, 64), np.linspace(0, 1, 32)
    fl, p, _ = nb.get_predefined_flow("double_gyre")
    for prec in ("fp64", "mixed"):
        a = nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p, precision=prec)
        b = nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p, precision=prec)
        assert np.array_equal(a, b), prec


def _err_stats(fm, truth):
    e = np.abs(fm - truth).max(axis=-1).ravel()
    return {"mean": e.mean(), "median": np.median(e), "q99": np.quantile(e, 0.99), "max": e.max()}


@pytest.mark.parametrize("rtol", [1e-6, 1e-7])
def test_mixed_precision_vs_converged_truth(nb, orc, rtol):
    """Double gyre, mixed path against an FP64 solution converged to rtol
    1e-12.  Its FP32 right-hand side carries ~1e-7 relative error, which the
    gyre's stretching amplifies to a floor of ~1e-6 in the end points: the
    median error must stay within 1e-6 of the domain extent (2), the 99th
    percentile within 1e-5 of it, and at rtol 1e-6, where truncation error
    dominates, within 3x of the plain FP64 path's."""
    x, y = np.linspace(0, 2, 81), np.linspace(0, 1, 41)
    fl, p, _ = nb.get_predefined_flow("double_gyre", int_direction=-1.0)
    truth = orc.flowmap_grid_2D(orc.double_gyre(), 0.0, -10.0, x, y, p, rtol=1e-12, atol=1e-14)
    plain, sp = nb.flowmap_grid_2D(fl, 0.0, -10.0, x, y, p, rtol=rtol, atol=1e-2 * rtol,
                                   return_status=True)
    mixed, sm = nb.flowmap_grid_2D(fl, 0.0, -10.0, x, y, p, rtol=rtol, atol=1e-2 * rtol,
                                   precision="mixed", return_status=True)
    assert (sp == 0).all() and (sm == 0).all()
    ep, em = _err_stats(plain, truth), _err_stats(mixed, truth)
    assert em["median"] <= 2e-6, (em, ep)
    assert em["q99"] <= 2e-5, (em, ep)
    if rtol >= 1e-6:
        assert em["q99"] <= 3 * ep["q99"], (em, ep)


def test_mixed_precision_geo_vs_fp64(nb, orc):
    # spline flow, spherical: mixed vs plain at the same rtol, both vs a tight FP64 solve
    t, lon, lat, U, V = _small_geo(orc)
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, lon, lat, U, V)
    fl = nb.get_flow_2D(grid, Cu, Cv, spherical=1)
    xf = np.linspace(lon[0], lon[-1], 81)
    yf = np.linspace(lat[0], lat[-1], 41)
    p = np.array([-1.0])
    truth = nb.flowmap_grid_2D(fl, 180.0, -72.0, xf, yf, p, rtol=1e-12, atol=1e-14)
    for rtol in (1e-6, 1e-7):
        plain = nb.flowmap_grid_2D(fl, 180.0, -72.0, xf, yf, p, rtol=rtol, atol=1e-2 * rtol)
        mixed, st = nb.flowmap_grid_2D(fl, 180.0, -72.0, xf, yf, p, rtol=rtol, atol=1e-2 * rtol,
                                       precision="mixed", return_status=True)
        assert (st == 0).all()
        ep, em = _err_stats(plain, truth), _err_stats(mixed, truth)
        assert em["median"] <= 3 * ep["median"] + 1e-9, (rtol, em, ep)
        assert em["q99"] <= 3 * ep["q99"] + 1e-8, (rtol, em, ep)
    # a particle at (1e-12, 4e-15): sk ~ atol, so HINIT proposes h ~ 1e-12; the
    # compensated time pair must still advance (no spurious step underflow)
    one = np.array([1.4210854715202004e-12]), np.array([4.440892098500626e-15])
    m1, s1 = nb.flowmap_grid_2D(fl, 180.0, -72.0, *one, p, precision="mixed", return_status=True)
    d1, _ = nb.flowmap_grid_2D(fl, 180.0, -72.0, *one, p, return_status=True)
    assert s1.item() == 0 and np.abs(m1 - d1).max() < 1e-3


def test_status_codes(nb):
    x, y = np.linspace(0.1, 1.9, 8), np.linspace(0.1, 0.9, 4)
    fl, p, _ = nb.get_predefined_flow("double_gyre")
    # step limit injected from the host
    fm, st = nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p, max_steps=1, return_status=True)
    assert (st == -2).all()
    with pytest.warns(RuntimeWarning):
        nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p, max_steps=1)
    # NaN parameters -> NaN error estimate -> NONFINITE (no hang, no fault)
    pn = p.copy()
    pn[1] = np.nan
    for prec in ("fp64", "mixed"):
        _, st = nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, pn, return_status=True, precision=prec)
        assert (st == -4).all(), prec
    # T = 0 returns the initial grid
    fm0 = nb.flowmap_grid_2D(fl, 0.0, 0.0, x, y, p)
    X, Y = np.meshgrid(x, y, indexing="ij")
    assert np.array_equal(fm0, np.stack([X, Y], -1))


@pytest.mark.parametrize("shape", [(0, 5), (1, 7), (9, 1), (1, 1)])
def test_flowmap_degenerate_grids(nb, orc, shape):
    """Empty, single-row, single-column and single-point grids: the shapes the
    reference's prange loop returns; FP64 flow maps within the double-gyre
    parity bound of the oracle's (the RHS calls CUDA's sin / cos), the FTLE
    of the same flow map bit-identical (all zero: no interior points)."""
    nx, ny = shape
    x, y = np.linspace(0.1, 1.9, nx), np.linspace(0.1, 0.9, ny)
    fl, p, _ = nb.get_predefined_flow("double_gyre")
    for prec in ("fp64", "mixed"):
        fm, st = nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p, precision=prec, return_status=True)
        assert fm.shape == (nx, ny, 2) and st.shape == (nx, ny)
        assert (st == 0).all()
    fm = nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p)
    ofm = orc.flowmap_grid_2D(orc.double_gyre(), 0.0, 8.0, x, y, p)
    assert fm.shape == ofm.shape and (fm.size == 0 or np.abs(fm - ofm).max() <= 2e-6)
    f = nb.ftle_grid_2D(fm, 8.0, 0.1, 0.1)
    assert f.shape == (nx, ny) and np.array_equal(f, orc.ftle_grid_2D(fm, 8.0, 0.1, 0.1))


def test_flowmap_all_masked(nb):
    x, y = np.linspace(0.1, 1.9, 12), np.linspace(0.1, 0.9, 6)
    fl, p, _ = nb.get_predefined_flow("double_gyre")
    mask = np.ones((12, 6), bool)
    for prec in ("fp64", "mixed"):
        fm, st = nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p, mask=mask, precision=prec,
                                    return_status=True)
        assert np.array_equal(fm, np.zeros((12, 6, 2)))
        assert (st == st.flat[0]).all() and st.flat[0] != 0


def test_mixed_precision_non_dyadic_grid(nb):
    """A spline grid whose nodes are not floats (0.9 deg and 50/83 deg
    spacings): the mixed path takes the compensated cell search and stays as
    close to a tight FP64 solve as the FP64 path at the same rtol."""
    from numbacs_gb300 import workloads as W
    t = np.arange(41) * 3.0
    lon, lat = np.linspace(-100.0, 35.0, 151), np.linspace(-5.0, 45.0, 84)
    _, _, _, U, V = W.geo_velocity(0, t=t, lon=lon, lat=lat, nmodes=64)
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, lon, lat, U, V)
    fl = nb.get_flow_2D(grid, Cu, Cv, spherical=1)
    xf, yf = np.linspace(-90.0, 25.0, 61), np.linspace(0.0, 40.0, 31)
    p = np.array([-1.0])
    truth = nb.flowmap_grid_2D(fl, 100.0, -48.0, xf, yf, p, rtol=1e-12, atol=1e-14)
    plain = nb.flowmap_grid_2D(fl, 100.0, -48.0, xf, yf, p, rtol=1e-7, atol=1e-9)
    mixed, st = nb.flowmap_grid_2D(fl, 100.0, -48.0, xf, yf, p, rtol=1e-7, atol=1e-9,
                                   precision="mixed", return_status=True)
    assert (st == 0).all()
    ep, em = _err_stats(plain, truth), _err_stats(mixed, truth)
    assert em["median"] <= 3 * ep["median"] + 1e-9, (em, ep)
    assert em["q99"] <= 3 * ep["q99"] + 1e-8, (em, ep)


def test_status_nan_spline_coefficients(nb, orc):
    """Host-injected fault: one NaN velocity sample.  The natural-BC prefilter
    couples whole lines, so every coefficient turns NaN; particles that start
    inside the grid box return NONFINITE (-4), those outside (zero velocity)
    return OK -- on both paths, as the oracle does, with no hang or fault.
    The batched kernels report the same codes, and MAX_STEPS (-2) under a
    one-step limit (as the oracle does: even a particle at rest needs many
    growing steps to cover 18 h)."""
    from numbacs_gb300.batch import FTLEBatch, Field
    tv, lon, lat = np.arange(9) * 3.0, np.linspace(-20.0, 20.0, 11), np.linspace(0.0, 30.0, 9)
    T3, X3, Y3 = np.meshgrid(tv, lon, lat, indexing="ij")
    U = 30.0 * np.sin(0.15 * X3 + 0.05 * T3) * np.cos(0.1 * Y3)
    V = 20.0 * np.cos(0.12 * X3) * np.sin(0.2 * Y3 - 0.03 * T3)
    U[4, 5, 4] = np.nan
    grid, Cu, Cv = nb.get_interp_arrays_2D(tv, lon, lat, U, V)
    fl = nb.get_flow_2D(grid, Cu, Cv, spherical=1)
    og, oCu, oCv = orc.get_interp_arrays_2D(tv, lon, lat, U, V)
    ofl = orc.spline_flow(og, oCu, oCv, spherical=1)
    xs, ys, p = np.linspace(-30.0, 30.0, 13), np.linspace(5.0, 25.0, 5), np.array([-1.0])
    inside = np.abs(xs)[:, None] <= 20.0 + 0 * ys[None, :]
    _, ost, _ = orc.flowmap_grid_2D(ofl, 24.0, -18.0, xs, ys, p, return_status=True)
    assert np.array_equal(ost, np.where(inside, -4, 0))
    for prec in ("fp64", "mixed"):
        _, st = nb.flowmap_grid_2D(fl, 24.0, -18.0, xs, ys, p, return_status=True, precision=prec)
        assert np.array_equal(st, ost), prec
    for sched in (-1, -2, 2):
        f = Field(fl, 24.0, -18.0, xs, ys, p)
        FTLEBatch([f], precision="mixed", blocks_per_sm=sched, graph=False).run()
        assert np.array_equal(f.status.cpu().numpy(), ost), sched
    # a one-step limit in the batch: MAX_STEPS where the oracle gives up too
    U[4, 5, 4] = 1.0
    grid, Cu, Cv = nb.get_interp_arrays_2D(tv, lon, lat, U, V)
    fl = nb.get_flow_2D(grid, Cu, Cv, spherical=1)
    og, oCu, oCv = orc.get_interp_arrays_2D(tv, lon, lat, U, V)
    _, ost1, _ = orc.flowmap_grid_2D(orc.spline_flow(og, oCu, oCv, spherical=1), 24.0, -18.0, xs,
                                     ys, p, nmax=1, return_status=True)
    assert (ost1 == -2).all()
    for sched in (-1, -2, 2):
        f = Field(fl, 24.0, -18.0, xs, ys, p)
        FTLEBatch([f], precision="mixed", blocks_per_sm=sched, graph=False, max_steps=1).run()
        assert np.array_equal(f.status.cpu().numpy(), ost1), sched


def test_flowmap_pts(nb, orc, golden, coords_dg, mask_dg):
    """flowmap / flowmap_grid_ND (integration.py:8-62, :186-247): a point list
    laid out 8 points to a row of a virtual grid; 231 points leave a partial
    last row that is neither integrated nor written."""
    x, y = coords_dg
    X, Y = np.meshgrid(x, y, indexing="ij")
    pts = np.column_stack((X.ravel(), Y.ravel()))
    fl, p, _ = nb.get_predefined_flow("double_gyre")
    fm = nb.flowmap(fl, 0.0, 8.0, pts, p)
    assert fm.shape == (231, 2)
    assert np.allclose(fm.reshape(21, 11, 2).astype(np.float32), golden["fm"])
    # the same particles as the grid call, so the same bits
    for prec in ("fp64", "mixed"):
        g = nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p, precision=prec)
        f = nb.flowmap(fl, 0.0, 8.0, pts, p, precision=prec)
        assert np.array_equal(f.reshape(21, 11, 2), g), prec
    fmm, st = nb.flowmap(fl, 0.0, 8.0, pts, p, mask=mask_dg.ravel(), return_status=True)
    exp = golden["fm"].copy()
    exp[mask_dg] = 0.0
    assert np.allclose(fmm.reshape(21, 11, 2).astype(np.float32), exp)
    assert np.array_equal(st == 1, mask_dg.ravel()) and (st[~mask_dg.ravel()] == 0).all()
    assert np.array_equal(nb.flowmap_grid_ND(fl, 0.0, 8.0, pts.ravel(), 2, p), fm)
    assert nb.flowmap(fl, 0.0, 8.0, np.zeros((0, 2)), p).shape == (0, 2)
    # a spline flow on scattered points: FP64 bit-identical to the oracle, with
    # identical statuses (points outside the grid box stay put)
    tv, lon, lat = np.arange(9) * 3.0, np.linspace(-20.0, 20.0, 11), np.linspace(0.0, 30.0, 9)
    T3, X3, Y3 = np.meshgrid(tv, lon, lat, indexing="ij")
    U = 30.0 * np.sin(0.15 * X3 + 0.05 * T3) * np.cos(0.1 * Y3)
    V = 20.0 * np.cos(0.12 * X3) * np.sin(0.2 * Y3 - 0.03 * T3)
    grid, Cu, Cv = nb.get_interp_arrays_2D(tv, lon, lat, U, V)
    sfl = nb.get_flow_2D(grid, Cu, Cv, spherical=1)
    og, oCu, oCv = orc.get_interp_arrays_2D(tv, lon, lat, U, V)
    ofl = orc.spline_flow(og, oCu, oCv, spherical=1)
    rng = np.random.default_rng(3)
    sp = np.column_stack((rng.uniform(-25.0, 25.0, 1003), rng.uniform(-2.0, 32.0, 1003)))
    sm = rng.random(1003) < 0.1
    ps = np.array([-1.0])
    f64, s64 = nb.flowmap(sfl, 24.0, -18.0, sp, ps, mask=sm, return_status=True)
    of, ost = orc.flowmap(ofl, 24.0, -18.0, sp, ps, mask=sm, return_status=True)
    assert np.array_equal(f64, of) and np.array_equal(s64, ost)
    f32 = nb.flowmap(sfl, 24.0, -18.0, sp, ps, mask=sm, precision="mixed")
    # mixed against FP64 at the default rtol: FP32-stage noise, except where a
    # trajectory grazes the box edge and the two leave it at different times
    e = np.abs(f32 - of).max(-1)
    assert np.median(e) <= 1e-5 and np.quantile(e, 0.99) <= 1e-3, (np.median(e), e.max())
    # torch in, torch out, on the device
    tp = torch.from_numpy(sp).cuda()
    ft = nb.flowmap(sfl, 24.0, -18.0, tp, ps, mask=torch.from_numpy(sm).cuda())
    assert ft.is_cuda and torch.equal(ft.cpu(), torch.from_numpy(f64))


def test_flowmap_n(nb, orc, golden, coords_dg, mask_dg):
    """flowmap_n / flowmap_n_grid_2D (integration.py:65-121, :468-534) by
    dense output: the reference's fm_n.npy, plain and masked; the last output
    is flowmap_grid_2D's end point; a spline flow bit-identical to the oracle,
    forward and backward, including T = 0 and n = 1."""
    x, y = coords_dg
    X, Y = np.meshgrid(x, y, indexing="ij")
    pts = np.column_stack((X.ravel(), Y.ravel()))
    fl, p, _ = nb.get_predefined_flow("double_gyre")
    fm_n, te = nb.flowmap_n(fl, 0.0, 8.0, pts, p, n=4)
    assert np.allclose(te, p[0] * np.linspace(0.0, 8.0, 4))
    assert np.allclose(fm_n.reshape(21, 11, 4, 2).astype(np.float32), golden["fm_n"])
    g, te2 = nb.flowmap_n_grid_2D(fl, 0.0, 8.0, x, y, p, n=4)
    assert np.array_equal(g, fm_n.reshape(21, 11, 4, 2)) and np.array_equal(te, te2)
    # the interpolant at the end is (y1 - y0) + y0: y1 up to one rounding
    assert np.abs(g[:, :, -1] - nb.flowmap_grid_2D(fl, 0.0, 8.0, x, y, p)).max() <= 1e-15
    gm, _, st = nb.flowmap_n_grid_2D(fl, 0.0, 8.0, x, y, p, n=4, mask=mask_dg,
                                      return_status=True)
    assert np.allclose(gm.astype(np.float32), apply_mask(golden["fm_n"], mask_dg))
    assert np.array_equal(st == 1, mask_dg)
    # spline flow: the same arithmetic as the oracle
    tv, lon, lat = np.arange(9) * 3.0, np.linspace(-20.0, 20.0, 11), np.linspace(0.0, 30.0, 9)
    T3, X3, Y3 = np.meshgrid(tv, lon, lat, indexing="ij")
    U = 30.0 * np.sin(0.15 * X3 + 0.05 * T3) * np.cos(0.1 * Y3)
    V = 20.0 * np.cos(0.12 * X3) * np.sin(0.2 * Y3 - 0.03 * T3)
    grid, Cu, Cv = nb.get_interp_arrays_2D(tv, lon, lat, U, V)
    sfl = nb.get_flow_2D(grid, Cu, Cv, spherical=1)
    og, oCu, oCv = orc.get_interp_arrays_2D(tv, lon, lat, U, V)
    ofl = orc.spline_flow(og, oCu, oCv, spherical=1)
    rng = np.random.default_rng(5)
    sp = np.column_stack((rng.uniform(-25.0, 25.0, 301), rng.uniform(-2.0, 32.0, 301)))
    ps = np.array([-1.0])
    for t0, T, n in ((24.0, -18.0, 7), (3.0, 20.0, 5), (10.0, 0.0, 3), (10.0, 5.0, 1)):
        a, ta, sa = nb.flowmap_n(sfl, t0, T, sp, ps, n=n, return_status=True)
        b, tb, sb = orc.flowmap_n(ofl, t0, T, sp, ps, n=n, return_status=True)
        assert np.array_equal(a, b) and np.array_equal(ta, tb) and np.array_equal(sa, sb), (t0, T)
    # torch in, torch out
    at, _ = nb.flowmap_n(sfl, 24.0, -18.0, torch.from_numpy(sp).cuda(), ps, n=7)
    assert at.is_cuda and torch.equal(at.cpu(), torch.from_numpy(nb.flowmap_n(sfl, 24.0, -18.0, sp, ps, n=7)[0]))
