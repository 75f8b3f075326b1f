"""The CPU oracle against the reference's golden vectors (CPU only).

Mirrors the reference tests: tests/test_integration.py:55-64,
tests/test_diagnostics.py:82-96 and :133-150, tests/test_extraction.py:6-20,
tests/test_flows.py:68-139, :208-237 and :307-357.  Comparisons are the
reference's own: np.allclose on float32-cast results.
"""
import numpy as np
import pytest

from conftest import apply_mask, reconstruct

T_FIX = 8.0


def test_flowmap_grid_2D(orc, golden, coords_dg, mask_dg):
    x, y = coords_dg
    p = orc.double_gyre_params(1.0)
    fm, st, stats = orc.flowmap_grid_2D(orc.double_gyre(), 0.0, T_FIX, x, y, p, return_status=True)
    assert np.allclose(fm.astype(np.float32), golden["fm"])
    assert (st == 0).all()
    # DOP853 work counters: 12 RHS per attempted step + 2 (initial step) + 1
    # (first derivative); nfcn = 2 + 12*attempted - (#rejected) (no FSAL on rejection)
    att = stats[..., 0] + stats[..., 1]
    assert (stats[..., 2] <= 2 + 12 * att + 1).all()
    fmm = orc.flowmap_grid_2D(orc.double_gyre(), 0.0, T_FIX, x, y, p, mask=mask_dg)
    assert np.allclose(fmm.astype(np.float32), apply_mask(golden["fm"], mask_dg))


def test_libm_mode_reproduces_golden_and_matches_in_accuracy(orc, golden, coords_dg):
    """The oracle's default arithmetic uses two deterministic helpers that the
    GPU library shares (err^(1/8) as three square roots, a Taylor-series cos
    in the spherical metric) so that the two can be compared bit for bit.  Its
    libm mode makes the reference's literal pow / cos calls instead.  Both
    reproduce the golden flow map; on the geophysical spline flow the helpers
    move trajectories by the flow's sensitivity to one ulp, and both runs are
    equally accurate against a converged solution."""
    x, y = coords_dg
    p = orc.double_gyre_params(1.0)
    a = orc.flowmap_grid_2D(orc.double_gyre(), 0.0, T_FIX, x, y, p)
    b = orc.flowmap_grid_2D(orc.double_gyre(libm=True), 0.0, T_FIX, x, y, p)
    assert np.array_equal(a.astype(np.float32), golden["fm"])
    assert np.array_equal(b.astype(np.float32), golden["fm"])
    assert np.abs(a - b).max() <= 1e-10
    from numbacs_gb300 import workloads as W
    t, lon, lat, U, V = W.geo_velocity(seed=0, device="cpu")
    g, cu, cv = orc.get_interp_arrays_2D(t, lon, lat, U, V)
    lonf, latf = W.geo_ftle_grid(0.2)
    xs, pm = lonf[::16], np.array([-1.0])
    det = orc.flowmap_grid_2D(orc.spline_flow(g, cu, cv, spherical=1), 180.0, -72.0, xs, latf, pm,
                              rtol=1e-7, atol=1e-9)
    lib = orc.flowmap_grid_2D(orc.spline_flow(g, cu, cv, spherical=1, libm=True), 180.0, -72.0, xs,
                              latf, pm, rtol=1e-7, atol=1e-9)
    tr = orc.flowmap_grid_2D(orc.spline_flow(g, cu, cv, spherical=1, libm=True), 180.0, -72.0, xs,
                             latf, pm, rtol=1e-12, atol=1e-14)
    bound = 1e-6 * (lon[-1] - lon[0])
    d = np.abs(det - lib).max(-1)
    assert np.median(d) <= 1e-3 * bound
    e_det, e_lib = np.abs(det - tr).max(-1), np.abs(lib - tr).max(-1)
    assert abs(e_det.mean() - e_lib.mean()) <= 0.05 * e_lib.mean()
    assert abs(np.quantile(e_det, 0.99) - np.quantile(e_lib, 0.99)) <= 0.05 * np.quantile(e_lib, 0.99)


def test_ftle_grid_2D(orc, golden, mask_dg):
    fm = golden["fm"].astype(np.float64)
    f = orc.ftle_grid_2D(fm, T_FIX, 0.1, 0.1)
    assert np.allclose(f.astype(np.float32), golden["ftle"])
    fmk = orc.ftle_grid_2D(fm, T_FIX, 0.1, 0.1, mask=mask_dg)
    assert np.allclose(fmk.astype(np.float32), apply_mask(golden["ftle"], mask_dg))


def test_C_eig_2D(orc, golden, mask_dg):
    fm = golden["fm"].astype(np.float64)
    ev, vec = orc.C_eig_2D(fm, 0.1, 0.1)
    C_exp = reconstruct(golden["Cevals"], golden["Cevecs"])
    assert np.allclose(reconstruct(ev.astype(np.float32), vec.astype(np.float32)), C_exp)
    evm, vecm = orc.C_eig_2D(fm, 0.1, 0.1, mask_dg)
    assert np.allclose(reconstruct(evm.astype(np.float32), vecm.astype(np.float32)),
                       apply_mask(C_exp, mask_dg))
    # ftle_from_eig(eigvals[...,1]) reproduces the FTLE fixture
    f = orc.ftle_from_eig(ev[..., 1], T_FIX)
    assert np.allclose(f.astype(np.float32), golden["ftle"])


def test_ridge_pts_and_ridges(orc, golden, coords_dg):
    x, y = coords_dg
    f = golden["ftle"].astype(np.float64)
    e = golden["Cevecs"][:, :, :, 1].astype(np.float64)
    rp = orc.ftle_ridge_pts(f, e, x, y)
    assert rp.shape == golden["ridge_pts"].shape
    assert np.allclose(rp, golden["ridge_pts"])
    ridges = orc.ftle_ridges(f, e, x, y)
    assert len(ridges) == int(golden["n_ridges"])
    for k, r in enumerate(ridges):
        assert np.allclose(r, golden["ridges_%d" % k])


def _spline_case():
    t = np.array([0.0, 0.1, 0.2])
    xs = np.array([0.0, 0.5, 1.0])
    T, X, Y = np.meshgrid(t, xs, xs, indexing="ij")
    u = np.sin(X) * np.cos(Y) + np.sin(T)
    v = np.cos(X) * np.sin(Y) + np.cos(T)
    xi = np.array([0.1, 0.4, 0.7])
    ti = np.array([0.05, 0.12, 0.18])
    Ti, Xi, Yi = np.meshgrid(ti, xi, xi, indexing="ij")
    pts = np.column_stack((Ti.ravel(), Xi.ravel(), Yi.ravel()))
    return t, xs, u, v, pts


def test_spline_prefilter_and_eval(orc, golden):
    t, xs, u, v, pts = _spline_case()
    grid, Cu, Cv = orc.get_interp_arrays_2D(t, xs, xs, u, v)
    assert np.allclose(Cu, golden["spline_Cu"]) and np.allclose(Cv, golden["spline_Cv"])
    vel = np.array([[orc.eval_spline_3d(grid, Cu, *q), orc.eval_spline_3d(grid, Cv, *q)] for q in pts])
    assert np.allclose(vel, golden["spline_vel"])


def test_predefined_rhs(orc, golden):
    *_, pts = _spline_case()
    dg = np.array([orc.rhs(orc.double_gyre(), q[0], q[1:], orc.double_gyre_params(1.0)) for q in pts])
    assert np.allclose(dg, golden["dg_vel"])
    bj = np.array([orc.rhs(orc.bickley_jet(), q[0], q[1:], orc.bickley_params()) for q in pts])
    assert np.allclose(bj, golden["bickley_vel"])


@pytest.mark.parametrize("n", [1, 2, 11, 1000, 4097])
@pytest.mark.parametrize("q", [0.0, 12.5, 50.0, 90.0, 99.9, 100.0])
def test_percentile_matches_numpy(orc, n, q):
    # numba's linear-rank percentile agrees with numpy's linear method to
    # rounding; both pick the same two order statistics
    rng = np.random.default_rng(n)
    a = rng.standard_normal(n)
    a[: n // 3] = 0.0  # ties, like the zero border of an FTLE field
    assert np.isclose(orc.percentile(a, q), np.percentile(a, q), rtol=1e-14, atol=1e-14)


def test_percentile_nan_inf_rules(orc):
    assert np.isnan(orc.percentile(np.array([1.0, np.nan, 3.0]), 50))
    assert np.isnan(orc.percentile(np.array([1.0, np.inf, 3.0]), 100))
    assert orc.percentile(np.array([1.0, -np.inf, 3.0]), 100) == 3.0


def test_deterministic_math_accuracy(orc):
    # shared + - * / sqrt implementations: within ~1 ulp of libm
    for d in np.concatenate([np.linspace(-400, 400, 20001), [0.0, 45.0, 90.0, -90.0, 180.0]]):
        c, r = orc.cos_deg(d), np.cos(np.radians(d))
        assert abs(c - r) <= 4.5e-16 * max(1.0, abs(r)) + 1e-16, d
    for x in np.concatenate([np.geomspace(1e-300, 1e300, 2001), [0.0, 1.0]]):
        assert abs(orc.root8(x) - x ** 0.125) <= 3e-16 * x ** 0.125, x


def test_extrapolation_is_constant(orc):
    # extrap_mode="constant" (the interpolation package's CONSTANT option): 0
    # strictly outside the grid box, the spline's value on it
    t, xs, u, v, pts = _spline_case()
    grid, Cu, _ = orc.get_interp_arrays_2D(t, xs, xs, u, v)
    (t0, t1, _), (x0, x1, _), (y0, y1, _) = grid
    on_edge = orc.eval_spline_3d(grid, Cu, t0, x1, y0)
    assert on_edge != 0.0
    assert orc.eval_spline_3d(grid, Cu, t0, np.nextafter(x1, 2 * x1), y0) == 0.0
    assert orc.eval_spline_3d(grid, Cu, np.nextafter(t0, -1.0), x0, y0) == 0.0
    assert orc.eval_spline_3d(grid, Cu, 0.5 * (t0 + t1), 0.5 * (x0 + x1), y1 + 1.0) == 0.0


def _linear_field(a=0.3, bt=-0.7, bx=1.9, by=0.45):
    """Samples of a field linear in (t, x, y): the natural-boundary cubic
    spline reproduces it exactly inside the box."""
    t = np.linspace(0.0, 6.0, 7)
    x = np.linspace(-2.0, 3.0, 11)
    y = np.linspace(1.0, 2.5, 6)
    T, X, Y = np.meshgrid(t, x, y, indexing="ij")
    return t, x, y, a + bt * T + bx * X + by * Y, (a, bt, bx, by)


def test_extrapolation_nearest_and_linear(orc):
    """extrap_mode "nearest" and "linear" (no reference fixture pins them; the
    oracle's definition): nearest = the value at the clamped point; linear =
    that value plus derivative x distance along each clamped axis, which
    continues a linear field exactly."""
    t, x, y, U, (a, bt, bx, by) = _linear_field()
    grid, C, _ = orc.get_interp_arrays_2D(t, x, y, U, U)
    lin = lambda p: a + bt * p[0] + bx * p[1] + by * p[2]
    rng = np.random.default_rng(5)
    inside = np.column_stack([rng.uniform(0, 6, 20), rng.uniform(-2, 3, 20), rng.uniform(1, 2.5, 20)])
    outside = inside + rng.choice([-1.0, 0.0, 1.0], (20, 3)) * rng.uniform(0.1, 4.0, (20, 3))
    lo = np.array([0.0, -2.0, 1.0])
    hi = np.array([6.0, 3.0, 2.5])
    for p in np.vstack([inside, outside]):
        c = np.clip(p, lo, hi)
        v1 = orc.eval_spline_3d(grid, C, *p, extrap=1)
        assert v1 == orc.eval_spline_3d(grid, C, *c, extrap=1)
        assert v1 == orc.eval_spline_3d(grid, C, *c, extrap=0)
        assert abs(v1 - lin(c)) <= 1e-12
        v2 = orc.eval_spline_3d(grid, C, *p, extrap=2)
        assert abs(v2 - lin(p)) <= 1e-11, (p, v2, lin(p))
        if np.any(p != c):
            assert orc.eval_spline_3d(grid, C, *p, extrap=0) == 0.0
    # a curved field: "linear" is continuous at the box surface and its slope
    # beyond it is the one-sided derivative there
    t, xs, u, v, _ = _spline_case()
    grid, Cu, _ = orc.get_interp_arrays_2D(t, xs, xs, u, v)
    edge = orc.eval_spline_3d(grid, Cu, 0.1, 1.0, 0.3, extrap=2)
    assert orc.eval_spline_3d(grid, Cu, 0.1, 1.0 + 1e-9, 0.3, extrap=2) == pytest.approx(edge, abs=1e-8)
    d_in = (edge - orc.eval_spline_3d(grid, Cu, 0.1, 1.0 - 1e-6, 0.3)) / 1e-6
    d_out = (orc.eval_spline_3d(grid, Cu, 0.1, 1.5, 0.3, extrap=2) - edge) / 0.5
    assert d_out == pytest.approx(d_in, rel=1e-5)


GRID_DG = ((0.0, 2.0, 21), (0.0, 1.0, 11))


def test_flowmap_composition_initial(orc, golden, coords_dg):
    """tests/test_integration.py:92-103: double gyre, t0 = 0, T = 8, h = 1 -> nT = 8."""
    x, y = coords_dg
    p = orc.double_gyre_params(1.0)
    fm0, fms, nT = orc.flowmap_composition_initial(orc.double_gyre(), 0.0, T_FIX, 1.0, x, y,
                                                   GRID_DG, p)
    assert nT == 8
    assert np.allclose(fms.astype(np.float32), golden["fms_ci"])
    assert np.allclose(fm0.astype(np.float32), golden["fm_ci"])


def test_flowmap_composition_step(orc, golden, coords_dg):
    """tests/test_integration.py:105-114: one step from the float32 fixture maps at t0 = 8."""
    x, y = coords_dg
    p = orc.double_gyre_params(1.0)
    fms = golden["fms_ci"].astype(np.float64)
    fmk, fms2 = orc.flowmap_composition_step(fms, orc.double_gyre(), T_FIX, 1.0, 8, x, y,
                                             GRID_DG, p)
    assert np.allclose(fmk.astype(np.float32), golden["fm_cs"])
    assert np.allclose(fms2.astype(np.float32), golden["fms_cs"])


def test_flowmap_composition_ring_order_and_nT1(orc, golden):
    """Ring order (first = r) equals composing the rolled stack; nT = 1 composes the
    single map with itself, as integration.py:630-640 does."""
    fms = golden["fms_ci"].astype(np.float64)
    ref = orc.flowmap_composition(fms, GRID_DG, 8)
    for r in (1, 3, 7):
        ring = np.roll(fms, r, axis=0)  # map j of the sequence sits at index (j + r) % 8
        assert np.array_equal(orc.flowmap_composition(ring, GRID_DG, 8, first=r), ref)
    one = orc.flowmap_composition(fms[:1], GRID_DG, 1)
    two = orc.flowmap_composition(np.stack([fms[0], fms[0]]), GRID_DG, 2)
    assert np.array_equal(one, two)


def test_flowmap_aux_grid_2D(orc, golden, coords_dg, mask_dg):
    """tests/test_integration.py:66-75."""
    x, y = coords_dg
    p = orc.double_gyre_params(1.0)
    fa, st, _ = orc.flowmap_aux_grid_2D(orc.double_gyre(), 0.0, T_FIX, x, y, p, return_status=True)
    assert fa.shape == (21, 11, 5, 2)
    assert np.allclose(fa.astype(np.float32), golden["fm_aux"])
    # edge points integrate their centre particle only; interior points all five
    edge = np.zeros((21, 11), bool)
    edge[[0, -1], :] = True
    edge[:, [0, -1]] = True
    assert (st[edge][:, :4] == 1).all() and (st[edge][:, 4] == 0).all()
    assert (st[~edge] == 0).all()
    # the centre particles are the plain flow map
    fm = orc.flowmap_grid_2D(orc.double_gyre(), 0.0, T_FIX, x, y, p)
    assert np.array_equal(fa[:, :, 4], fm)
    fam = orc.flowmap_aux_grid_2D(orc.double_gyre(), 0.0, T_FIX, x, y, p, mask=mask_dg)
    assert np.allclose(fam.astype(np.float32), apply_mask(golden["fm_aux"], mask_dg))


def test_flowmap_aux_grid_2D_variants(orc, coords_dg):
    """eig_main=False (4 aux particles) and compute_edge=False skip rules
    (integration.py:320-464)."""
    x, y = coords_dg
    p = orc.double_gyre_params(1.0)
    f4, s4, _ = orc.flowmap_aux_grid_2D(orc.double_gyre(), 0.0, 2.0, x, y, p, eig_main=False,
                                        return_status=True)
    assert f4.shape == (21, 11, 4, 2) and (s4 == 0).all()
    f5 = orc.flowmap_aux_grid_2D(orc.double_gyre(), 0.0, 2.0, x, y, p)
    assert np.array_equal(f4[1:-1, 1:-1], f5[1:-1, 1:-1, :4])
    fn, sn, _ = orc.flowmap_aux_grid_2D(orc.double_gyre(), 0.0, 2.0, x, y, p, compute_edge=False,
                                        return_status=True)
    assert (sn[[0, -1]] == 1).all() and (sn[:, [0, -1]] == 1).all()
    assert (fn[[0, -1]] == 0).all() and (fn[:, [0, -1]] == 0).all()
    assert np.array_equal(fn[1:-1, 1:-1], f5[1:-1, 1:-1])


def test_C_eig_aux_2D(orc, golden, mask_dg):
    """tests/test_diagnostics.py:112-131 (fed the float32 fixture, as there)."""
    fa = golden["fm_aux"].astype(np.float64)
    ev, vec = orc.C_eig_aux_2D(fa, 0.1, 0.1)
    C_exp = reconstruct(golden["Cevals_aux"], golden["Cevecs_aux"])
    assert np.allclose(reconstruct(ev.astype(np.float32), vec.astype(np.float32)), C_exp)
    evm, vecm = orc.C_eig_aux_2D(fa, 0.1, 0.1, mask=mask_dg)
    assert np.allclose(reconstruct(evm.astype(np.float32), vecm.astype(np.float32)),
                       apply_mask(C_exp, mask_dg))
    # eig_main=False: both from the aux stencil, over the 1-wide interior
    ev4, vec4 = orc.C_eig_aux_2D(fa[:, :, :4], 0.1, 0.1, eig_main=False)
    assert np.array_equal(vec4[2:-2, 2:-2], vec[2:-2, 2:-2])
    assert (ev4[1:-1, 1:-1, 1] > 0).all()


def _native_ordered():
    from numbacs_gb300 import build
    build.build()
    from numbacs_gb300.extraction.ordered import ordered_from_ridge_field
    return ordered_from_ridge_field


@pytest.mark.parametrize("impl", ["oracle", "native"])
def test_ordered_ridges_golden(orc, golden, coords_dg, impl):
    """tests/test_extraction.py:22-28: the linking of the oracle restatement
    and of the native nbcs_order_ridges (host code), fed by the oracle's ridge
    test."""
    if impl == "oracle":
        from oracle.ordered_ref import ordered_from_ridge_field
    else:
        ordered_from_ridge_field = _native_ordered()
    x, y = coords_dg
    f = golden["ftle"].astype(np.float64)
    e = np.ascontiguousarray(golden["Cevecs"][:, :, :, 1].astype(np.float64))
    rpts, mask, _ = orc.ridge_field(f, e, x, y)
    ridges = ordered_from_ridge_field(f, e, x, y, mask, rpts, 0.1)
    n = int(golden["n_ordered"])
    assert len(ridges) == n
    for k in range(n):
        assert ridges[k].shape == golden["ordered_%d" % k].shape
        assert np.allclose(ridges[k], golden["ordered_%d" % k])


def _ridge_test_field(orc, nx, ny, seed):
    rng = np.random.default_rng(seed)
    x, y = np.linspace(0, 2, nx), np.linspace(0, 1, ny)
    X, Y = np.meshgrid(x, y, indexing="ij")
    fm = np.stack([X + 0.05 * np.sin(7 * Y + 3 * X) + 0.03 * np.sin(23 * X * Y),
                   Y + 0.05 * np.cos(5 * X) + 0.02 * np.cos(17 * Y - 4 * X)], -1)
    fm = fm + 1e-3 * rng.standard_normal(fm.shape)
    ev, vec = orc.C_eig_2D(fm, x[1] - x[0], y[1] - y[0])
    f = orc.ftle_from_eig(ev[..., 1], 5.0)
    return x, y, f, np.ascontiguousarray(vec[..., :, 1])


@pytest.mark.parametrize("nx,ny,seed,pct,tol", [(301, 157, 0, 0, 0.02), (676, 251, 1, 90, 0.05),
                                                (400, 400, 2, 50, 0.01), (120, 90, 3, 0, 0.2)])
def test_ordered_ridges_native_equals_oracle(orc, nx, ny, seed, pct, tol):
    """The native linker makes the restatement's decisions: the same curves,
    point for point, on fields with thousands of ridge points."""
    from oracle.ordered_ref import ordered_from_ridge_field as ref
    native = _native_ordered()
    x, y, f, e = _ridge_test_field(orc, nx, ny, seed)
    rpts, mask, _ = orc.ridge_field(f, e, x, y, 0.0, pct)
    assert mask.sum() > 100
    for kw in ({}, {"min_ridge_pts": 2, "ep_tan_ang": 0.3}, {"c": 0.0}):
        a = ref(f, e, x, y, mask, rpts, tol, **kw)
        b = native(f, e, x, y, mask, rpts, tol, **kw)
        assert len(a) == len(b) and len(a) > 0
        for ra, rb in zip(a, b):
            assert np.array_equal(ra, rb)


def test_ordered_ridges_options(orc, golden, coords_dg):
    """min_ridge_pts and the endpoint tolerances act as filters: fewer or equal
    curves, every curve one of the ridge points' paths."""
    ordered_from_ridge_field = _native_ordered()
    x, y = coords_dg
    f = golden["ftle"].astype(np.float64)
    e = np.ascontiguousarray(golden["Cevecs"][:, :, :, 1].astype(np.float64))
    rpts, mask, _ = orc.ridge_field(f, e, x, y)
    pts = {tuple(p) for p in rpts[mask.ravel()]}
    for kw in ({"min_ridge_pts": 2}, {"min_ridge_pts": 7}, {"dist_tol": 1e-3},
               {"ep_tan_ang": 0.1}):
        args = dict(dist_tol=0.1)
        args.update(kw)
        ridges = ordered_from_ridge_field(f, e, x, y, mask, rpts, args.pop("dist_tol"), **args)
        for r in ridges:
            assert all(tuple(p) in pts for p in r)


def test_ordered_ridges_native_buffers(orc, golden, coords_dg):
    """nbcs_order_ridges reports the totals and refuses buffers that are too
    small (host code; no GPU)."""
    import ctypes
    from numbacs_gb300 import _lib, build
    build.build()
    L = _lib.load()
    x, y = coords_dg
    f = np.ascontiguousarray(golden["ftle"].astype(np.float64))
    e = np.ascontiguousarray(golden["Cevecs"][:, :, :, 1].astype(np.float64))
    rpts, mask, _ = orc.ridge_field(f, e, x, y)
    m = np.ascontiguousarray(mask, np.uint8)
    rp = np.ascontiguousarray(rpts)
    n_pts, n_r = ctypes.c_int64(0), ctypes.c_int64(0)
    vp = _lib._vp
    args = [f.ctypes.data_as(vp), e.ctypes.data_as(vp), x.ctypes.data_as(vp), len(x),
            y.ctypes.data_as(vp), len(y), m.ctypes.data_as(vp), rp.ctypes.data_as(vp), 0.1,
            np.pi / 4, 5, 0.0, 1.0]
    pts = np.empty((1, 2))
    lens = np.empty(1, np.int64)
    rc = L.nbcs_order_ridges(*args, pts.ctypes.data_as(vp), 1, lens.ctypes.data_as(vp), 1,
                             ctypes.byref(n_pts), ctypes.byref(n_r))
    assert rc == -3 and n_r.value == int(golden["n_ordered"])
    assert n_pts.value == sum(golden["ordered_%d" % k].shape[0] for k in range(n_r.value))
    rc = L.nbcs_order_ridges(*args, None, 0, None, 0, None, None)
    assert rc == -1


def _cauchy_green(g):
    """C = F^T F from the stencil tuple (dFx/dx, dFx/dy, dFy/dx, dFy/dy), as the
    reference assembles it (diagnostics.py:161-175)."""
    a, b, c, d = g
    off = a * b + c * d
    return np.array([[a * a + c * c, off], [off, b * b + d * d]])


def stencil_literal_checks(C_eig_2D, C_eig_aux_2D, golden, coords_dg):
    """The reference's stencil literals (tests/test_utils.py:74-120, 190-199)
    through the Cauchy-Green eigen-solvers: C at grid point (5, 5) of fm.npy and
    fm_aux.npy, and eigvalsh_max_2D of B^T B via a linear flow map."""
    x, y = coords_dg
    dx, dy = x[1], y[1]
    fm = golden["fm"].astype(np.float64)
    ev, vec = (np.asarray(a) for a in C_eig_2D(fm, dx, dy))
    C = vec[5, 5] @ np.diag(ev[5, 5]) @ vec[5, 5].T
    assert np.allclose(C, _cauchy_green(golden["gradF_55"]))
    fa = golden["fm_aux"].astype(np.float64)
    ev, vec = (np.asarray(a) for a in C_eig_aux_2D(fa, dx, dy, 1e-5))
    # eig_main: eigenvalues of the main-grid C, eigenvectors of the +-h C
    assert np.allclose(ev[5, 5], np.linalg.eigvalsh(_cauchy_green(golden["gradF_main_55"])))
    _, v_aux = np.linalg.eigh(_cauchy_green(golden["gradF_aux_55"]))
    assert np.allclose(np.abs(np.sum(vec[5, 5] * v_aux, axis=0)), 1.0)
    ev4, vec4 = (np.asarray(a) for a in C_eig_aux_2D(np.ascontiguousarray(fa[:, :, :4]), dx, dy,
                                                       1e-5, eig_main=False))
    C4 = vec4[5, 5] @ np.diag(ev4[5, 5]) @ vec4[5, 5].T
    assert np.allclose(C4, _cauchy_green(golden["gradF_aux_55"]))
    # a linear flow map F(x, y) = B (x, y): central differences give F = B exactly
    # up to rounding, so lambda_max(C) is eigvalsh_max_2D(B^T B)
    B = golden["eigvalsh_B"]
    xg, yg = np.linspace(0.0, 1.0, 7), np.linspace(0.0, 2.0, 9)
    X, Y = np.meshgrid(xg, yg, indexing="ij")
    lin = np.stack([B[0, 0] * X + B[0, 1] * Y, B[1, 0] * X + B[1, 1] * Y], axis=-1)
    ev, _ = (np.asarray(a) for a in C_eig_2D(lin, xg[1], yg[1]))
    lmax = ev[1:-1, 1:-1, 1]
    assert np.allclose(lmax, float(golden["eigvalsh_max"]), rtol=1e-12, atol=0)


def test_stencil_golden_literals(orc, golden, coords_dg):
    stencil_literal_checks(orc.C_eig_2D, orc.C_eig_aux_2D, golden, coords_dg)


def test_flowmap_pts_golden(orc, golden, coords_dg, mask_dg):
    """flowmap on the grid's points (tests/test_integration.py:37-41), plain
    and masked (a mask over the points leaves their rows 0)."""
    x, y = coords_dg
    X, Y = np.meshgrid(x, y, indexing="ij")
    pts = np.column_stack((X.ravel(), Y.ravel()))
    dg = orc.double_gyre()
    p = np.array([1.0, 0.1, 0.25, 0.0, 0.2 * np.pi, 0.0])
    fm = orc.flowmap(dg, 0.0, 8.0, pts, p).reshape(len(x), len(y), 2)
    assert np.allclose(fm.astype(np.float32), golden["fm"])
    assert np.array_equal(fm, orc.flowmap_grid_2D(dg, 0.0, 8.0, x, y, p))
    fmm, st = orc.flowmap(dg, 0.0, 8.0, pts, p, mask=mask_dg.ravel(), return_status=True)
    exp = golden["fm"].copy()
    exp[mask_dg] = 0.0
    assert np.allclose(fmm.reshape(len(x), len(y), 2).astype(np.float32), exp)
    assert np.array_equal(st == 1, mask_dg.ravel())


def test_C_tensor_2D_golden(orc, golden, mask_dg):
    """C_tensor_2D of fm_aux.npy (tests/test_diagnostics.py:99-109), plain and masked."""
    fa = golden["fm_aux"].astype(np.float64)
    C = orc.C_tensor_2D(fa, 0.1, 0.1)
    assert np.allclose(C.astype(np.float32), golden["C"])
    exp = golden["C"].copy()
    exp[mask_dg] = 0.0
    assert np.allclose(orc.C_tensor_2D(fa, 0.1, 0.1, mask=mask_dg).astype(np.float32), exp)


def test_flowmap_n_golden(orc, golden, coords_dg, mask_dg):
    """flowmap_n / flowmap_n_grid_2D (tests/test_integration.py:45-52, :78-90):
    dop853's dense output over one run reproduces fm_n.npy, plain and masked;
    the last output is flowmap_grid_2D's end point."""
    x, y = coords_dg
    X, Y = np.meshgrid(x, y, indexing="ij")
    pts = np.column_stack((X.ravel(), Y.ravel()))
    dg = orc.double_gyre()
    p = np.array([1.0, 0.1, 0.25, 0.0, 0.2 * np.pi, 0.0])
    fm_n, te = orc.flowmap_n(dg, 0.0, 8.0, pts, p, n=4)
    assert np.allclose(te, p[0] * np.linspace(0.0, 8.0, 4))
    assert np.allclose(fm_n.reshape(21, 11, 4, 2).astype(np.float32), golden["fm_n"])
    g, _ = orc.flowmap_n_grid_2D(dg, 0.0, 8.0, x, y, p, n=4)
    assert np.array_equal(g, fm_n.reshape(21, 11, 4, 2))
    assert np.array_equal(g[:, :, -1], orc.flowmap_grid_2D(dg, 0.0, 8.0, x, y, p))
    gm, _ = orc.flowmap_n_grid_2D(dg, 0.0, 8.0, x, y, p, n=4, mask=mask_dg)
    exp = golden["fm_n"].copy()
    exp[mask_dg] = 0.0
    assert np.allclose(gm.astype(np.float32), exp)
