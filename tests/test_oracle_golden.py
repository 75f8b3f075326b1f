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
    # extrap_mode="constant": outside the grid box the value on its boundary
    t, xs, u, v, pts = _spline_case()
    grid, Cu, _ = orc.get_interp_arrays_2D(t, xs, xs, u, v)
    inside = orc.eval_spline_3d(grid, Cu, 0.2, 1.0, 0.3)
    assert orc.eval_spline_3d(grid, Cu, 0.7, 5.0, 0.3) == inside
