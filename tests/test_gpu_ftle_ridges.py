"""CUDA FTLE / Cauchy-Green / percentile / ridge kernels against the golden
vectors and the CPU oracle."""
import numpy as np
import pytest
import torch

from conftest import apply_mask, reconstruct

pytestmark = pytest.mark.gpu


def test_ftle_golden(nb, golden, mask_dg):
    fm = golden["fm"].astype(np.float64)
    f = nb.ftle_grid_2D(fm, 8.0, 0.1, 0.1)
    assert np.allclose(f.astype(np.float32), golden["ftle"])
    fk = nb.ftle_grid_2D(fm, 8.0, 0.1, 0.1, mask=mask_dg)
    assert np.allclose(fk.astype(np.float32), apply_mask(golden["ftle"], mask_dg))


def test_C_eig_golden(nb, golden, mask_dg):
    fm = golden["fm"].astype(np.float64)
    ev, vec = nb.C_eig_2D(fm, 0.1, 0.1)
    C_exp = reconstruct(golden["Cevals"], golden["Cevecs"])
    assert np.allclose(reconstruct(ev.astype(np.float32), vec.astype(np.float32)), C_exp)
    evm, vecm = nb.C_eig_2D(fm, 0.1, 0.1, mask_dg)
    assert np.allclose(reconstruct(evm.astype(np.float32), vecm.astype(np.float32)),
                       apply_mask(C_exp, mask_dg))
    f = nb.ftle_from_eig(ev[..., 1], 8.0)
    assert np.allclose(f.astype(np.float32), golden["ftle"])


def _random_flowmap(nx, ny, seed=0):
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(np.linspace(0, 2, nx), np.linspace(0, 1, ny), indexing="ij")
    fm = np.stack([X + 0.05 * np.sin(7 * Y + 3 * X), Y + 0.05 * np.cos(5 * X)], -1)
    return fm + 1e-3 * rng.standard_normal(fm.shape)


@pytest.mark.parametrize("shape", [(3, 3), (5, 7), (257, 129), (1000, 37)])
def test_ftle_and_eig_parity(nb, orc, shape):
    nx, ny = shape
    fm = _random_flowmap(nx, ny)
    dx, dy = 2.0 / (nx - 1), 1.0 / (ny - 1)
    mask = np.random.default_rng(1).random((nx, ny)) < 0.1
    for m in (None, mask):
        f = nb.ftle_grid_2D(fm, -10.0, dx, dy, mask=m)
        of = orc.ftle_grid_2D(fm, -10.0, dx, dy, mask=m)
        # identical arithmetic up to the last bit of log()
        np.testing.assert_allclose(f, of, rtol=5e-16, atol=0)
        ev, vec = nb.C_eig_2D(fm, dx, dy, mask=m)
        oev, ovec = orc.C_eig_2D(fm, dx, dy, mask=m)
        assert np.array_equal(ev, oev) and np.array_equal(vec, ovec)
        # the fused entry point scales by reciprocals and normalises by a
        # reciprocal square root: within a few ulp of C_eig_2D + ftle_from_eig
        fe, ve = nb.ftle_evec_2D(fm, -10.0, dx, dy, mask=m)
        ofe = orc.ftle_from_eig(oev[..., 1], -10.0)
        # (the contract is 1e-5 relative where lambda_max > 1 + 1e-6; the
        # fused stencil's log takes its mantissa part in FP32: ~3e-7)
        nondeg = oev[..., 1] > 1.0 + 1e-6
        np.testing.assert_allclose(fe[nondeg], ofe[nondeg], rtol=1e-6, atol=0)
        assert np.abs(fe[~nondeg] - ofe[~nondeg]).max(initial=0.0) <= 1e-7
        assert np.all(fe[oev[..., 1] <= 1.0 - 1e-9] == 0.0)
        sep = oev[..., 1] - oev[..., 0] > 1e-6 * np.abs(oev[..., 1])
        np.testing.assert_allclose(ve[sep], ovec[..., :, 1][sep], rtol=0, atol=1e-12)
        assert np.array_equal(ve[oev[..., 1] == 0.0], ovec[..., :, 1][oev[..., 1] == 0.0])


@pytest.mark.parametrize("n", [1, 2, 3, 10, 1000, 169676, 1 << 20])
@pytest.mark.parametrize("q", [0.0, 0.5, 37.5, 90.0, 99.99, 100.0])
def test_percentile_bit_exact(nb, orc, n, q):
    from numbacs_gb300 import _device as D
    from numbacs_gb300 import _lib
    rng = np.random.default_rng(n)
    a = np.abs(rng.standard_normal(n))
    a[: n // 4] = 0.0  # the zero border / non-stretching region of an FTLE field
    if n > 10:
        a[n // 2: n // 2 + 7] = a[n // 2]  # ties inside
        a[-3:] = -a[-3:]
    rng.shuffle(a)
    t = torch.from_numpy(a).cuda()
    L = _lib.load()
    nbytes = L.nbcs_percentile_scratch_bytes(n)
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    _lib.check(L.nbcs_percentile(D.ptr(t), n, q, D.ptr(out), D.ptr(scratch), nbytes, D.stream_ptr()))
    got = out.item()
    exp = orc.percentile(a, q)
    assert got == exp or (np.isnan(got) and np.isnan(exp)), (got, exp)


def test_percentile_special_values(nb, orc):
    from numbacs_gb300 import _device as D
    from numbacs_gb300 import _lib
    L = _lib.load()
    cases = [np.array([1.0, np.nan, 3.0]), np.array([1.0, np.inf, 3.0]),
             np.array([-np.inf, 2.0, 3.0, 4.0]), np.array([-0.0, 0.0, -0.0, 1.0]),
             np.array([np.inf, -np.inf])]
    for a in cases:
        for q in (0.0, 50.0, 100.0):
            t = torch.from_numpy(a).cuda()
            sc = torch.empty(L.nbcs_percentile_scratch_bytes(len(a)), dtype=torch.uint8, device="cuda")
            out = torch.empty(1, dtype=torch.float64, device="cuda")
            _lib.check(L.nbcs_percentile(D.ptr(t), len(a), q, D.ptr(out), D.ptr(sc), sc.numel(),
                                         D.stream_ptr()))
            got, exp = out.item(), orc.percentile(a, q)
            assert got == exp or (np.isnan(got) and np.isnan(exp)), (a, q, got, exp)


def test_ridge_golden(nb, golden, coords_dg):
    x, y = coords_dg
    f = golden["ftle"].astype(np.float64)
    e = golden["Cevecs"][:, :, :, 1].astype(np.float64)
    rp = nb.ftle_ridge_pts(f, e, x, y)
    assert rp.shape == golden["ridge_pts"].shape and np.allclose(rp, golden["ridge_pts"])
    ridges = nb.ftle_ridges(f, e, x, y)
    assert len(ridges) == int(golden["n_ridges"])
    for k, r in enumerate(ridges):
        assert np.allclose(r, golden["ridges_%d" % k])


def _ridge_field(nx, ny, seed=0):
    x, y = np.linspace(0, 2, nx), np.linspace(0, 1, ny)
    fm = _random_flowmap(nx, ny, seed)
    return x, y, fm


@pytest.mark.parametrize("shape,pct,sdd", [((64, 32), 0, 0.0), ((676, 251), 90, 0.0),
                                           ((301, 157), 50, 1e-3), ((2001, 7), 90, 0.0),
                                           ((5, 5), 0, 0.0), ((4, 9), 90, 0.0)])
def test_ridge_mask_bit_identical(nb, orc, shape, pct, sdd):
    nx, ny = shape
    x, y, fm = _ridge_field(nx, ny)
    dx, dy = x[1] - x[0], y[1] - y[0]
    # both sides get the SAME FTLE field and eigenvectors
    oev, ovec = orc.C_eig_2D(fm, dx, dy)
    f = orc.ftle_from_eig(oev[..., 1], 5.0)
    e = np.ascontiguousarray(ovec[..., :, 1])
    r_pts, rb, _, _ = nb.extraction._ftle_ridges(f, e, x, y, sdd, pct)
    orp, orb, _ = orc.ridge_field(f, e, x, y, sdd, pct)
    assert np.array_equal(rb, orb)
    assert np.array_equal(r_pts, orp)
    pts = nb.ftle_ridge_pts(f, e, x, y, sdd, pct)
    assert np.array_equal(pts, orc.ftle_ridge_pts(f, e, x, y, sdd, pct))


@pytest.mark.parametrize("pct", [0, 60])
def test_ridge_threshold_special_values(nb, orc, pct):
    """The threshold test f > f_min on NaN, +-0, +-inf and values equal to the
    threshold: masks and points bit-identical to the oracle (the kernel
    compares bit patterns as integers)."""
    nx, ny = 48, 40
    x, y, fm = _ridge_field(nx, ny, seed=3)
    dx, dy = x[1] - x[0], y[1] - y[0]
    oev, ovec = orc.C_eig_2D(fm, dx, dy)
    f = orc.ftle_from_eig(oev[..., 1], 5.0)
    e = np.ascontiguousarray(ovec[..., :, 1])
    rng = np.random.default_rng(7)
    thr = 0.0 if pct == 0 else orc.percentile(f, pct)
    for v in (np.nan, 0.0, -0.0, np.inf, -np.inf, thr, np.nextafter(thr, np.inf),
              np.nextafter(thr, -np.inf)):
        idx = rng.integers(2, nx - 2, 12), rng.integers(2, ny - 2, 12)
        f[idx] = v
    r_pts, rb, _, _ = nb.extraction._ftle_ridges(f, e, x, y, 0.0, pct)
    orp, orb, _ = orc.ridge_field(f, e, x, y, 0.0, pct)
    assert np.array_equal(rb, orb)
    assert np.array_equal(r_pts, orp, equal_nan=True)


def test_ridge_compaction_large(nb):
    # size-independent properties at a large size: count == mask sum, the
    # compacted list is the row-major gather of the full array
    nx, ny = 4001, 2001
    x, y = torch.linspace(0, 2, nx, dtype=torch.float64, device="cuda"), torch.linspace(
        0, 1, ny, dtype=torch.float64, device="cuda")
    X, Y = torch.meshgrid(x, y, indexing="ij")
    f = torch.sin(40 * X) * torch.cos(23 * Y) + 0.5 * torch.sin(9 * X * Y)
    e = torch.stack([torch.cos(3 * Y), torch.sin(3 * Y)], -1).contiguous()
    full, rb, _, _ = nb.extraction._ftle_ridges(f, e, x, y, 0.0, 90)
    pts = nb.ftle_ridge_pts(f, e, x, y, 0.0, 90)
    assert pts.shape[0] == int(rb.sum())
    assert torch.equal(pts, full[rb.reshape(-1)])
    assert pts.shape[0] > 1000


@pytest.mark.parametrize("shape,density,seed", [((1, 1), 1.0, 0), ((7, 5), 0.5, 1),
                                                ((64, 33), 0.3, 2), ((301, 157), 0.12, 3),
                                                ((1000, 1000), 0.45, 4), ((4096, 3), 0.7, 5)])
def test_label8_matches_scipy(nb, shape, density, seed):
    from scipy.ndimage import generate_binary_structure, label
    from numbacs_gb300.extraction.ridges import label8
    m = np.random.default_rng(seed).random(shape) < density
    lab, n = label8(m)
    ref, nref = label(m, structure=generate_binary_structure(2, 2))
    assert n == nref
    assert np.array_equal(lab.cpu().numpy(), ref)
    # a spiral: one long component, worst case for path lengths
    s = np.zeros((64, 64), bool)
    s[0, :] = s[:, -1] = s[-1, 1:] = s[2:, 0] = s[2, :-2] = True
    lab, n = label8(s)
    assert n == nref_spiral(s) and np.array_equal(lab.cpu().numpy(), label(s, np.ones((3, 3)))[0])


def nref_spiral(s):
    from scipy.ndimage import label
    return label(s, np.ones((3, 3)))[1]


def test_ridges_large_field_groups(nb):
    # ridge grouping at a realistic size vs scipy on the GPU mask
    from scipy.ndimage import generate_binary_structure, label
    nx, ny = 676, 251
    x, y, fm = _ridge_field(nx, ny, seed=3)
    dx, dy = x[1] - x[0], y[1] - y[0]
    oev, ovec = orc_like_eig(fm, dx, dy)
    f = np.where(oev[..., 1] > 1, np.log(np.maximum(oev[..., 1], 1e-300)) / 10.0, 0.0)
    e = np.ascontiguousarray(ovec[..., :, 1])
    r_pts, rb, _, _ = nb.extraction._ftle_ridges(f, e, x, y, 0.0, 50)
    ridges = nb.ftle_ridges(f, e, x, y, 0.0, 50, min_ridge_pts=3)
    lab, nl = label(rb, structure=generate_binary_structure(2, 2))
    ind = np.arange(nx * ny).reshape(nx, ny)
    ref = [r_pts[ind[lab == k]] for k in range(1, nl + 1) if (lab == k).sum() >= 3]
    assert len(ridges) == len(ref) > 3
    for a, b in zip(ridges, ref):
        assert np.array_equal(a, b)


def orc_like_eig(fm, dx, dy):
    import oracle
    return oracle.C_eig_2D(fm, dx, dy)


def test_ordered_ridges_golden(nb, golden, coords_dg):
    """tests/test_extraction.py:22-28 through the drop-in (GPU ridge test)."""
    x, y = coords_dg
    f = golden["ftle"].astype(np.float64)
    e = np.ascontiguousarray(golden["Cevecs"][:, :, :, 1].astype(np.float64))
    ridges = nb.ftle_ordered_ridges(f, e, x, y, 0.1)
    n = int(golden["n_ordered"])
    assert len(ridges) == n
    for k in range(n):
        assert np.allclose(ridges[k], golden["ordered_%d" % k])


@pytest.mark.parametrize("pct", [0, 80])
def test_ordered_ridges_match_oracle_fed(nb, orc, pct):
    """A larger field: the GPU ridge test + native linking equal the oracle's
    ridge test + the oracle's restatement of the linking."""
    from oracle.ordered_ref import ordered_from_ridge_field
    nx, ny = 301, 157
    x, y, fm = _ridge_field(nx, ny, seed=5)
    dx, dy = x[1] - x[0], y[1] - y[0]
    oev, ovec = orc.C_eig_2D(fm, dx, dy)
    f = orc.ftle_from_eig(oev[..., 1], 5.0)
    e = np.ascontiguousarray(ovec[..., :, 1])
    ridges = nb.ftle_ordered_ridges(f, e, x, y, 3 * dx, percentile=pct)
    rpts, mask, _ = orc.ridge_field(f, e, x, y, 0.0, pct)
    ref = ordered_from_ridge_field(f, e, x, y, mask, rpts, 3 * dx)
    assert len(ridges) == len(ref) and len(ref) > 0
    for a, b in zip(ridges, ref):
        assert np.array_equal(a, b)


def test_stencil_golden_literals_gpu(nb, golden, coords_dg):
    """The reference's stencil literals (tests/test_utils.py) through the GPU
    C_eig_2D / C_eig_aux_2D kernels (the checks of test_oracle_golden.py)."""
    from test_oracle_golden import stencil_literal_checks
    stencil_literal_checks(nb.C_eig_2D, nb.C_eig_aux_2D, golden, coords_dg)
