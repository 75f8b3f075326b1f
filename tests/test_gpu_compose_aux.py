"""Flow-map composition and the auxiliary-grid flow map / Cauchy-Green
eigen-decomposition on the GPU, through the C ABI: against the reference's
golden vectors (tests/test_integration.py:66-75, :92-114,
tests/test_diagnostics.py:112-131) and against the CPU oracle."""
import numpy as np
import pytest
import torch

from conftest import apply_mask, reconstruct

pytestmark = pytest.mark.gpu

T_FIX = 8.0
GRID_DG = ((0.0, 2.0, 21), (0.0, 1.0, 11))


def test_composition_initial_golden(nb, orc, golden, coords_dg):
    x, y = coords_dg
    dg, p, _ = nb.get_predefined_flow("double_gyre")
    fm0, fms, nT = nb.flowmap_composition_initial(dg, 0.0, T_FIX, 1.0, x, y,
                                                  nb.UCGrid(*GRID_DG), p)
    assert nT == 8 and fms.shape == (8, 21, 11, 2)
    assert np.allclose(fms.astype(np.float32), golden["fms_ci"])
    assert np.allclose(fm0.astype(np.float32), golden["fm_ci"])
    # the composition itself is bit-identical to the oracle's on the same maps
    assert np.array_equal(fm0, orc.flowmap_composition(fms, GRID_DG, 8))


def test_composition_step_golden(nb, golden, coords_dg):
    x, y = coords_dg
    dg, p, _ = nb.get_predefined_flow("double_gyre")
    fms = golden["fms_ci"].astype(np.float64)
    fmk, fms2 = nb.flowmap_composition_step(fms, dg, T_FIX, 1.0, 8, x, y, GRID_DG, p)
    assert fms2 is fms  # updated in place, as in the reference
    assert np.allclose(fmk.astype(np.float32), golden["fm_cs"])
    assert np.allclose(fms2.astype(np.float32), golden["fms_cs"])


def test_composition_step_torch_in_place(nb, golden, coords_dg):
    x, y = coords_dg
    dg, p, _ = nb.get_predefined_flow("double_gyre")
    fms = torch.from_numpy(golden["fms_ci"].astype(np.float64)).cuda()
    fmk, fms2 = nb.flowmap_composition_step(fms, dg, T_FIX, 1.0, 8, torch.from_numpy(x).cuda(),
                                            torch.from_numpy(y).cuda(), GRID_DG, p)
    assert fms2.data_ptr() == fms.data_ptr() and fmk.is_cuda
    assert np.allclose(fmk.cpu().numpy().astype(np.float32), golden["fm_cs"])
    assert np.allclose(fms.cpu().numpy().astype(np.float32), golden["fms_cs"])


@pytest.mark.parametrize("nT,first", [(1, 0), (2, 1), (5, 0), (5, 3), (9, 8)])
def test_compose_matches_oracle(nb, orc, nT, first):
    """Synthetic maps that push points outside the grid box (0 there) and a
    NaN, read in ring order: bit-identical to the oracle."""
    rng = np.random.default_rng(nT * 10 + first)
    nx, ny = 37, 23
    grid = ((-1.0, 3.0, nx), (0.5, 2.0, ny))
    X, Y = np.meshgrid(np.linspace(-1, 3, nx), np.linspace(0.5, 2, ny), indexing="ij")
    fms = np.empty((nT, nx, ny, 2))
    for k in range(nT):
        a = rng.uniform(-0.3, 0.3, 4)
        fms[k, ..., 0] = X + a[0] * np.sin(2 * Y + a[1]) + 0.05 * rng.standard_normal((nx, ny))
        fms[k, ..., 1] = Y + a[2] * np.cos(1.5 * X + a[3]) + 0.05 * rng.standard_normal((nx, ny))
    fms[first, 5, 7, 0] = np.nan  # the first map of the sequence
    gpu = nb.flowmap_composition(fms, grid, nT, first=first)
    cpu = orc.flowmap_composition(fms, grid, nT, first=first)
    assert np.array_equal(gpu, cpu, equal_nan=True)
    assert np.isnan(gpu[5, 7]).all()
    assert (gpu == 0.0).all(axis=-1).any()  # some points left the box


def test_compose_rejects_bad_grid(nb):
    fms = np.zeros((3, 4, 5, 2))
    with pytest.raises(ValueError):
        nb.flowmap_composition(fms, ((0.0, 1.0, 5), (0.0, 1.0, 5)), 3)
    with pytest.raises(ValueError):
        nb.flowmap_composition(fms, ((0.0, 1.0, 4), (0.0, 1.0, 5)), 2)


def _dg_close(gpu, cpu, extent):
    """The double gyre's only GPU/CPU difference is the last bit of sin/cos."""
    d = np.abs(gpu - cpu)
    assert d.max() <= 1e-6 * extent, d.max()
    assert np.median(d) <= 1e-12 * extent


def test_aux_grid_golden(nb, orc, golden, coords_dg, mask_dg):
    x, y = coords_dg
    dg, p, _ = nb.get_predefined_flow("double_gyre")
    fa, st = nb.flowmap_aux_grid_2D(dg, 0.0, T_FIX, x, y, p, return_status=True)
    assert fa.shape == (21, 11, 5, 2)
    assert np.allclose(fa.astype(np.float32), golden["fm_aux"])
    ref, sref, _ = orc.flowmap_aux_grid_2D(orc.double_gyre(), 0.0, T_FIX, x, y, p,
                                           return_status=True)
    assert np.array_equal(st, sref)
    _dg_close(fa, ref, 2.0)
    fam = nb.flowmap_aux_grid_2D(dg, 0.0, T_FIX, x, y, p, mask=mask_dg)
    assert np.allclose(fam.astype(np.float32), apply_mask(golden["fm_aux"], mask_dg))
    # the centre particles are the plain flow map (same FP64 solver, same start)
    fm = nb.flowmap_grid_2D(dg, 0.0, T_FIX, x, y, p)
    assert np.array_equal(fa[:, :, 4], fm)


@pytest.mark.parametrize("eig_main,compute_edge", [(False, True), (True, False), (False, False)])
def test_aux_grid_variants_match_oracle(nb, orc, coords_dg, eig_main, compute_edge):
    x, y = coords_dg
    dg, p, _ = nb.get_predefined_flow("double_gyre")
    fa, st = nb.flowmap_aux_grid_2D(dg, 0.0, 3.0, x, y, p, eig_main=eig_main,
                                    compute_edge=compute_edge, return_status=True)
    ref, sref, _ = orc.flowmap_aux_grid_2D(orc.double_gyre(), 0.0, 3.0, x, y, p,
                                           eig_main=eig_main, compute_edge=compute_edge,
                                           return_status=True)
    assert fa.shape == ref.shape and np.array_equal(st, sref)
    _dg_close(fa, ref, 2.0)


def test_aux_grid_spline_bit_identical(nb, orc):
    """Spherical spline flow, particles leaving the grid box (zero velocity
    outside): bit-identical to the oracle, counts included."""
    from numbacs_gb300 import workloads as W
    t, lon, lat = W.geo_grid()
    t, lon, lat = t[::4], lon[::4], lat[::4]
    _, _, _, U, V = W.geo_velocity(0, t=t, lon=lon, lat=lat, nmodes=64)
    grid, Cu, Cv = nb.get_interp_arrays_2D(t, lon, lat, U, V)
    fl = nb.get_flow_2D(grid, Cu, Cv, spherical=1)
    ofl = orc.spline_flow(grid, np.asarray(Cu), np.asarray(Cv), spherical=1)
    xs = np.linspace(lon[0], lon[-1], 23)
    ys = np.linspace(lat[0], lat[-1], 11)
    p = np.array([-1.0])
    fa, st = nb.flowmap_aux_grid_2D(fl, 180.0, -48.0, xs, ys, p, h=1e-3, return_status=True)
    ref, sref, _ = orc.flowmap_aux_grid_2D(ofl, 180.0, -48.0, xs, ys, p, h=1e-3,
                                           return_status=True)
    assert np.array_equal(st, sref)
    assert np.array_equal(fa, ref)
    # some trajectories leave the box and stop there
    inside = ((ref[..., 0] >= lon[0]) & (ref[..., 0] <= lon[-1]) & (ref[..., 1] >= lat[0])
              & (ref[..., 1] <= lat[-1]))
    assert not inside[sref == 0].all()


def test_C_eig_aux_golden_and_oracle(nb, orc, golden, mask_dg):
    fa = golden["fm_aux"].astype(np.float64)
    ev, vec = nb.C_eig_aux_2D(fa, 0.1, 0.1)
    C_exp = reconstruct(golden["Cevals_aux"], golden["Cevecs_aux"])
    assert np.allclose(reconstruct(ev.astype(np.float32), vec.astype(np.float32)), C_exp)
    oev, ovec = orc.C_eig_aux_2D(fa, 0.1, 0.1)
    assert np.array_equal(ev, oev) and np.array_equal(vec, ovec)
    evm, vecm = nb.C_eig_aux_2D(fa, 0.1, 0.1, mask=mask_dg)
    assert np.allclose(reconstruct(evm.astype(np.float32), vecm.astype(np.float32)),
                       apply_mask(C_exp, mask_dg))
    ev4, vec4 = nb.C_eig_aux_2D(fa[:, :, :4], 0.1, 0.1, eig_main=False)
    oev4, ovec4 = orc.C_eig_aux_2D(fa[:, :, :4], 0.1, 0.1, eig_main=False)
    assert np.array_equal(ev4, oev4) and np.array_equal(vec4, ovec4)
    with pytest.raises(ValueError):
        nb.C_eig_aux_2D(fa[:, :, :4], 0.1, 0.1)  # eig_main needs the centre particle


def test_C_tensor_golden_and_oracle(nb, orc, golden, mask_dg):
    """C_tensor_2D (diagnostics.py:69-111): the reference's C.npy, plain and
    masked, and bit-identical to the oracle (4 and 5 aux particles)."""
    fa = golden["fm_aux"].astype(np.float64)
    C = nb.C_tensor_2D(fa, 0.1, 0.1)
    assert np.allclose(C.astype(np.float32), golden["C"])
    assert np.array_equal(C, orc.C_tensor_2D(fa, 0.1, 0.1))
    Cm = nb.C_tensor_2D(fa, 0.1, 0.1, mask=mask_dg)
    assert np.allclose(Cm.astype(np.float32), apply_mask(golden["C"], mask_dg))
    assert np.array_equal(Cm, orc.C_tensor_2D(fa, 0.1, 0.1, mask=mask_dg))
    f4 = np.ascontiguousarray(fa[:, :, :4])
    assert np.array_equal(nb.C_tensor_2D(f4, 0.1, 0.1), orc.C_tensor_2D(f4, 0.1, 0.1))
