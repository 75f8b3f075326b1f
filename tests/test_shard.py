"""One field sharded over several ranks (numbacs_gb300/shard.py): the host
logic as gloo ranks on CPU (the oracle stands in for the GPU compute), and the
two phases with the CUDA kernels on one GPU."""
import os
import socket
import tempfile

import numpy as np
import pytest

from numbacs_gb300 import shard


class OracleOps:
    """The ops interface of shard.GpuOps, computed by the CPU oracle."""

    def __init__(self):
        import oracle
        oracle.build()
        self.o = oracle

    def flowmap(self, flow, t0, T, x, y, params, **kw):
        return self.o.flowmap_grid_2D(flow, t0, T, x, y, params, nthreads=1, **kw)

    def ftle_evec(self, fm, T, dx, dy):
        ev, vec = self.o.C_eig_2D(fm, dx, dy)
        return self.o.ftle_from_eig(ev[..., 1], T), np.ascontiguousarray(vec[..., :, 1])

    def percentile(self, f, q):
        return self.o.percentile(f, q)

    def ridge_pts(self, f, evec, x, y, dx, dy, sdd_thresh, f_min):
        return self.o.ridge_pts_fmin(f, evec, x, y, dx, dy, sdd_thresh, f_min)

    def ridge_field(self, f, evec, x, y, dx, dy, sdd_thresh, f_min):
        rpts, mask = self.o.ridge_field_fmin(f, evec, x, y, dx, dy, sdd_thresh, f_min)
        return mask, rpts

    def label8(self, mask):
        return self.o.label8(mask)

    def to_numpy(self, a):
        return np.asarray(a)


CASE = dict(t0=0.0, T=-6.0, nx=57, ny=23, percentile=80, sdd=0.0)


def _single(ops):
    import oracle
    x = np.linspace(0, 2, CASE["nx"])
    y = np.linspace(0, 1, CASE["ny"])
    p = oracle.double_gyre_params(-1.0)
    fm = ops.flowmap(oracle.double_gyre(), CASE["t0"], CASE["T"], x, y, p)
    f, ev = ops.ftle_evec(fm, CASE["T"], x[1] - x[0], y[1] - y[0])
    return oracle.ftle_ridge_pts(f, ev, x, y, CASE["sdd"], CASE["percentile"])


def _single_ridges(ops):
    import oracle
    x = np.linspace(0, 2, CASE["nx"])
    y = np.linspace(0, 1, CASE["ny"])
    p = oracle.double_gyre_params(-1.0)
    fm = ops.flowmap(oracle.double_gyre(), CASE["t0"], CASE["T"], x, y, p)
    f, ev = ops.ftle_evec(fm, CASE["T"], x[1] - x[0], y[1] - y[0])
    return oracle.ftle_ridges(f, ev, x, y, CASE["sdd"], CASE["percentile"], min_ridge_pts=3)


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    import oracle
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    try:
        x = np.linspace(0, 2, CASE["nx"])
        y = np.linspace(0, 1, CASE["ny"])
        pts = shard.sharded_ftle_ridge_pts(oracle.double_gyre(), CASE["t0"], CASE["T"], x, y,
                                           oracle.double_gyre_params(-1.0), CASE["sdd"],
                                           CASE["percentile"], ops=OracleOps())
        np.save(out_path + ".%d.npy" % rank, pts)
        ridges = shard.sharded_ftle_ridges(oracle.double_gyre(), CASE["t0"], CASE["T"], x, y,
                                           oracle.double_gyre_params(-1.0), CASE["sdd"],
                                           CASE["percentile"], 3, ops=OracleOps())
        np.savez(out_path + ".ridges.%d.npz" % rank, *ridges)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_row_blocks():
    for nx, world in [(10, 1), (10, 3), (57, 2), (57, 4), (8, 8)]:
        b = shard.row_blocks(nx, world)
        assert b[0][0] == 0 and b[-1][1] == nx
        assert all(b[r][1] == b[r + 1][0] for r in range(world - 1))
        sizes = [i1 - i0 for i0, i1 in b]
        assert max(sizes) - min(sizes) <= 1 and min(sizes) >= 1
        for i0, i1 in b:
            e0, e1 = shard.extended_rows(i0, i1, nx)
            assert e0 == max(0, i0 - 2) and e1 == min(nx, i1 + 2)
    with pytest.raises(ValueError):
        shard.row_blocks(3, 4)


def test_single_rank_equals_unsharded():
    pts = shard.sharded_ftle_ridge_pts(*_args(), ops=OracleOps())
    assert len(pts) > 0
    assert np.array_equal(pts, _single(OracleOps()))


def _args():
    import oracle
    oracle.build()
    return (oracle.double_gyre(), CASE["t0"], CASE["T"], np.linspace(0, 2, CASE["nx"]),
            np.linspace(0, 1, CASE["ny"]), oracle.double_gyre_params(-1.0), CASE["sdd"],
            CASE["percentile"])


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_ranks_match_single_process(world):
    """world gloo ranks on CPU, each its row block plus halos; the global
    percentile through the gathered FTLE rows: ridge points bit-identical to
    the unsharded pipeline, on every rank."""
    import torch.multiprocessing as mp
    ref = _single(OracleOps())
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "pts")
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        ref_ridges = _single_ridges(OracleOps())
        for r in range(world):
            assert np.array_equal(np.load(out + ".%d.npy" % r), ref), r
            got = np.load(out + ".ridges.%d.npz" % r)
            got = [got["arr_%d" % k] for k in range(len(got.files))]
            assert len(got) == len(ref_ridges), r
            assert all(np.array_equal(a, b) for a, b in zip(got, ref_ridges)), r


def test_ridge_merge_joins_components_across_blocks():
    """Components that cross block boundaries (also through several blocks and
    rejoining inside one) come out as the unsharded labelling's: order by
    first pixel, row-major points, the min_ridge_pts filter on the joined
    size."""
    import oracle
    ops = OracleOps()
    x = np.linspace(0, 2, CASE["nx"])
    y = np.linspace(0, 1, CASE["ny"])
    p = oracle.double_gyre_params(-1.0)
    fm = ops.flowmap(oracle.double_gyre(), CASE["t0"], CASE["T"], x, y, p)
    f, ev = ops.ftle_evec(fm, CASE["T"], x[1] - x[0], y[1] - y[0])
    ref = oracle.ftle_ridges(f, ev, x, y, CASE["sdd"], CASE["percentile"], min_ridge_pts=3)
    crossing = 0
    for world in (2, 3, 5, 8):
        blocks = shard.row_blocks(len(x), world)
        parts = []
        for r in range(world):
            st, _ = shard.block_ftle(ops, r, world, oracle.double_gyre(), CASE["t0"], CASE["T"], x,
                                     y, p)
            parts.append(shard.block_ridges(ops, st, f, CASE["sdd"], CASE["percentile"]))
        got = shard.merge_ridges(parts, 3)
        assert len(got) == len(ref) and all(np.array_equal(a, b) for a, b in zip(got, ref)), world
        rows = [np.searchsorted([b[1] for b in blocks], pt_rows, side="right")
                for pt_rows in [np.round((r[:, 0] - x[0]) / (x[1] - x[0])).astype(int) for r in ref]]
        crossing += sum(len(set(rw.tolist())) > 1 for rw in rows)
    assert crossing > 0  # the case has ridges that span blocks


@pytest.mark.gpu
def test_gpu_phases_match_one_gpu(nb):
    """The two phases with the CUDA kernels for three emulated ranks on one GPU
    (phase 1 of every rank, then phase 2 of every rank: no kernel waits on
    another) against the unsharded GPU pipeline: bit-identical."""
    x = np.linspace(0, 2, 301)
    y = np.linspace(0, 1, 151)
    dg, p, _ = nb.get_predefined_flow("double_gyre", int_direction=-1.0)
    fm = nb.flowmap_grid_2D(dg, 0.0, -8.0, x, y, p)
    f, e = nb.ftle_evec_2D(fm, -8.0, x[1] - x[0], y[1] - y[0])
    ref = nb.ftle_ridge_pts(f, e, x, y, 0.0, 85)
    ops = shard.GpuOps()
    world = 3
    states, rows = [], []
    for r in range(world):
        st, owned = shard.block_ftle(ops, r, world, dg, 0.0, -8.0, x, y, p)
        states.append(st)
        rows.append(owned)
    f_global = np.concatenate(rows)
    assert np.array_equal(f_global, f)
    pts = np.concatenate([shard.block_ridge_pts(ops, st, f_global, 0.0, 85) for st in states])
    assert len(pts) > 0 and np.array_equal(pts, ref)


@pytest.mark.gpu
def test_gpu_labelled_ridges_match_one_gpu(nb):
    """Labelled ridges with the CUDA kernels for four emulated ranks on one
    GPU (each phase of every rank in turn), joined across the block
    boundaries: the same list as the unsharded GPU ftle_ridges."""
    x = np.linspace(0, 2, 401)
    y = np.linspace(0, 1, 201)
    dg, p, _ = nb.get_predefined_flow("double_gyre", int_direction=-1.0)
    fm = nb.flowmap_grid_2D(dg, 0.0, -10.0, x, y, p)
    f, e = nb.ftle_evec_2D(fm, -10.0, x[1] - x[0], y[1] - y[0])
    ref = nb.ftle_ridges(f, e, x, y, 0.0, 90)
    ops = shard.GpuOps()
    world = 4
    states, rows = [], []
    for r in range(world):
        st, owned = shard.block_ftle(ops, r, world, dg, 0.0, -10.0, x, y, p)
        states.append(st)
        rows.append(owned)
    f_global = np.concatenate(rows)
    parts = [shard.block_ridges(ops, st, f_global, 0.0, 90) for st in states]
    got = shard.merge_ridges(parts, 3)
    assert len(got) == len(ref) > 0
    assert all(np.array_equal(a, b) for a, b in zip(got, ref))
