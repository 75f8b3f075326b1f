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
        for r in range(world):
            assert np.array_equal(np.load(out + ".%d.npy" % r), ref), r


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
