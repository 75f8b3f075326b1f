"""The allocation-free ridge entry point, called through the C ABI.

nbcs_ridge_pts_noalloc serves callers that cannot allocate device memory (a
plugin whose host program owns every cudaMalloc, or a caller with only a thin
FFI to this library): its scratch is a fixed array inside the library.  Its
results must equal those of nbcs_ridge_pts with caller-provided scratch, on
two calls in a row (the second finds the first call's leftovers in the shared
array), and it must refuse grids above its stated limit.

This file is named so that pytest collects it last.
"""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def _field(nx, ny, seed):
    x = torch.linspace(0.0, 2.0, nx, dtype=torch.float64, device="cuda")
    y = torch.linspace(0.0, 1.0, ny, dtype=torch.float64, device="cuda")
    X, Y = torch.meshgrid(x, y, indexing="ij")
    g = torch.Generator(device="cuda").manual_seed(seed)
    f = (torch.sin((7 + seed) * X) * torch.cos((5 + seed) * Y)
         + 0.1 * torch.rand((nx, ny), generator=g, dtype=torch.float64, device="cuda"))
    ang = 3.0 * Y + X
    e = torch.stack([torch.cos(ang), torch.sin(ang)], -1).contiguous()
    return f.contiguous(), e, x, y


def _outputs(nx, ny):
    return (torch.empty((nx, ny), dtype=torch.uint8, device="cuda"),
            torch.empty((nx * ny, 2), dtype=torch.float64, device="cuda"),
            torch.empty((nx * ny, 2), dtype=torch.float64, device="cuda"),
            torch.empty(1, dtype=torch.int64, device="cuda"))


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_scratch_entry_point(nb):
    from numbacs_gb300 import _lib
    L = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # calls in a row: the second finds the first call's leftovers in the
    # shared array; the third, on a smaller grid and without mask_out and
    # rpts_full, takes the library's internal mask (stale bytes of the larger
    # grids beyond its end) and the compaction that re-evaluates the ridge test
    cases = [(676, 251, 0, 90.0, 0.0, True), (301, 157, 1, 50.0, 1e-3, True),
             (157, 101, 2, 75.0, 0.0, False)]
    for nx, ny, seed, pct, sdd, full in cases:
        f, e, x, y = _field(nx, ny, seed)
        nbytes = L.nbcs_ridge_scratch_bytes(nx, ny)
        scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        m1, r1, p1, n1 = _outputs(nx, ny)
        m2, r2, p2, n2 = _outputs(nx, ny)
        p2.fill_(7.0)  # rows beyond the count are not part of the result
        a1 = (_p(m1), _p(r1)) if full else (None, None)
        a2 = (_p(m2), _p(r2)) if full else (None, None)
        _lib.check(L.nbcs_ridge_pts(_p(f), _p(e), _p(x), nx, _p(y), ny, sdd, pct, *a1, _p(p1),
                                    _p(n1), _p(scratch), nbytes, stream))
        _lib.check(L.nbcs_ridge_pts_noalloc(_p(f), _p(e), _p(x), nx, _p(y), ny, sdd, pct, *a2,
                                            _p(p2), _p(n2), stream))
        torch.cuda.synchronize()
        k = int(n1.item())
        assert k > 0 and int(n2.item()) == k
        assert torch.equal(p1[:k], p2[:k])
        if full:
            assert torch.equal(m1, m2)
            assert torch.equal(r1, r2)


def test_noalloc_rejects_grids_above_its_limit(nb):
    from numbacs_gb300 import _lib
    L = _lib.load()
    limit = 1 << 23
    nx, ny = 4097, 2048  # 8,390,656 points > limit
    assert nx * ny > limit
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = L.nbcs_ridge_pts_noalloc(_p(dummy), _p(dummy), _p(dummy), nx, _p(dummy), ny, 0.0, 0.0,
                                  None, None, _p(dummy), _p(cnt), None)
    assert rc == -1
    assert b"fixed scratch limit" in L.nbcs_last_error()
    assert L.nbcs_ridge_noalloc_scratch_bytes() >= limit
