"""Launch-shape autotuner for the integrators.

The persistent batched integrator's grid (blocks per SM) and the single-field
mixed integrator's lanes per particle / grid cap trade occupancy against
register and shared-memory use (stage derivatives take 96 B of shared memory
per thread; the spline RHS spends 64-96 registers per thread).  The
best point depends on the flow and the particle count, so it is measured:
each candidate is timed with CUDA events on the real workload, and the winner
is cached in ``_build/autotune.json`` keyed by GPU, precision, flow kinds and
a size bucket.
"""
import json
import math
import os
import threading

import torch

from . import _lib

_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")
_LOCK = threading.Lock()


def _load():
    try:
        with open(_CACHE) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(key, value):
    with _LOCK:
        data = _load()
        data[key] = value
        os.makedirs(os.path.dirname(_CACHE), exist_ok=True)
        tmp = _CACHE + ".tmp%d" % os.getpid()
        with open(tmp, "w") as fh:
            json.dump(data, fh, indent=1, sort_keys=True)
        os.replace(tmp, _CACHE)


def _gpu():
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return "%s-%dsm" % (p.name.replace(" ", "_"), p.multi_processor_count)


def _time(fn, reps=2):
    fn()  # warm-up
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


def tune_batch(batch, candidates=None, force=False):
    """Schedule for a prepared FTLEBatch (cached): blocks per SM of the
    persistent grid, -1 for one block per particle tile (mixed only), or -2
    for per-field launches on parallel streams."""
    if candidates is None:
        candidates = (2, 3, 4, 5, 6, 8, -2) + ((-1,) if batch.precision == "mixed" else ())
    kinds = sorted({(f.flow.kind, f.flow.spherical) for f in batch.fields})
    bucket = int(math.log2(max(1, batch.particles)))
    key = "batch/%s/%s/%s/%d" % (_gpu(), batch.precision, kinds, bucket)
    if not force:
        hit = _load().get(key)
        if hit is not None:
            batch.tuning = hit
            return hit["blocks_per_sm"]
    times = {}
    for c in candidates:
        times[c] = _time(lambda: batch.launch(blocks_per_sm=c))
    # within 2 % of the fastest, prefer the schedule with the fewest launches:
    # a persistent grid (one integrator launch), then per-class tile kernels
    # (one per flow class), then per-field launches
    fastest = min(times.values())
    launches = lambda c: 0 if c >= 0 else (1 if c == -1 else 2)  # noqa: E731
    best = min((c for c in times if times[c] <= 1.02 * fastest),
               key=lambda c: (launches(c), times[c]))
    batch.tuning = {"blocks_per_sm": best, "ms": times}
    _store(key, batch.tuning)
    return best


def tune_flowmap(flow, t0, T, x, y, params, rtol=1e-6, atol=1e-8, precision="mixed",
                 lanes=(1, 2, 4), blocks=(0,), force=False):
    """(lanes_per_particle, blocks_per_sm) for a single-field flow map (cached)."""
    from .integration import flowmap_grid_2D
    n = x.numel() * y.numel() if isinstance(x, torch.Tensor) else len(x) * len(y)
    key = "flowmap/%s/%s/%d-%d/%d" % (_gpu(), precision, flow.kind, flow.spherical,
                                      int(math.log2(max(1, n))))
    if not force:
        hit = _load().get(key)
        if hit is not None:
            return hit["lanes_per_particle"], hit["blocks_per_sm"]
    out = torch.empty((x.numel() if isinstance(x, torch.Tensor) else len(x),
                       y.numel() if isinstance(y, torch.Tensor) else len(y), 2),
                      dtype=torch.float64, device="cuda")
    lane_opts = lanes if flow.kind == _lib.FLOW_SPLINE2D and precision == "mixed" else (0,)
    times = {}
    for lp in lane_opts:
        for bps in blocks:
            times[(lp, bps)] = _time(lambda: flowmap_grid_2D(
                flow, t0, T, x, y, params, rtol=rtol, atol=atol, precision=precision, out=out,
                return_status=True, lanes_per_particle=lp, blocks_per_sm=bps))
    best = min(times, key=times.get)
    _store(key, {"lanes_per_particle": best[0], "blocks_per_sm": best[1],
                 "ms": {"%d/%d" % k: v for k, v in times.items()}})
    return best
