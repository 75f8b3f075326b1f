"""One FTLE field sharded over several GPUs: row blocks with halos.

The particles of flowmap_grid_2D are independent, so a field splits into
contiguous blocks of x rows, one per rank, with no exchange on the data path.
The stencils that follow need neighbours: the FTLE at row i reads the flow map
at rows i +- 1 and the ridge test at row i reads the FTLE at rows i +- 1, so a
rank integrates its block plus HALO = 2 rows on each side (redundantly with
its neighbours) and then owns exact FTLE values and ridge points for its own
rows.  The one global quantity is the ridge threshold, np.percentile of the
whole FTLE field (ridges.py:48-51): the owned FTLE rows (8 bytes per point)
are gathered once over the process group, every rank computes the same exact
percentile, and each extracts its rows' ridge points; gathering those in rank
order gives the single-GPU result bit for bit (row-major order is preserved
because the blocks are contiguous and in rank order).

Labelled ridges (``ftle_ridges``, ridges.py:186-229) shard the same way:
each rank labels the ridge mask of its own rows (8-connected), and a
component that crosses a block boundary is joined on the host: the last
owned row of rank r and the first of rank r + 1 are neighbours, so their
labels are united wherever two ridge pixels touch (|dj| <= 1).  Every rank
gathers the per-rank components (pixel indices and points) and builds the
same global list: components ordered by their first pixel in row-major order,
points in row-major order inside each, those with fewer than min_ridge_pts
points dropped -- the single-GPU result.

The compute goes through an ``ops`` object (flow map, FTLE + eigvec_max,
percentile, thresholded ridge points and mask, labels): :class:`GpuOps` is
the product path; a CPU object with the same methods lets the multi-process
logic run as gloo ranks without GPUs.
"""
import numpy as np

HALO = 2


def _all_gather_rows(a, group=None):
    """Every rank's array ``a`` (equal trailing shape, any number of rows),
    gathered in rank order with tensor collectives: the row counts, then the
    rows padded to the longest block.  CUDA tensors under NCCL, host tensors
    otherwise (gloo)."""
    import torch
    import torch.distributed as dist
    dev = (torch.device("cuda", torch.cuda.current_device())
           if dist.get_backend(group) == "nccl" else torch.device("cpu"))
    a = np.ascontiguousarray(a)
    world = dist.get_world_size(group)
    n = torch.tensor([a.shape[0]], dtype=torch.int64, device=dev)
    counts = [torch.empty_like(n) for _ in range(world)]
    dist.all_gather(counts, n, group=group)
    counts = [int(c.item()) for c in counts]
    buf = torch.zeros((max(counts),) + a.shape[1:], dtype=torch.from_numpy(a).dtype, device=dev)
    buf[:a.shape[0]] = torch.from_numpy(a).to(dev)
    outs = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(outs, buf, group=group)
    return [o[:c].cpu().numpy() for o, c in zip(outs, counts)]


def _gather_parts(part, group=None):
    """block_ridges of every rank, in rank order: each rank's components flattened
    to arrays (sizes, pixel indices, points) and its boundary rows, gathered
    with _all_gather_rows, then rebuilt."""
    comps = part["comps"]
    sizes = np.array([len(c[0]) for c in comps], np.int64)
    idx = np.concatenate([c[0] for c in comps]) if comps else np.zeros(0, np.int64)
    pts = np.concatenate([c[1] for c in comps]) if comps else np.zeros((0, 2))
    meta = np.array([part["rows"][0], part["rows"][1], part["ny"]], np.int64)
    edges = np.stack([np.asarray(part["top"], np.int64), np.asarray(part["bottom"], np.int64)])
    g = [_all_gather_rows(v, group) for v in (meta, sizes, idx.astype(np.int64),
                                              np.asarray(pts, np.float64), edges)]
    parts = []
    for meta_r, sizes_r, idx_r, pts_r, edges_r in zip(*g):
        cut = np.cumsum(np.concatenate([[0], sizes_r]))
        parts.append({"rows": (int(meta_r[0]), int(meta_r[1])), "ny": int(meta_r[2]),
                      "comps": [(idx_r[cut[k]:cut[k + 1]], pts_r[cut[k]:cut[k + 1]])
                                for k in range(len(sizes_r))],
                      "top": edges_r[0], "bottom": edges_r[1]})
    return parts


def row_blocks(nx, world):
    """Owned rows [i0, i1) of each rank: contiguous, in rank order, sizes
    differing by at most one."""
    if world < 1 or nx < world:
        raise ValueError("need 1 <= world <= nx")
    base, extra = divmod(nx, world)
    blocks, i0 = [], 0
    for r in range(world):
        i1 = i0 + base + (1 if r < extra else 0)
        blocks.append((i0, i1))
        i0 = i1
    return blocks


def extended_rows(i0, i1, nx, halo=HALO):
    """Rows a rank integrates: its block plus `halo` rows each side, clipped."""
    return max(0, i0 - halo), min(nx, i1 + halo)


class GpuOps:
    """The product path: the CUDA library through the drop-in functions."""

    def flowmap(self, flow, t0, T, x, y, params, **kw):
        from .integration import flowmap_grid_2D
        return flowmap_grid_2D(flow, t0, T, x, y, params, **kw)

    def ftle_evec(self, fm, T, dx, dy):
        from .diagnostics import ftle_evec_2D
        return ftle_evec_2D(fm, T, dx, dy)

    def percentile(self, f, q):
        from .extraction.ridges import percentile
        return percentile(f, q)

    def ridge_pts(self, f, evec, x, y, dx, dy, sdd_thresh, f_min):
        from .extraction.ridges import ridge_pts_fmin
        return ridge_pts_fmin(f, evec, x, y, dx, dy, sdd_thresh, f_min)

    def ridge_field(self, f, evec, x, y, dx, dy, sdd_thresh, f_min):
        """(ridge mask (n, ny) bool, r_pts (n * ny, 2)) with the threshold and
        spacing given."""
        from .extraction.ridges import _run
        _, _, mask, full = _run(f, evec, x, y, sdd_thresh, 0, True, True, f_min=f_min,
                                dxdy=(dx, dy))
        return mask.to(bool), full

    def label8(self, mask):
        from .extraction.ridges import label8
        return label8(mask)

    def to_numpy(self, a):
        return a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)


def block_ftle(ops, rank, world, flow, t0, T, x, y, params, **flowmap_kw):
    """Phase 1 on one rank: flow map, FTLE and eigvec_max of the rank's
    extended block.  Returns (state, owned FTLE rows as numpy)."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    nx = len(x)
    i0, i1 = row_blocks(nx, world)[rank]
    e0, e1 = extended_rows(i0, i1, nx)
    dx, dy = x[1] - x[0], y[1] - y[0]  # the global spacing (ridges.py:39-40)
    fm = ops.flowmap(flow, t0, T, x[e0:e1], y, params, **flowmap_kw)
    f, ev = ops.ftle_evec(fm, T, dx, dy)
    state = {"f": f, "ev": ev, "x": x[e0:e1], "y": y, "d": (dx, dy), "rows": (i0, i1, e0, e1)}
    return state, ops.to_numpy(f)[i0 - e0:i1 - e0]


def block_ridge_pts(ops, state, f_global, sdd_thresh=0.0, percentile=0):
    """Phase 2 on one rank: the global threshold from the whole FTLE field
    (0 when percentile == 0, as ridges.py:48-51) and the ridge points of the
    rank's rows (the extended block's 2-row border, which the stencil skips,
    is exactly its halo)."""
    f_min = 0.0 if percentile == 0 else ops.percentile(f_global, percentile)
    dx, dy = state["d"]
    pts = ops.ridge_pts(state["f"], state["ev"], state["x"], state["y"], dx, dy, sdd_thresh,
                        f_min)
    return ops.to_numpy(pts)


def sharded_ftle_ridge_pts(flow, t0, T, x, y, params, sdd_thresh=0.0, percentile=0, *,
                           group=None, ops=None, **flowmap_kw):
    """ftle_ridge_pts of the field's flow map, computed by every rank of the
    process group on its row block; every rank returns the full (k, 2) numpy
    array of ridge points, identical to the one-GPU pipeline
    flowmap_grid_2D -> ftle_evec_2D -> ftle_ridge_pts.  Collectives: tensor
    all_gathers of the owned FTLE rows and of the ridge points (each after a
    gather of the row counts)."""
    import torch.distributed as dist
    ops = ops or GpuOps()
    if dist.is_available() and dist.is_initialized():
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    else:
        rank, world = 0, 1
    state, owned = block_ftle(ops, rank, world, flow, t0, T, x, y, params, **flowmap_kw)
    rows = [owned] if world == 1 else _all_gather_rows(np.asarray(owned, np.float64), group)
    f_global = np.concatenate(rows, axis=0)
    pts = block_ridge_pts(ops, state, f_global, sdd_thresh, percentile)
    if world == 1:
        return pts
    return np.concatenate(_all_gather_rows(np.asarray(pts, np.float64), group), axis=0)


def block_ridges(ops, state, f_global, sdd_thresh=0.0, percentile=0):
    """Phase 2 of the labelled ridges on one rank: the global threshold, the
    ridge mask and points of the rank's own rows, their 8-connected labels.
    Returns {"rows": (i0, i1), "ny", "comps": [(flat pixel indices (global,
    row-major), points (m, 2))] in local label order, "top", "bottom": the
    labels of the first and last owned row}."""
    f_min = 0.0 if percentile == 0 else ops.percentile(f_global, percentile)
    dx, dy = state["d"]
    i0, i1, e0, e1 = state["rows"]
    mask, full = ops.ridge_field(state["f"], state["ev"], state["x"], state["y"], dx, dy,
                                 sdd_thresh, f_min)
    ny = len(state["y"])
    mask = ops.to_numpy(mask)[i0 - e0:i1 - e0]
    full = ops.to_numpy(full).reshape(e1 - e0, ny, 2)[i0 - e0:i1 - e0]
    lab, n = ops.label8(np.ascontiguousarray(mask))
    lab = ops.to_numpy(lab).astype(np.int64)
    flat = np.arange(i0, i1)[:, None] * ny + np.arange(ny)[None, :]
    sel = lab.ravel() > 0
    keys = lab.ravel()[sel]
    order = np.argsort(keys, kind="stable")  # row-major inside each label
    idx, pts = flat.ravel()[sel][order], full.reshape(-1, 2)[sel][order]
    bounds = np.searchsorted(keys[order], np.arange(1, n + 2))
    comps = [(idx[bounds[k]:bounds[k + 1]], pts[bounds[k]:bounds[k + 1]]) for k in range(n)]
    return {"rows": (i0, i1), "ny": ny, "comps": comps,
            "top": lab[0] if i1 > i0 else np.zeros(ny, np.int64),
            "bottom": lab[-1] if i1 > i0 else np.zeros(ny, np.int64)}


def merge_ridges(parts, min_ridge_pts=3):
    """Join the per-rank components (block_ridges of every rank, in rank
    order) across block boundaries: the global ftle_ridges list."""
    offs = np.cumsum([0] + [len(p["comps"]) for p in parts])
    parent = list(range(int(offs[-1])))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for r in range(len(parts) - 1):
        b, t = parts[r]["bottom"], parts[r + 1]["top"]
        ny = len(b)
        for j in np.nonzero(b)[0]:
            for jj in range(max(0, j - 1), min(ny, j + 2)):
                if t[jj]:
                    ra, rb = find(offs[r] + b[j] - 1), find(offs[r + 1] + t[jj] - 1)
                    if ra != rb:
                        parent[max(ra, rb)] = min(ra, rb)
    groups = {}
    for r, p in enumerate(parts):
        for k, comp in enumerate(p["comps"]):
            groups.setdefault(find(offs[r] + k), []).append(comp)
    out = []
    for members in groups.values():
        idx = np.concatenate([m[0] for m in members])
        pts = np.concatenate([m[1] for m in members])
        o = np.argsort(idx, kind="stable")
        out.append((idx[o[0]] if len(o) else 0, pts[o]))
    out.sort(key=lambda c: c[0])
    return [pts for _, pts in out if len(pts) >= min_ridge_pts]


def sharded_ftle_ridges(flow, t0, T, x, y, params, sdd_thresh=0.0, percentile=0,
                        min_ridge_pts=3, *, group=None, ops=None, **flowmap_kw):
    """ftle_ridges of the field's flow map (list of (m, 2) numpy arrays),
    computed by every rank on its row block and joined across the block
    boundaries; identical on every rank to the one-GPU pipeline
    flowmap_grid_2D -> ftle_evec_2D -> ftle_ridges.  Collectives: tensor
    all_gathers of the owned FTLE rows and of the per-rank components
    (_gather_parts)."""
    import torch.distributed as dist
    ops = ops or GpuOps()
    if dist.is_available() and dist.is_initialized():
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    else:
        rank, world = 0, 1
    state, owned = block_ftle(ops, rank, world, flow, t0, T, x, y, params, **flowmap_kw)
    rows = [owned] if world == 1 else _all_gather_rows(np.asarray(owned, np.float64), group)
    part = block_ridges(ops, state, np.concatenate(rows, axis=0), sdd_thresh, percentile)
    parts = [part] if world == 1 else _gather_parts(part, group)
    return merge_ridges(parts, min_ridge_pts)
