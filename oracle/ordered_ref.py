"""Ordered FTLE ridges: restatement in Python of the reference's linking and
endpoint joining (src/numbacs/extraction/ridges.py:322-1054).

TEST INFRASTRUCTURE ONLY (the oracle): the product links ridge points with the
native nbcs_order_ridges (numbacs_gb300/csrc/ordered.cu); the tests check it
against this restatement and this restatement against the reference's
ordered_ridges.pkl fixture.

The ridge points are visited in increasing second directional derivative
(strongest ridges first) and each unvisited one grows a curve in both
directions (_linked_ridge_pts, ridges.py:419-603), stepping to the neighbour --
among the three grid neighbours facing the ridge tangent -- that minimises
distance / h + c * angle between normals (_link_points_stepper,
ridges.py:322-416); curves of one point are dropped.  Curves whose endpoints
lie within `dist_tol` with tangents within `ep_tan_ang` are then joined
(_endpoint_distances / _connect_endpoints, ridges.py:607-717), and joined
curves shorter than `min_ridge_pts` points are dropped
(ftle_ordered_ridges, ridges.py:720-1054).
"""
import math

import numpy as np

# grid neighbours in counter-clockwise order starting below-right (i+1, j-1);
# the first two repeat so that three consecutive entries exist for any start
_NEIGHBOURS = ((1, -1), (1, 0), (1, 1), (0, 1), (-1, 1), (-1, 0), (-1, -1), (0, -1), (1, -1), (1, 0))


def _acos(v):
    """acos with NaN outside [-1, 1] (a dot of unit vectors can round past 1)."""
    return math.acos(v) if -1.0 <= v <= 1.0 else math.nan


def _ridge_sdd(f, evec, k, ny, dx, dy):
    """Second directional derivative c2 at flat grid indices k: the kernel's
    FP64 expression (ridges.py:290-306), evaluated in the same order."""
    ff = np.asarray(f, np.float64).ravel()
    ev = np.asarray(evec, np.float64).reshape(-1, 2)
    fxx = (ff[k + ny] - 2.0 * ff[k] + ff[k - ny]) / (dx * dx)
    fyy = (ff[k + 1] - 2.0 * ff[k] + ff[k - 1]) / (dy * dy)
    fxy = (ff[k + ny + 1] - ff[k + ny - 1] - ff[k - ny + 1] + ff[k - ny - 1]) / (4.0 * dx * dy)
    ex, ey = ev[k, 0], ev[k, 1]
    return ex * (fxx * ex + fxy * ey) + ey * (fxy * ex + fyy * ey)


class _Linker:
    """Growth of curves through the ridge points (ridges.py:321-603)."""

    def __init__(self, rpts, rvecs, sdd, ny, h, c, sdd_thresh):
        self.rpts, self.rvecs, self.sdd = rpts, rvecs, sdd
        self.offsets = [i * ny + j for i, j in _NEIGHBOURS]
        self.a, self.c, self.sdd_thresh = 1.0 / h, c, sdd_thresh

    def step(self, pt, nvec, ind, ridge):
        """The next point of a curve from `pt` (index `ind`) along the tangent
        of normal `nvec`, or None; claims the point for `ridge`."""
        ang = math.atan2(nvec[0], -nvec[1]) % (2.0 * math.pi)
        sector = int(math.floor(ang * 4.0 / math.pi + 0.5)) % 8
        metric = np.full(3, 10000.0)
        cand, vecs, ks = np.zeros((3, 2)), np.zeros((3, 2)), [0, 0, 0]
        found = False
        for q in range(3):
            k = ind + self.offsets[sector + q]
            ks[q] = k
            cand[q] = self.rpts[k, :2]
            if self.sdd[k] + self.sdd_thresh < 0:
                d = ((cand[q, 0] - pt[0]) ** 2 + (cand[q, 1] - pt[1]) ** 2) ** 0.5
                n1 = self.rvecs[k]
                dot = nvec[0] * n1[0] + nvec[1] * n1[1]
                if dot < 0:
                    vecs[q] = -n1
                    dot = -dot
                else:
                    vecs[q] = n1
                metric[q] = self.a * d + self.c * _acos(dot)
                found = True
        if not found:
            return None
        q = int(np.argmin(metric))
        k = ks[q]
        if self.rpts[k, 2] + 0.5 < 0:
            self.rpts[k, 2] = ridge
            return cand[q].copy(), vecs[q].copy(), k
        return None

    def grow(self, start, nvec, ridge):
        pt, n, ind, far, pts = self.rpts[start, :2].copy(), nvec, start, None, []
        far = pt
        for _ in range(10000):
            nxt = self.step(pt, n, ind, ridge)
            if nxt is None:
                break
            pt, n, ind = nxt
            far = pt
            pts.append(pt)
        return pts, far


def _link(rpts, rvecs, sdd, order, ny, h, c, sdd_thresh):
    """Curves of linked ridge points: (points (m, 2) in curve order, per-curve
    (end index, length), endpoints (2n, 3) with the curve number k at the start
    and -(k + 0.1) at the end, unit tangents at the endpoints (2n, 2))."""
    lk = _Linker(rpts, rvecs, sdd, ny, h, c, sdd_thresh)
    pts, lens, eps, tans = [], [], [], []
    ridge = 0
    for si in order:
        if not rpts[si, 2] + 0.5 < 0:
            continue  # already on a curve
        if not sdd[si] < -sdd_thresh:
            break
        rpts[si, 2] = ridge
        fwd, ept0 = lk.grow(si, rvecs[si].copy(), ridge)
        bwd, ept1 = lk.grow(si, -rvecs[si].copy(), ridge)
        curve = fwd[::-1] + [rpts[si, :2].copy()] + bwd
        if len(curve) == 1:
            continue  # a lone point: dropped, its number reused, the point stays claimed
        t0 = curve[1] - ept0
        t0 = t0 / (t0[0] ** 2 + t0[1] ** 2) ** 0.5
        t1 = ept1 - curve[-2]
        t1 = t1 / (t1[0] ** 2 + t1[1] ** 2) ** 0.5
        pts.extend(curve)
        lens.append((len(pts), len(curve)))
        eps += [(ept0[0], ept0[1], float(ridge)), (ept1[0], ept1[1], -(ridge + 0.1))]
        tans += [t0, t1]
        ridge += 1
    return (np.array(pts, np.float64).reshape(-1, 2), np.array(lens, np.int64).reshape(-1, 2),
            np.array(eps, np.float64).reshape(-1, 3), np.array(tans, np.float64).reshape(-1, 2))


def _distances(pt, arr, tol):
    """Distances from pt to arr's points, the offsets (unit length where the
    distance is below tol) and the below-tol mask (ridges.py:606-644)."""
    tan = arr - pt
    dist = (tan[:, 0] ** 2 + tan[:, 1] ** 2) ** 0.5
    close = dist < tol
    with np.errstate(invalid="ignore", divide="ignore"):
        tan[close] = tan[close] / ((tan[close, 0] ** 2 + tan[close, 1] ** 2) ** 0.5)[:, None]
    return dist, tan, close


def _join(ep, tan, rem, rem_tan, ang_tol, tol):
    """Join the curve end `ep` (tangent `tan`) to the nearest remaining endpoint
    whose offset and tangent are both within ang_tol; returns the remaining
    endpoints without the joined curve, the joined endpoint's value, the
    joined curve's other end and its tangent (None when nothing joins)."""
    dist, off, close = _distances(ep[:2], rem[:, :2], tol)
    if close.any():
        sign = int(math.copysign(1, ep[2]))
        for _ in range(int(close.sum())):
            e = int(np.argmin(dist))
            new_sign = int(math.copysign(1, rem[e, 2]))
            o, nt = off[e], rem_tan[e]
            if (_acos(-sign * (o[0] * tan[0] + o[1] * tan[1])) < ang_tol
                    and _acos(new_sign * (nt[0] * o[0] + nt[1] * o[1])) < ang_tol):
                val = rem[e, 2]
                other = e + int(math.copysign(1, val))
                new_ep, new_tan = rem[other].copy(), rem_tan[other].copy()
                keep = np.ones(len(rem), bool)
                keep[[e, other]] = False
                return rem[keep], rem_tan[keep], val, new_ep, new_tan
            dist[e] = 10 * tol
    return rem, rem_tan, -1, None, tan


def _walk(val, ep, tan, rem, rem_tan, nridges, ang_tol, tol):
    """The chain of curves joined from endpoint `ep` (value `val`): the list of
    endpoint values, first -(val + 0.1) for the starting curve."""
    chain = [-(val + 0.1)]
    for _ in range(nridges):
        rem, rem_tan, joined, ep, tan = _join(ep, tan, rem, rem_tan, ang_tol, tol)
        if ep is None:
            break
        chain.append(joined)
    return chain, rem, rem_tan


def _assemble(chain, pts, lens):
    """Concatenate the curves of a chain; a negative entry runs backwards."""
    parts = []
    for v in chain:
        end, n = lens[int(round(abs(v)))]
        seg = pts[end - n:end]
        parts.append(seg[::-1] if v + 0.01 < 0 else seg)
    return np.concatenate(parts, axis=0)


def order_ridges(pts, lens, eps, tans, dist_tol, ep_tan_ang=math.pi / 4, min_ridge_pts=5):
    """Join linked curves at nearby endpoints (ridges.py:720-1054)."""
    rem, rem_tan = eps.copy(), tans.copy()
    nridges = len(eps) // 2
    ridges = []

    def length(chain):
        return int(sum(lens[int(round(abs(v)))][1] for v in chain))

    while rem.size > 0:
        cur, cur_tan = rem[:2].copy(), rem_tan[:2].copy()
        rem, rem_tan = rem[2:], rem_tan[2:]
        d0, _, c0 = _distances(cur[0, :2], rem[:, :2], dist_tol)
        d1, _, c1 = _distances(cur[1, :2], rem[:, :2], dist_tol)
        case = int(c0.any()) + 2 * int(c1.any())
        if case == 3:  # both ends have close endpoints: walk from the closer end first
            e = int(np.argmin([d0.min(), d1.min()]))
            chain0, rem, rem_tan = _walk(cur[e, 2], cur[e], cur_tan[e], rem, rem_tan, nridges,
                                         ep_tan_ang, dist_tol)
            e2 = e + int(math.copysign(1, cur[e, 2]))
            chain1, rem, rem_tan = _walk(cur[e2, 2], cur[e2], cur_tan[e2], rem, rem_tan, nridges,
                                         ep_tan_ang, dist_tol)
            if len(chain0) > 1 and len(chain1) > 1:
                chain = [-(v + 0.1) for v in chain0[::-1]] + chain1[1:]
            elif len(chain0) > 1:
                chain = chain0
            else:
                chain = chain1
            if len(chain0) + len(chain1) > 2:
                if length(chain) >= min_ridge_pts:
                    ridges.append(_assemble(chain, pts, lens))
                continue
        elif case in (1, 2):  # only one end (0 or 1) has close endpoints
            e = case - 1
            chain, rem, rem_tan = _walk(cur[e, 2], cur[e], cur_tan[e], rem, rem_tan, nridges,
                                        ep_tan_ang, dist_tol)
            if len(chain) > 1:
                if length(chain) >= min_ridge_pts:
                    ridges.append(_assemble(chain, pts, lens))
                continue
            if case == 1:  # the reference keeps this lone curve whatever its length
                end, n = lens[int(round(abs(chain[0])))]
                ridges.append(pts[end - n:end])
                continue
        else:
            chain = [cur[0, 2]]
        end, n = lens[int(round(abs(chain[0])))]
        if n >= min_ridge_pts:
            ridges.append(pts[end - n:end])
    return ridges


def ordered_from_ridge_field(f, eigvec_max, x, y, ridge_mask, r_pts, dist_tol,
                             ep_tan_ang=math.pi / 4, min_ridge_pts=5, sdd_thresh=0.0, c=1.0):
    """ftle_ordered_ridges from the ridge mask (nx, ny) and the full ridge-point
    array (nx * ny, 2) of the ridge test (host arrays)."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    nx, ny = np.shape(f)
    dx, dy = x[1] - x[0], y[1] - y[0]
    k = np.flatnonzero(np.asarray(ridge_mask).ravel())
    rpts = -np.ones((nx * ny, 3))
    rvecs = np.zeros((nx * ny, 2))
    sdd = np.zeros(nx * ny)
    if k.size:
        rpts[k, :2] = np.asarray(r_pts, np.float64).reshape(-1, 2)[k]
        rvecs[k] = np.asarray(eigvec_max, np.float64).reshape(-1, 2)[k]
        sdd[k] = _ridge_sdd(f, eigvec_max, k, ny, dx, dy)
    order = k[np.argsort(sdd[k], kind="stable")]
    pts, lens, eps, tans = _link(rpts, rvecs, sdd, order, ny, min(dx, dy), c, sdd_thresh)
    return order_ridges(pts, lens, eps, tans, dist_tol, ep_tan_ang, min_ridge_pts)
