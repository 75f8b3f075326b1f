// Ordered FTLE ridges: linking of the ridge points into curves and joining of
// curves at nearby endpoints (host code; the ridge test itself runs on the GPU).
//
//   ftle_ordered_ridges   extraction/ridges.py:720-1054
//   _linked_ridge_pts     extraction/ridges.py:419-603 (curve growth)
//   _link_points_stepper  extraction/ridges.py:322-416 (one step of a curve)
//   _endpoint_distances   extraction/ridges.py:607-644
//   _connect_endpoints    extraction/ridges.py:647-717
//
// Serial by nature: the ridge points are visited in increasing second
// directional derivative and each decision depends on the points earlier
// decisions claimed.  The decision order, tie breaks (first minimum) and the
// floating-point expressions follow the reference; where Python evaluates a
// scalar power (x ** 2, x ** 0.5) the C library's pow is called, where numpy
// evaluates it on arrays (square, sqrt) the product and sqrt are used, so this
// code makes the decisions of the Python restatement bit for bit.  Compiled
// with -ffp-contract=off.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "nbcs_internal.cuh"

namespace nbcs {
namespace ordered {

constexpr double kPi = 3.141592653589793;

// grid neighbours counter-clockwise from below-right (i+1, j-1); the first two
// repeat so that three consecutive entries exist for any start sector
constexpr int kNbr[10][2] = {{1, -1}, {1, 0}, {1, 1}, {0, 1}, {-1, 1},
                             {-1, 0}, {-1, -1}, {0, -1}, {1, -1}, {1, 0}};

// acos with NaN outside [-1, 1] (Python's math.acos raises there; the
// restatement maps that to NaN, which then fails every "< tolerance" test)
static double acos_nan(double v) { return (v >= -1.0 && v <= 1.0) ? acos(v) : NAN; }

// Python float modulo: the result takes the sign of the (positive) divisor
static double py_mod(double a, double b)
{
    double m = fmod(a, b);
    if (m != 0.0) {
        if ((b < 0.0) != (m < 0.0)) m += b;
    } else {
        m = copysign(0.0, b);
    }
    return m;
}

// index of the first minimum; a NaN, if any, wins (numpy.argmin)
static int argmin_np(const double* v, int n)
{
    int best = 0;
    for (int i = 0; i < n; ++i) {
        if (v[i] != v[i]) return i;
        if (v[i] < v[best]) best = i;
    }
    return best;
}

struct Curves {
    std::vector<double> pts;      // (m, 2) points in curve order
    std::vector<int64_t> end;     // per curve: index one past its last point
    std::vector<int64_t> len;     // per curve: number of points
    std::vector<double> eps;      // (2n, 3): x, y, value (k at the start, -(k + 0.1) at the end)
    std::vector<double> tans;     // (2n, 2) unit tangents at the endpoints
};

struct Linker {
    double* rpts;         // (nx*ny, 3): x, y, ridge number (-1: free)
    const double* rvecs;  // (nx*ny, 2)
    const double* sdd;    // (nx*ny)
    long offsets[10];
    double a, c, sdd_thresh;

    // next point from pt (index ind) along the tangent of normal n; claims it
    bool step(double* pt, double* n, long* ind, double ridge)
    {
        double ang = py_mod(atan2(n[0], -n[1]), 2.0 * kPi);
        int sector = (int)floor(ang * 4.0 / kPi + 0.5);
        sector = ((sector % 8) + 8) % 8;
        double metric[3] = {10000.0, 10000.0, 10000.0};
        double cand[3][2] = {{0, 0}, {0, 0}, {0, 0}}, vecs[3][2] = {{0, 0}, {0, 0}, {0, 0}};
        long ks[3] = {0, 0, 0};
        bool found = false;
        for (int q = 0; q < 3; ++q) {
            long k = *ind + offsets[sector + q];
            ks[q] = k;
            cand[q][0] = rpts[3 * k];
            cand[q][1] = rpts[3 * k + 1];
            if (sdd[k] + sdd_thresh < 0.0) {
                double d = pow(pow(cand[q][0] - pt[0], 2.0) + pow(cand[q][1] - pt[1], 2.0), 0.5);
                double n1x = rvecs[2 * k], n1y = rvecs[2 * k + 1];
                double dot = n[0] * n1x + n[1] * n1y;
                if (dot < 0.0) {
                    vecs[q][0] = -n1x;
                    vecs[q][1] = -n1y;
                    dot = -dot;
                } else {
                    vecs[q][0] = n1x;
                    vecs[q][1] = n1y;
                }
                metric[q] = a * d + c * acos_nan(dot);
                found = true;
            }
        }
        if (!found) return false;
        int q = argmin_np(metric, 3);
        long k = ks[q];
        if (rpts[3 * k + 2] + 0.5 < 0.0) {
            rpts[3 * k + 2] = ridge;
            pt[0] = cand[q][0];
            pt[1] = cand[q][1];
            n[0] = vecs[q][0];
            n[1] = vecs[q][1];
            *ind = k;
            return true;
        }
        return false;
    }

    // grow a curve from `start` along normal (nx0, ny0): its points in order
    // and the far end (the start itself when nothing was added)
    void grow(long start, double nx0, double ny0, double ridge, std::vector<double>* out,
              double* far)
    {
        double pt[2] = {rpts[3 * start], rpts[3 * start + 1]}, n[2] = {nx0, ny0};
        long ind = start;
        far[0] = pt[0];
        far[1] = pt[1];
        for (int it = 0; it < 10000; ++it) {
            if (!step(pt, n, &ind, ridge)) break;
            far[0] = pt[0];
            far[1] = pt[1];
            out->push_back(pt[0]);
            out->push_back(pt[1]);
        }
    }
};

// the linked curves, strongest ridge points first
static void link(double* rpts, const double* rvecs, const double* sdd, const std::vector<long>& order,
                 long ny, double h, double c, double sdd_thresh, Curves* C)
{
    Linker L;
    L.rpts = rpts;
    L.rvecs = rvecs;
    L.sdd = sdd;
    for (int q = 0; q < 10; ++q) L.offsets[q] = (long)kNbr[q][0] * ny + kNbr[q][1];
    L.a = 1.0 / h;
    L.c = c;
    L.sdd_thresh = sdd_thresh;
    double ridge = 0.0;
    std::vector<double> fwd, bwd, curve;
    for (long si : order) {
        if (!(rpts[3 * si + 2] + 0.5 < 0.0)) continue;  // already on a curve
        if (!(sdd[si] < -sdd_thresh)) break;
        rpts[3 * si + 2] = ridge;
        double ept0[2], ept1[2];
        fwd.clear();
        bwd.clear();
        L.grow(si, rvecs[2 * si], rvecs[2 * si + 1], ridge, &fwd, ept0);
        L.grow(si, -rvecs[2 * si], -rvecs[2 * si + 1], ridge, &bwd, ept1);
        curve.clear();
        for (long p = (long)fwd.size() / 2 - 1; p >= 0; --p) {
            curve.push_back(fwd[2 * p]);
            curve.push_back(fwd[2 * p + 1]);
        }
        curve.push_back(rpts[3 * si]);
        curve.push_back(rpts[3 * si + 1]);
        curve.insert(curve.end(), bwd.begin(), bwd.end());
        const long m = (long)curve.size() / 2;
        if (m == 1) continue;  // a lone point: dropped, its number reused, the point stays claimed
        double t0x = curve[2] - ept0[0], t0y = curve[3] - ept0[1];
        double n0 = pow(pow(t0x, 2.0) + pow(t0y, 2.0), 0.5);
        double t1x = ept1[0] - curve[2 * (m - 2)], t1y = ept1[1] - curve[2 * (m - 2) + 1];
        double n1 = pow(pow(t1x, 2.0) + pow(t1y, 2.0), 0.5);
        C->pts.insert(C->pts.end(), curve.begin(), curve.end());
        C->end.push_back((int64_t)(C->pts.size() / 2));
        C->len.push_back(m);
        const double e0[3] = {ept0[0], ept0[1], ridge}, e1[3] = {ept1[0], ept1[1], -(ridge + 0.1)};
        C->eps.insert(C->eps.end(), e0, e0 + 3);
        C->eps.insert(C->eps.end(), e1, e1 + 3);
        const double tt[4] = {t0x / n0, t0y / n0, t1x / n1, t1y / n1};
        C->tans.insert(C->tans.end(), tt, tt + 4);
        ridge += 1.0;
    }
}

// remaining endpoints (values and tangents), in order
struct Endpoints {
    std::vector<double> e;  // (r, 3)
    std::vector<double> t;  // (r, 2)
    long size() const { return (long)e.size() / 3; }
    void erase2(long a, long b)  // remove entries a and b, keeping the order
    {
        if (a < b) std::swap(a, b);
        e.erase(e.begin() + 3 * a, e.begin() + 3 * a + 3);
        t.erase(t.begin() + 2 * a, t.begin() + 2 * a + 2);
        e.erase(e.begin() + 3 * b, e.begin() + 3 * b + 3);
        t.erase(t.begin() + 2 * b, t.begin() + 2 * b + 2);
    }
};

// distances from p to the remaining endpoints, offsets (unit where close) and
// the close mask (ridges.py:607-644; numpy array arithmetic)
static void distances(const double* p, const Endpoints& R, double tol, std::vector<double>* dist,
                      std::vector<double>* off, std::vector<char>* close)
{
    const long r = R.size();
    dist->resize(r);
    off->resize(2 * r);
    close->resize(r);
    for (long i = 0; i < r; ++i) {
        double tx = R.e[3 * i] - p[0], ty = R.e[3 * i + 1] - p[1];
        double d = sqrt(tx * tx + ty * ty);
        (*dist)[i] = d;
        (*close)[i] = d < tol;
        if (d < tol) {
            double nn = sqrt(tx * tx + ty * ty);
            tx = tx / nn;
            ty = ty / nn;
        }
        (*off)[2 * i] = tx;
        (*off)[2 * i + 1] = ty;
    }
}

// join the curve end ep (tangent tan) to the nearest remaining endpoint whose
// offset and tangent are both within ang_tol (ridges.py:647-717); on success
// removes that curve's two endpoints, sets *val to the joined endpoint's
// value and ep/tan to the joined curve's other end
static bool join(double* ep, double* tan, Endpoints* R, double ang_tol, double tol, double* val)
{
    std::vector<double> dist, off;
    std::vector<char> close;
    distances(ep, *R, tol, &dist, &off, &close);
    long nclose = 0;
    for (char cc : close) nclose += cc ? 1 : 0;
    if (nclose == 0) return false;
    const int sign = (int)copysign(1.0, ep[2]);
    for (long it = 0; it < nclose; ++it) {
        const long e = argmin_np(dist.data(), (int)dist.size());
        const int new_sign = (int)copysign(1.0, R->e[3 * e + 2]);
        const double ox = off[2 * e], oy = off[2 * e + 1];
        const double ntx = R->t[2 * e], nty = R->t[2 * e + 1];
        if (acos_nan(-sign * (ox * tan[0] + oy * tan[1])) < ang_tol &&
            acos_nan(new_sign * (ntx * ox + nty * oy)) < ang_tol) {
            *val = R->e[3 * e + 2];
            const long other = e + (long)copysign(1.0, *val);
            ep[0] = R->e[3 * other];
            ep[1] = R->e[3 * other + 1];
            ep[2] = R->e[3 * other + 2];
            tan[0] = R->t[2 * other];
            tan[1] = R->t[2 * other + 1];
            R->erase2(e, other);
            return true;
        }
        dist[e] = 10.0 * tol;
    }
    return false;
}

// the chain of curves joined from endpoint ep (value val): endpoint values,
// first -(val + 0.1) for the starting curve
static std::vector<double> walk(const double* ep0, const double* tan0, Endpoints* R, long nridges,
                                double ang_tol, double tol)
{
    std::vector<double> chain{-(ep0[2] + 0.1)};
    double ep[3] = {ep0[0], ep0[1], ep0[2]}, tan[2] = {tan0[0], tan0[1]};
    for (long it = 0; it < nridges; ++it) {
        double v;
        if (!join(ep, tan, R, ang_tol, tol, &v)) break;
        chain.push_back(v);
    }
    return chain;
}

static long curve_of(double v) { return (long)llround(fabs(v)); }

static int64_t chain_len(const std::vector<double>& chain, const Curves& C)
{
    int64_t n = 0;
    for (double v : chain) n += C.len[curve_of(v)];
    return n;
}

// append the curves of a chain (a negative entry runs backwards)
static void assemble(const std::vector<double>& chain, const Curves& C, std::vector<double>* out)
{
    for (double v : chain) {
        const long k = curve_of(v);
        const int64_t end = C.end[k], n = C.len[k];
        if (v + 0.01 < 0.0) {
            for (int64_t p = end - 1; p >= end - n; --p) {
                out->push_back(C.pts[2 * p]);
                out->push_back(C.pts[2 * p + 1]);
            }
        } else {
            out->insert(out->end(), C.pts.begin() + 2 * (end - n), C.pts.begin() + 2 * end);
        }
    }
}

struct Result {
    std::vector<double> pts;
    std::vector<int64_t> lens;
    void add(const std::vector<double>& p)
    {
        pts.insert(pts.end(), p.begin(), p.end());
        lens.push_back((int64_t)p.size() / 2);
    }
};

static void order_ridges(const Curves& C, double dist_tol, double ang_tol, int64_t min_pts,
                         Result* res)
{
    Endpoints R;
    R.e = C.eps;
    R.t = C.tans;
    const long nridges = (long)C.eps.size() / 6;
    std::vector<double> d0, d1, off;
    std::vector<char> c0, c1;
    std::vector<double> buf;
    while (R.size() > 0) {
        double cur[2][3], ct[2][2];
        for (int q = 0; q < 2; ++q) {
            for (int w = 0; w < 3; ++w) cur[q][w] = R.e[3 * q + w];
            for (int w = 0; w < 2; ++w) ct[q][w] = R.t[2 * q + w];
        }
        R.e.erase(R.e.begin(), R.e.begin() + 6);
        R.t.erase(R.t.begin(), R.t.begin() + 4);
        distances(cur[0], R, dist_tol, &d0, &off, &c0);
        distances(cur[1], R, dist_tol, &d1, &off, &c1);
        const bool any0 = std::any_of(c0.begin(), c0.end(), [](char v) { return v != 0; });
        const bool any1 = std::any_of(c1.begin(), c1.end(), [](char v) { return v != 0; });
        const int kase = (any0 ? 1 : 0) + (any1 ? 2 : 0);
        std::vector<double> chain;
        if (kase == 3) {  // both ends have close endpoints: walk from the closer end first
            double mins[2] = {d0[argmin_np(d0.data(), (int)d0.size())],
                              d1[argmin_np(d1.data(), (int)d1.size())]};
            const int e = argmin_np(mins, 2);
            std::vector<double> chain0 = walk(cur[e], ct[e], &R, nridges, ang_tol, dist_tol);
            const int e2 = e + (int)copysign(1.0, cur[e][2]);
            std::vector<double> chain1 = walk(cur[e2], ct[e2], &R, nridges, ang_tol, dist_tol);
            if (chain0.size() > 1 && chain1.size() > 1) {
                for (long q = (long)chain0.size() - 1; q >= 0; --q) chain.push_back(-(chain0[q] + 0.1));
                chain.insert(chain.end(), chain1.begin() + 1, chain1.end());
            } else if (chain0.size() > 1) {
                chain = chain0;
            } else {
                chain = chain1;
            }
            if (chain0.size() + chain1.size() > 2) {
                if (chain_len(chain, C) >= min_pts) {
                    buf.clear();
                    assemble(chain, C, &buf);
                    res->add(buf);
                }
                continue;
            }
        } else if (kase == 1 || kase == 2) {  // only one end has close endpoints
            const int e = kase - 1;
            chain = walk(cur[e], ct[e], &R, nridges, ang_tol, dist_tol);
            if (chain.size() > 1) {
                if (chain_len(chain, C) >= min_pts) {
                    buf.clear();
                    assemble(chain, C, &buf);
                    res->add(buf);
                }
                continue;
            }
            if (kase == 1) {  // the reference keeps this lone curve whatever its length
                const long k = curve_of(chain[0]);
                buf.assign(C.pts.begin() + 2 * (C.end[k] - C.len[k]), C.pts.begin() + 2 * C.end[k]);
                res->add(buf);
                continue;
            }
        } else {
            chain.assign(1, cur[0][2]);
        }
        const long k = curve_of(chain[0]);
        if (C.len[k] >= min_pts) {
            buf.assign(C.pts.begin() + 2 * (C.end[k] - C.len[k]), C.pts.begin() + 2 * C.end[k]);
            res->add(buf);
        }
    }
}

}  // namespace ordered
}  // namespace nbcs

using namespace nbcs;
using namespace nbcs::ordered;

extern "C" int nbcs_order_ridges(const double* f, const double* evec_max, const double* x,
                                 int32_t nx, const double* y, int32_t ny,
                                 const uint8_t* ridge_mask, const double* r_pts, double dist_tol,
                                 double ep_tan_ang, int64_t min_ridge_pts, double sdd_thresh,
                                 double c, double* pts_out, int64_t max_pts, int64_t* ridge_len_out,
                                 int64_t max_ridges, int64_t* n_pts, int64_t* n_ridges)
{
    NBCS_RANGE();
    if (nx < 3 || ny < 3 || !f || !evec_max || !x || !y || !ridge_mask || !r_pts || !n_pts ||
        !n_ridges)
        return set_error(NBCS_ERR_INVALID, "order_ridges: need nx, ny >= 3 and non-NULL arrays");
    const long n = (long)nx * ny;
    const double dx = x[1] - x[0], dy = y[1] - y[0];
    std::vector<double> rpts(3 * (size_t)n, -1.0), rvecs(2 * (size_t)n, 0.0), sdd((size_t)n, 0.0);
    std::vector<long> order;
    for (long k = 0; k < n; ++k) {
        if (!ridge_mask[k]) continue;
        const long i = k / ny, j = k - i * ny;
        if (i < 1 || i > nx - 2 || j < 1 || j > ny - 2) continue;  // no stencil (never a ridge point)
        rpts[3 * k] = r_pts[2 * k];
        rpts[3 * k + 1] = r_pts[2 * k + 1];
        rvecs[2 * k] = evec_max[2 * k];
        rvecs[2 * k + 1] = evec_max[2 * k + 1];
        // second directional derivative at k (ridges.py:290-306, same order)
        const double fxx = (f[k + ny] - 2.0 * f[k] + f[k - ny]) / (dx * dx);
        const double fyy = (f[k + 1] - 2.0 * f[k] + f[k - 1]) / (dy * dy);
        const double fxy = (f[k + ny + 1] - f[k + ny - 1] - f[k - ny + 1] + f[k - ny - 1]) / (4.0 * dx * dy);
        const double ex = evec_max[2 * k], ey = evec_max[2 * k + 1];
        sdd[k] = ex * (fxx * ex + fxy * ey) + ey * (fxy * ex + fyy * ey);
        order.push_back(k);
    }
    std::stable_sort(order.begin(), order.end(), [&](long a, long b) { return sdd[a] < sdd[b]; });
    Curves C;
    link(rpts.data(), rvecs.data(), sdd.data(), order, ny, dx < dy ? dx : dy, c, sdd_thresh, &C);
    Result res;
    order_ridges(C, dist_tol, ep_tan_ang, min_ridge_pts, &res);
    *n_pts = (int64_t)res.pts.size() / 2;
    *n_ridges = (int64_t)res.lens.size();
    if (*n_pts > max_pts || *n_ridges > max_ridges)
        return set_error(NBCS_ERR_SCRATCH, "order_ridges: output needs %lld points, %lld ridges",
                         (long long)*n_pts, (long long)*n_ridges);
    if (*n_pts && pts_out) std::copy(res.pts.begin(), res.pts.end(), pts_out);
    if (*n_ridges && ridge_len_out) std::copy(res.lens.begin(), res.lens.end(), ridge_len_out);
    return NBCS_OK;
}
