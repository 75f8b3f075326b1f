// FP32 device right-hand sides for the mixed-precision integrator.
//
// Same fields as flows64.cuh (double gyre flows.py:1146-1158, Bickley jet
// flows.py:1182-1213, tricubic spline flows.py:154-254) evaluated on the FP32
// pipe.  Positions and times arrive as unevaluated pairs (hi, s) -- the
// particle's compensated coordinate plus the stage increment -- so that the
// spline can form its cell-local offsets to FP32 *relative* accuracy: an
// absolute coordinate rounded to one float (lon ~ 100 deg, t ~ 150 h) would
// carry ~4e-6 of absolute error into every velocity sample.
//
// The double gyre is written as sin(pi f) = -sinpi(w), w = f - 1 =
// a x (x - 2) + (x - 1), which is exactly +-1 on the invariant walls x = 0 and
// x = 2 (FP32 rounding of f = a x^2 + (1 - 2a) x would push wall particles into
// the unstable direction).
//
// The spline RHS can be evaluated cooperatively by a group of LP = 1, 2 or 4
// adjacent lanes that hold the same particle: lane q of the group sums 4/LP of
// the time levels of the 4x4x4 stencil and a butterfly of
// __shfl_xor_sync adds the partial sums, so every lane of the group ends with
// bit-identical velocities (float addition is commutative).
#pragma once

#include "nbcs_internal.cuh"

namespace nbcs {

struct ParamsF {
    float v[NBCS_MAX_PARAMS];
};

struct FlowDG32 {
    static constexpr int LP = 1;
    __device__ __forceinline__ void operator()(float th, float ts, const float* yh, const float* ys,
                                               float* dy, const ParamsF& P) const
    {
        const float* p = P.v;
        float tt = p[0] * (th + ts);
        float x = yh[0] + ys[0], y = yh[1] + ys[1];
        // x - 1, x - 2 and the reflected y from the pair (the hi-part
        // differences are exact near the walls) keep the sine arguments at
        // FP32 relative accuracy
        float xm1 = (yh[0] - 1.0f) + ys[0], xm2 = (yh[0] - 2.0f) + ys[0];
        float a = p[2] * sinf(fmaf(p[4], tt, p[5]));
        float b = fmaf(-2.0f, a, 1.0f);
        float w = fmaf(a * x, xm2, xm1);  // f - 1
        float df = fmaf(2.0f * a, x, b);
        float sw, cw, sy, cy;
        sincospif(w, &sw, &cw);  // sin(pi f) = -sw, cos(pi f) = -cw
        if (yh[1] > 0.5f) {      // sin(pi y) = sin(pi (1 - y)), cos(pi y) = -cos(pi (1 - y))
            sincospif((1.0f - yh[1]) - ys[1], &sy, &cy);
            cy = -cy;
        } else {
            sincospif(y, &sy, &cy);
        }
        const float piA = 3.14159265358979f * p[1];
        dy[0] = p[0] * fmaf(piA * sw, cy, -p[3] * x);
        dy[1] = p[0] * fmaf(-piA * cw * sy, df, -p[3] * y);
    }
};

struct FlowBickley32 {
    static constexpr int LP = 1;
    __device__ __forceinline__ void operator()(float th, float ts, const float* yh, const float* ys,
                                               float* dy, const ParamsF& P) const
    {
        const float* p = P.v;
        float tt = p[0] * (th + ts);
        float x = yh[0] + ys[0], y = yh[1] + ys[1];
        float Y = y / p[2];
        // tanh(Y) and sech^2(Y) from e = exp(-2|Y|): tanh = (1-e)/(1+e), sech^2 = 4e/(1+e)^2
        float e = __expf(-2.0f * fabsf(Y));
        float inv = 1.0f / (1.0f + e);
        float th_ = copysignf((1.0f - e) * inv, Y);
        float sech2 = 4.0f * e * inv * inv;
        float sn1, cs1, sn2, cs2, sn3, cs3;
        sincosf(p[6] * fmaf(-p[9], tt, x), &sn1, &cs1);
        sincosf(p[7] * fmaf(-p[10], tt, x), &sn2, &cs2);
        sincosf(p[8] * fmaf(-p[11], tt, x), &sn3, &cs3);
        float cs = fmaf(p[3], cs1, fmaf(p[4], cs2, p[5] * cs3));
        float sn = fmaf(p[3] * p[6], sn1, fmaf(p[4] * p[7], sn2, p[5] * p[8] * sn3));
        dy[0] = p[0] * (p[1] * sech2 * fmaf(2.0f * th_, cs, 1.0f));
        dy[1] = -p[0] * (p[1] * p[2] * sech2 * sn);
    }
};

// One spline axis: node k sits at a + k*d, with a, d and the far end b kept as
// float pairs (hi + lo) so node positions can be rebuilt to ~2^-48 relative
// accuracy and the box test is exact in its sign.
struct AxisF {
    float a_h, a_l, d_h, d_l, dinv, b_h, b_l;
    int n;
};

struct SplineGridF {
    AxisF ax[3];  // t, x, y
    int sx, st;   // node strides of the (nt+2, nx+2, ny+2) coefficient block
};

inline SplineGridF make_grid_f(const double* g)
{
    SplineGridF s;
    for (int d = 0; d < 3; ++d) {
        double a = g[3 * d], b = g[3 * d + 1];
        int n = (int)g[3 * d + 2];
        double dd = (b - a) / (double)(n - 1);
        AxisF& A = s.ax[d];
        A.a_h = (float)a;
        A.a_l = (float)(a - (double)A.a_h);
        A.d_h = (float)dd;
        A.d_l = (float)(dd - (double)A.d_h);
        A.dinv = (float)((double)(n - 1) / (b - a));
        A.b_h = (float)b;
        A.b_l = (float)(b - (double)A.b_h);
        A.n = n;
    }
    s.sx = s.ax[2].n + 2;
    s.st = (s.ax[1].n + 2) * (s.ax[2].n + 2);
    return s;
}

// True when every node a + k d of every axis of the grid tuple g (t0, t1, nt,
// x0, x1, nx, y0, y1, ny) is a float that fmaf(k, d_h, a_h) reproduces
// exactly, and so is every product k d_h -- dyadic spacings such as 3 h,
// 0.625 deg, 0.5 deg, 0.25 deg.  Then the compensated node sum of
// locate_pair has zero error terms and the one-FMA form gives the same bits.
// The check runs the device formulas in double (exact there for these
// magnitudes).
inline bool grid_nodes_exact_f(const double* g)
{
    for (int d = 0; d < 3; ++d) {
        double a = g[3 * d], b = g[3 * d + 1];
        int n = (int)g[3 * d + 2];
        double dd = (b - a) / (double)(n - 1);
        float a_h = (float)a, d_h = (float)dd;
        if ((double)a_h != a || (double)d_h != dd) return false;
        for (int k = 0; k < n; ++k) {
            double pk = (double)k * (double)d_h;
            double v = (double)a_h + pk;
            if ((double)(float)pk != pk || (double)(float)v != v || v != a + (double)k * dd)
                return false;
        }
    }
    return true;
}

// Cell index and offset t of the coordinate vh + vs on one axis.  The cell is
// picked from the rounded coordinate, the offset is formed from the pair
// (so t may sit a rounding error outside [0, 1] next to a knot, where the two
// cubic pieces agree).  A coordinate strictly outside [a, b] sets *outside.
// That test subtracts the ends as pairs -- the hi parts cancel exactly next
// to an end -- so its sign is the FP64 path's: a particle grid that
// overshoots the box by 1e-12 (np.arange end points) starts outside on both
// paths.  With extrapolation mode XM = 1 ("nearest") or 2 ("linear") an
// outside coordinate is clamped to the box (t = 0 or 1), and for XM = 2 *dl
// receives its distance beyond the box in cells of this axis.
// EXACT: the axis nodes are floats and fmaf(k, d_h, a_h) gives them exactly
// (AxisF::exact, checked on the host); the node position then needs no
// compensated sum, and the result is the same.
template <bool EXACT = false, int XM = 0>
__device__ __forceinline__ int locate_pair(const AxisF& A, float vh, float vs, float* t,
                                           bool* outside, float* dl = nullptr)
{
    float u = ((vh + vs) - A.a_h) * A.dinv;
    // NaN needs no branch: fmaxf picks cell 0 and the offset below is NaN
    const float top = (float)(A.n - 2);
    // floor of uc in [0, n - 2] (below 2^23) by the magic-number method:
    // adding 2^23 rounded toward -inf leaves 2^23 + floor(uc), whose low
    // mantissa bits are the cell index (full-rate adds instead of conversions)
    const float fl = __fadd_rd(fminf(fmaxf(u, 0.0f), top), 8388608.0f);
    const int i = __float_as_int(fl) - 0x4B000000;
    const float fi = fl - 8388608.0f;  // exact
    float s, lo;
    if (EXACT) {  // the node is a float: one FMA (same result as the sum below)
        s = fmaf(fi, A.d_h, A.a_h);
        lo = 0.0f;
    } else {
        // node position a + i*d as s + lo (exact product, two-sum on the hi parts)
        float p = __fmul_rn(fi, A.d_h);
        float e = fmaf(fi, A.d_h, -p);
        e = fmaf(fi, A.d_l, e);
        s = __fadd_rn(A.a_h, p);
        float bb = __fsub_rn(s, A.a_h);
        float err = __fadd_rn(__fsub_rn(A.a_h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
        lo = err + (e + A.a_l);
    }
    // vs - 0 is vs exactly: the exact-node form subtracts nothing
    float r = EXACT ? __fadd_rn(__fsub_rn(vh, s), vs)
                    : __fadd_rn(__fsub_rn(vh, s), __fsub_rn(vs, lo));
    *t = r * A.dinv;
    // one test for both end cells (i = 0 or n - 2): interior cells skip it
    if ((unsigned)(i - 1) >= (unsigned)(A.n - 3)) {
        if (i == 0) {
            const float ex = __fadd_rn(__fsub_rn(vh, A.a_h), __fsub_rn(vs, A.a_l));
            if (ex < 0.0f) {
                *outside = true;
                if (XM != 0) *t = 0.0f;
                if (XM == 2) *dl = ex * A.dinv;
            }
        }
        if (i == A.n - 2) {  // not "else": on a 2-node axis cell 0 holds both ends
            const float ex = __fadd_rn(__fsub_rn(vh, A.b_h), __fsub_rn(vs, A.b_l));
            if (ex > 0.0f) {
                *outside = true;
                if (XM != 0) *t = 1.0f;
                if (XM == 2) *dl = ex * A.dinv;
            }
        }
    }
    return i;
}

__device__ __forceinline__ void bspline_w32(float t, float* w)
{
    const float s = 1.0f / 6.0f;
    float u = 1.0f - t;
    float t2 = t * t;
    w[0] = s * u * u * u;
    w[1] = s * fmaf(fmaf(3.0f, t, -6.0f), t2, 4.0f);
    w[2] = s * fmaf(fmaf(fmaf(-3.0f, t, 3.0f), t, 3.0f), t, 1.0f);
    w[3] = s * t2 * t;
}

// Group-cooperative tricubic evaluation.  Coefficients use the "quad" layout:
// entry k (32 bytes, 32-byte aligned) holds (u_j, v_j) for j = k .. k+3, so the
// 4 y taps of a stencil row are ONE 256-bit load (ld.global.nc.v8.f32).  The
// gathers are what bounds this kernel (the L1 data stage, not DRAM: the
// coefficients stay in L2); against two 16-byte loads per row this halves the
// load requests and trims the L1 data wavefronts by ~9% (measured on the
// geophysical workload; the 2701 x 1001 field integrates ~7% faster).
// Work split of a lane group: lane q takes time levels q*4/LP .. (q+1)*4/LP - 1.
template <int LP>
struct SplineSplit {
    static constexpr int kLevels = 4 / LP;  // time levels per lane
    __device__ static int first_level(int q) { return q * kLevels; }
    // weight of this lane's r-th level from the four time weights w (selects
    // on the lane index, no lane-dependent polynomial coefficients)
    __device__ static float level_weight(const float* w, int q, int r)
    {
        if (LP == 1) return w[r];
        if (LP == 2) return q ? w[2 + r] : w[r];
        return q == 0 ? w[0] : q == 1 ? w[1] : q == 2 ? w[2] : w[3];
    }
};

// one stencil row: taps iy .. iy+3 of (u, v) from a quad entry
__device__ __forceinline__ void ldg_row8(const float* __restrict__ p, float* r)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]), "=f"(r[6]),
          "=f"(r[7])
        : "l"(p));
}

// Stencil row at quad entry e: one 256-bit load (in the checked build only
// when e lies inside the (nt+2)(nx+2)(ny+2)-entry block; zeros otherwise).
__device__ __forceinline__ void spline_row32(const SplineGridF& g, const float* __restrict__ c,
                                             unsigned e, float* p)
{
    if (NBCS_CHECKED(e < (unsigned)g.st * (unsigned)(g.ax[0].n + 2), NBCS_CHECK_SPLINE_GATHER)) {
        ldg_row8(c + 8 * (size_t)e, p);
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) p[k] = 0.0f;
    }
}

// w * (a.x, a.y) + (c.x, c.y) as one paired FP32 FMA (fma.rn.f32x2, sm_100 and
// later): each half rounds exactly as fmaf does, so a sum built from these is
// bit-identical to the same sum of scalar fmaf calls in the same order.
__device__ __forceinline__ float2 fma_pair(float w, float2 a, float2 c)
{
    return __ffma2_rn(make_float2(w, w), a, c);
}

template <int LP>
__device__ __forceinline__ void spline_eval_uv32(const SplineGridF& g, const float* __restrict__ c,
                                                 int it, int ix, int iy, float ft, const float* wx,
                                                 const float* wy, float* u, float* v)
{
    using S = SplineSplit<LP>;
    const int q = (LP > 1) ? (int)(threadIdx.x & (LP - 1)) : 0;
    const int a0 = S::first_level(q);  // first time level
    float wt4[4];
    bspline_w32(ft, wt4);
    // (u, v) contracted together: the quad layout interleaves u and v, so the
    // two halves of every tap are one register pair and one paired FMA
    float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int r = 0; r < S::kLevels; ++r) {
        const int a = a0 + r;
        const float wt = S::level_weight(wt4, q, r);
        // quad-entry index in 32 bits (flows with 2^32 entries or more are refused)
        const unsigned e0 = (unsigned)(it + a) * (unsigned)g.st + (unsigned)ix * (unsigned)g.sx +
                            (unsigned)iy;
        float2 s = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            float p[8];
            spline_row32(g, c, e0 + (unsigned)b * (unsigned)g.sx, p);
            float2 bb = __fmul2_rn(make_float2(wy[3], wy[3]), make_float2(p[6], p[7]));
            bb = fma_pair(wy[2], make_float2(p[4], p[5]), bb);
            bb = fma_pair(wy[1], make_float2(p[2], p[3]), bb);
            bb = fma_pair(wy[0], make_float2(p[0], p[1]), bb);
            s = fma_pair(wx[b], bb, s);
        }
        acc = fma_pair(wt, s, acc);
    }
    if (LP > 1) {
        const unsigned lane = threadIdx.x & 31u;
        const unsigned gmask = ((1u << LP) - 1u) << (lane & ~(unsigned)(LP - 1));
#pragma unroll
        for (int o = 1; o < LP; o <<= 1)
            acc = __fadd2_rn(acc, make_float2(__shfl_xor_sync(gmask, acc.x, o),
                                              __shfl_xor_sync(gmask, acc.y, o)));
    }
    *u = acc.x;
    *v = acc.y;
}

// derivative of the cubic B-spline basis with respect to the cell offset t
__device__ __forceinline__ void bspline_dw32(float t, float* d)
{
    float u = 1.0f - t;
    d[0] = -0.5f * u * u;
    d[1] = t * fmaf(1.5f, t, -2.0f);                  // (3t^2 - 4t) / 2
    d[2] = fmaf(t, fmaf(-1.5f, t, 1.0f), 0.5f);      // (-3t^2 + 2t + 1) / 2
    d[3] = 0.5f * t * t;
}

// Value and cell-offset derivatives of the tricubic (u, v): r = {u, v, du/dfx,
// du/dfy, dv/dfx, dv/dfy}, same group-cooperative split and butterfly as
// spline_eval_uv32.
template <int LP>
__device__ __forceinline__ void spline_eval_uv32_grad(const SplineGridF& g,
                                                      const float* __restrict__ c, int it, int ix,
                                                      int iy, float ft, const float* wx,
                                                      const float* wy, const float* dwx,
                                                      const float* dwy, float* r)
{
    using S = SplineSplit<LP>;
    const int q = (LP > 1) ? (int)(threadIdx.x & (LP - 1)) : 0;
    const int a0 = S::first_level(q);
    float wt4[4];
    bspline_w32(ft, wt4);
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int rr = 0; rr < S::kLevels; ++rr) {
        const int a = a0 + rr;
        const float wt = S::level_weight(wt4, q, rr);
        const unsigned e0 = (unsigned)(it + a) * (unsigned)g.st + (unsigned)ix * (unsigned)g.sx +
                            (unsigned)iy;
        float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            float p[8];
            spline_row32(g, c, e0 + (unsigned)b * (unsigned)g.sx, p);
            const float bu = fmaf(wy[0], p[0], fmaf(wy[1], p[2], fmaf(wy[2], p[4], wy[3] * p[6])));
            const float bv = fmaf(wy[0], p[1], fmaf(wy[1], p[3], fmaf(wy[2], p[5], wy[3] * p[7])));
            const float du = fmaf(dwy[0], p[0], fmaf(dwy[1], p[2], fmaf(dwy[2], p[4], dwy[3] * p[6])));
            const float dv = fmaf(dwy[0], p[1], fmaf(dwy[1], p[3], fmaf(dwy[2], p[5], dwy[3] * p[7])));
            s[0] = fmaf(wx[b], bu, s[0]);
            s[1] = fmaf(wx[b], bv, s[1]);
            s[2] = fmaf(dwx[b], bu, s[2]);
            s[3] = fmaf(wx[b], du, s[3]);
            s[4] = fmaf(dwx[b], bv, s[4]);
            s[5] = fmaf(wx[b], dv, s[5]);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) acc[k] = fmaf(wt, s[k], acc[k]);
    }
    if (LP > 1) {
        const unsigned lane = threadIdx.x & 31u;
        const unsigned gmask = ((1u << LP) - 1u) << (lane & ~(unsigned)(LP - 1));
#pragma unroll
        for (int o = 1; o < LP; o <<= 1)
#pragma unroll
            for (int k = 0; k < 6; ++k) acc[k] += __shfl_xor_sync(gmask, acc[k], o);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) r[k] = acc[k];
}

// Value plus first-order continuation beyond the box (extrapolation "linear"):
// u + sum_d dl[d] du/d(offset_d) at the clamped point, same for v, with dl in
// cells of each axis.  Same group split and butterfly as spline_eval_uv32;
// taken only by particles whose stage point left the grid box.
template <int LP>
__device__ __forceinline__ void spline_eval_uv32_lin(const SplineGridF& g, const float* __restrict__ c,
                                                  int it, int ix, int iy, float ft, float fx,
                                                  float fy, const float* dl, float* u, float* v)
{
    using S = SplineSplit<LP>;
    const int q = (LP > 1) ? (int)(threadIdx.x & (LP - 1)) : 0;
    const int a0 = S::first_level(q);
    float wt4[4], dwt4[4], wx[4], wy[4], dwx[4], dwy[4];
    bspline_w32(ft, wt4);
    bspline_dw32(ft, dwt4);
    bspline_w32(fx, wx);
    bspline_w32(fy, wy);
    bspline_dw32(fx, dwx);
    bspline_dw32(fy, dwy);
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // (u, v) x (value, d/dt, d/dx, d/dy)
#pragma unroll
    for (int rr = 0; rr < S::kLevels; ++rr) {
        const int a = a0 + rr;
        const float wt = S::level_weight(wt4, q, rr), dwt = S::level_weight(dwt4, q, rr);
        const unsigned e0 = (unsigned)(it + a) * (unsigned)g.st + (unsigned)ix * (unsigned)g.sx +
                            (unsigned)iy;
        float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // (u, v) x (value, d/dx, d/dy) at this level
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            float p[8];
            spline_row32(g, c, e0 + (unsigned)b * (unsigned)g.sx, p);
            const float bu = fmaf(wy[0], p[0], fmaf(wy[1], p[2], fmaf(wy[2], p[4], wy[3] * p[6])));
            const float bv = fmaf(wy[0], p[1], fmaf(wy[1], p[3], fmaf(wy[2], p[5], wy[3] * p[7])));
            const float du = fmaf(dwy[0], p[0], fmaf(dwy[1], p[2], fmaf(dwy[2], p[4], dwy[3] * p[6])));
            const float dv = fmaf(dwy[0], p[1], fmaf(dwy[1], p[3], fmaf(dwy[2], p[5], dwy[3] * p[7])));
            s[0] = fmaf(wx[b], bu, s[0]);
            s[1] = fmaf(wx[b], bv, s[1]);
            s[2] = fmaf(dwx[b], bu, s[2]);
            s[3] = fmaf(dwx[b], bv, s[3]);
            s[4] = fmaf(wx[b], du, s[4]);
            s[5] = fmaf(wx[b], dv, s[5]);
        }
        acc[0] = fmaf(wt, s[0], acc[0]);
        acc[1] = fmaf(wt, s[1], acc[1]);
        acc[2] = fmaf(dwt, s[0], acc[2]);
        acc[3] = fmaf(dwt, s[1], acc[3]);
        acc[4] = fmaf(wt, s[2], acc[4]);
        acc[5] = fmaf(wt, s[3], acc[5]);
        acc[6] = fmaf(wt, s[4], acc[6]);
        acc[7] = fmaf(wt, s[5], acc[7]);
    }
    if (LP > 1) {
        const unsigned lane = threadIdx.x & 31u;
        const unsigned gmask = ((1u << LP) - 1u) << (lane & ~(unsigned)(LP - 1));
#pragma unroll
        for (int o = 1; o < LP; o <<= 1)
#pragma unroll
            for (int k = 0; k < 8; ++k) acc[k] += __shfl_xor_sync(gmask, acc[k], o);
    }
    *u = fmaf(dl[2], acc[6], fmaf(dl[1], acc[4], fmaf(dl[0], acc[2], acc[0])));
    *v = fmaf(dl[2], acc[7], fmaf(dl[1], acc[5], fmaf(dl[0], acc[3], acc[1])));
}

// EXACT: all three axes have float nodes (AxisF::exact): the cell search skips
// the compensated node sums (same results).
// XM: extrapolation mode outside the grid box (0 "constant": zero velocity,
// 1 "nearest", 2 "linear"; the definitions of spline_eval_uv64).
template <int SPH, int LP_, bool EXACT = false, int XM = 0>
struct FlowSpline32 {
    static constexpr int LP = LP_;
    SplineGridF g;
    const float* __restrict__ c;  // quad layout, 32-byte aligned
    float deg_per_km;  // 180 / (pi r)

    __device__ __forceinline__ void operator()(float th, float ts, const float* yh, const float* ys,
                                               float* dy, const ParamsF& P) const
    {
        const float* p = P.v;
        const float p0 = p[0];
        float xh = yh[0];
        if (SPH == 1 || SPH == 2) {
            // lon wrap: ((x - 180) % 360) - 180 = x - 360 floor((x + 180) / 360)   (SPH 1)
            //           x % 360               = x - 360 floor(x / 360)             (SPH 2)
            float xv = yh[0] + ys[0];
            float k = floorf((SPH == 1 ? xv + 180.0f : xv) * (1.0f / 360.0f));
            xh = fmaf(-360.0f, k, xh);  // exact no-op for k = 0
        }
        float ft, fx, fy, wx[4], wy[4];
        float dl[3] = {0.0f, 0.0f, 0.0f};
        bool out = false;
        int it = locate_pair<EXACT, XM>(g.ax[0], p0 * th, p0 * ts, &ft, &out, dl);
        int ix = locate_pair<EXACT, XM>(g.ax[1], xh, ys[0], &fx, &out, dl + 1);
        int iy = locate_pair<EXACT, XM>(g.ax[2], yh[1], ys[1], &fy, &out, dl + 2);
        if (XM == 0 && out) {  // the lanes of a group agree: they hold the same particle
            dy[0] = 0.0f;
            dy[1] = 0.0f;
            return;
        }
        float u, v;
        if (XM == 2 && out) {
            spline_eval_uv32_lin<LP>(g, c, it, ix, iy, ft, fx, fy, dl, &u, &v);
        } else {
            bspline_w32(fx, wx);
            bspline_w32(fy, wy);
            spline_eval_uv32<LP>(g, c, it, ix, iy, ft, wx, wy, &u, &v);
        }
        if (SPH == 1 || SPH == 2) {
            float lat = yh[1] + ys[1];
            // approximate reciprocal (2 ulp): far inside the FP32 stage error
            dy[0] = __fdividef(p0 * u * deg_per_km, cospif(lat * (1.0f / 180.0f)));
            dy[1] = p0 * v * deg_per_km;
        } else {
            dy[0] = p0 * u;
            dy[1] = p0 * v;
        }
    }

    // RHS plus its spatial Jacobian J = d(dy)/d(x, y) (row-major 2x2), from
    // the derivative of the B-spline basis; the metric factor 1/cos(lat) of
    // the spherical modes is held fixed (its own derivative is left out).
    // Used for the learned step proposer's features.  Returns false (and zero
    // velocity and Jacobian) outside the grid box.
    __device__ __forceinline__ bool eval_grad(float th, float ts, const float* yh, const float* ys,
                                              float* dy, float* J, const ParamsF& P) const
    {
        const float p0 = P.v[0];
        float xh = yh[0];
        if (SPH == 1 || SPH == 2) {
            float xv = yh[0] + ys[0];
            float k = floorf((SPH == 1 ? xv + 180.0f : xv) * (1.0f / 360.0f));
            xh = fmaf(-360.0f, k, xh);  // exact no-op for k = 0
        }
        float ft, fx, fy, wx[4], wy[4], dwx[4], dwy[4], r[6];
        bool out = false;
        int it = locate_pair<EXACT>(g.ax[0], p0 * th, p0 * ts, &ft, &out);
        int ix = locate_pair<EXACT>(g.ax[1], xh, ys[0], &fx, &out);
        int iy = locate_pair<EXACT>(g.ax[2], yh[1], ys[1], &fy, &out);
        if (out) {
            dy[0] = dy[1] = 0.0f;
            J[0] = J[1] = J[2] = J[3] = 0.0f;
            return false;
        }
        bspline_w32(fx, wx);
        bspline_w32(fy, wy);
        bspline_dw32(fx, dwx);
        bspline_dw32(fy, dwy);
        spline_eval_uv32_grad<LP>(g, c, it, ix, iy, ft, wx, wy, dwx, dwy, r);
        float kx = p0, ky = p0;
        if (SPH == 1 || SPH == 2) {
            float lat = yh[1] + ys[1];
            kx = p0 * deg_per_km / cospif(lat * (1.0f / 180.0f));
            ky = p0 * deg_per_km;
        }
        const float gx = g.ax[1].dinv, gy = g.ax[2].dinv;
        dy[0] = kx * r[0];
        dy[1] = ky * r[1];
        J[0] = kx * r[2] * gx;  // du/dx
        J[1] = kx * r[3] * gy;  // du/dy
        J[2] = ky * r[4] * gx;  // dv/dx
        J[3] = ky * r[5] * gy;  // dv/dy
        return true;
    }
};

}  // namespace nbcs
