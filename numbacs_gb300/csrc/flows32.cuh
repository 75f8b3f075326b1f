// FP32 device right-hand sides for the mixed-precision integrator.
//
// Same fields as flows64.cuh (double gyre flows.py:1146-1158, Bickley jet
// flows.py:1182-1213, tricubic spline flows.py:154-254) rewritten for the FP32
// pipe: sincospif instead of sin(pi*x), one expf for tanh/sech^2, FMA-friendly
// B-spline weights, FP32 coefficients interleaved (u, v) per node.
#pragma once

#include "nbcs_internal.cuh"

namespace nbcs {

struct ParamsF {
    float v[NBCS_MAX_PARAMS];
};

struct FlowDG32 {
    __device__ __forceinline__ void operator()(float t, const float* y, float* dy,
                                               const ParamsF& P) const
    {
        const float* p = P.v;
        float tt = p[0] * t;
        float a = p[2] * sinf(fmaf(p[4], tt, p[5]));
        float b = fmaf(-2.0f, a, 1.0f);
        float x0 = y[0];
        float f = fmaf(a, x0, b) * x0;
        float df = fmaf(2.0f * a, x0, b);
        float sf, cf, sy, cy;
        sincospif(f, &sf, &cf);
        sincospif(y[1], &sy, &cy);
        const float piA = 3.14159265358979f * p[1];
        dy[0] = p[0] * fmaf(-piA * sf, cy, -p[3] * x0);
        dy[1] = p[0] * fmaf(piA * cf * sy, df, -p[3] * y[1]);
    }
};

struct FlowBickley32 {
    __device__ __forceinline__ void operator()(float t, const float* y, float* dy,
                                               const ParamsF& P) const
    {
        const float* p = P.v;
        float tt = p[0] * t;
        float Y = y[1] / p[2];
        // tanh(Y) and sech^2(Y) from e = exp(-2|Y|): tanh = (1-e)/(1+e), sech^2 = 4e/(1+e)^2
        float e = __expf(-2.0f * fabsf(Y));
        float inv = 1.0f / (1.0f + e);
        float th = copysignf((1.0f - e) * inv, Y);
        float sech2 = 4.0f * e * inv * inv;
        float sn1, cs1, sn2, cs2, sn3, cs3;
        sincosf(p[6] * fmaf(-p[9], tt, y[0]), &sn1, &cs1);
        sincosf(p[7] * fmaf(-p[10], tt, y[0]), &sn2, &cs2);
        sincosf(p[8] * fmaf(-p[11], tt, y[0]), &sn3, &cs3);
        float cs = fmaf(p[3], cs1, fmaf(p[4], cs2, p[5] * cs3));
        float sn = fmaf(p[3] * p[6], sn1, fmaf(p[4] * p[7], sn2, p[5] * p[8] * sn3));
        dy[0] = p[0] * (p[1] * sech2 * fmaf(2.0f * th, cs, 1.0f));
        dy[1] = -p[0] * (p[1] * p[2] * sech2 * sn);
    }
};

struct SplineGridF {
    float a[3], b[3], dinv[3];
    int n[3];
    int sx, st;
};

inline SplineGridF make_grid_f(const double* g)
{
    SplineGridF s;
    for (int d = 0; d < 3; ++d) {
        s.a[d] = (float)g[3 * d];
        s.b[d] = (float)g[3 * d + 1];
        s.n[d] = (int)g[3 * d + 2];
        s.dinv[d] = (float)((double)(s.n[d] - 1) / (g[3 * d + 1] - g[3 * d]));
    }
    s.sx = s.n[2] + 2;
    s.st = (s.n[1] + 2) * (s.n[2] + 2);
    return s;
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

__device__ __forceinline__ int spline_locate32(const SplineGridF& g, int d, float x, float* t)
{
    x = fminf(fmaxf(x, g.a[d]), g.b[d]);  // extrap_mode "constant"
    float u = (x - g.a[d]) * g.dinv[d];
    int i = (int)floorf(u);
    i = max(0, min(i, g.n[d] - 2));
    *t = u - (float)i;
    return i;
}

__device__ __forceinline__ void spline_eval_uv32(const SplineGridF& g, const float2* __restrict__ c,
                                                 float t, float x, float y, float* u, float* v)
{
    float ft, fx, fy, wt[4], wx[4], wy[4];
    int it = spline_locate32(g, 0, t, &ft);
    int ix = spline_locate32(g, 1, x, &fx);
    int iy = spline_locate32(g, 2, y, &fy);
    bspline_w32(ft, wt);
    bspline_w32(fx, wx);
    bspline_w32(fy, wy);
    const float2* base = c + (size_t)it * g.st + (size_t)ix * g.sx + iy;
    float au = 0.0f, av = 0.0f;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        float su = 0.0f, sv = 0.0f;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const float2* row = base + (size_t)a * g.st + (size_t)b * g.sx;
            float2 r0 = __ldg(row), r1 = __ldg(row + 1), r2 = __ldg(row + 2), r3 = __ldg(row + 3);
            float bu = fmaf(wy[0], r0.x, fmaf(wy[1], r1.x, fmaf(wy[2], r2.x, wy[3] * r3.x)));
            float bv = fmaf(wy[0], r0.y, fmaf(wy[1], r1.y, fmaf(wy[2], r2.y, wy[3] * r3.y)));
            su = fmaf(wx[b], bu, su);
            sv = fmaf(wx[b], bv, sv);
        }
        au = fmaf(wt[a], su, au);
        av = fmaf(wt[a], sv, av);
    }
    *u = au;
    *v = av;
}

// Python float modulo in FP32.
__device__ __forceinline__ float py_fmodf(float a, float b)
{
    float m = fmodf(a, b);
    if (m != 0.0f && ((b < 0.0f) != (m < 0.0f))) m += b;
    return m;
}

template <int SPH>
struct FlowSpline32 {
    SplineGridF g;
    const float2* __restrict__ c;
    float deg_per_km;  // 180 / (pi r)

    __device__ __forceinline__ void operator()(float t, const float* y, float* dy,
                                               const ParamsF& P) const
    {
        const float* p = P.v;
        float tt = p[0] * t;
        float u, v;
        if (SPH == 1 || SPH == 2) {
            float xx = SPH == 1 ? py_fmodf(y[0] - 180.0f, 360.0f) - 180.0f : py_fmodf(y[0], 360.0f);
            float yy = y[1];
            spline_eval_uv32(g, c, tt, xx, yy, &u, &v);
            dy[0] = p[0] * u * deg_per_km / cospif(yy * (1.0f / 180.0f));
            dy[1] = p[0] * v * deg_per_km;
        } else {
            spline_eval_uv32(g, c, tt, y[0], y[1], &u, &v);
            dy[0] = p[0] * u;
            dy[1] = p[0] * v;
        }
    }
};

}  // namespace nbcs
