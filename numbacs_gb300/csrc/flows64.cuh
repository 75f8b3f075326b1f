// FP64 device right-hand sides.
//
// These restate the reference's numba @cfunc bodies operation for operation
// (same operand order, every + - * / separately rounded: this file is only
// compiled with -fmad=false), so that with the same inputs they produce the
// same doubles as the CPU oracle apart from the last-bit differences of the
// transcendental functions.
//
//   double gyre   flows.py:1146-1158
//   Bickley jet   flows.py:1182-1213
//   spline RHS    flows.py:154-254 (interpolation.eval_spline, k=3)
#pragma once

#include "detmath.h"
#include "nbcs_internal.cuh"

namespace nbcs {

#define NBCS_PI 3.141592653589793

struct FlowDG64 {
    __device__ __forceinline__ void operator()(double t, const double* y, double* dy,
                                               const Params& P) const
    {
        const double* p = P.v;
        double tt = p[0] * t;
        double a = p[2] * sin(p[4] * tt + p[5]);
        double b = 1.0 - 2.0 * a;
        double f = a * (y[0] * y[0]) + b * y[0];
        double df = 2.0 * a * y[0] + b;
        double sf, cf, sy, cy;
        sincos(NBCS_PI * f, &sf, &cf);
        sincos(NBCS_PI * y[1], &sy, &cy);
        dy[0] = p[0] * (-NBCS_PI * p[1] * sf * cy - p[3] * y[0]);
        dy[1] = p[0] * (NBCS_PI * p[1] * cf * sy * df - p[3] * y[1]);
    }
};

struct FlowBickley64 {
    __device__ __forceinline__ void operator()(double t, const double* y, double* dy,
                                               const Params& P) const
    {
        const double* p = P.v;
        double tt = p[0] * t;
        double Y = y[1] / p[2];
        double ch = cosh(Y);
        double sech2 = 1.0 / (ch * ch);
        double s1 = y[0] - p[9] * tt, s2 = y[0] - p[10] * tt, s3 = y[0] - p[11] * tt;
        double sn1, cs1, sn2, cs2, sn3, cs3;
        sincos(p[6] * s1, &sn1, &cs1);
        sincos(p[7] * s2, &sn2, &cs2);
        sincos(p[8] * s3, &sn3, &cs3);
        dy[0] = p[0] * (p[1] * sech2 + 2.0 * p[1] * tanh(Y) * sech2
                                           * (p[3] * cs1 + p[4] * cs2 + p[5] * cs3));
        dy[1] = -p[0] * (p[1] * p[2] * sech2
                         * (p[3] * p[6] * sn1 + p[4] * p[7] * sn2 + p[5] * p[8] * sn3));
    }
};

// Python's float modulo (sign of the divisor), as numba evaluates `%`.
__device__ __forceinline__ double py_fmod(double a, double b)
{
    double m = fmod(a, b);
    if (m != 0.0) {
        if ((b < 0.0) != (m < 0.0)) m += b;
    } else {
        m = copysign(0.0, b);
    }
    return m;
}

__device__ __forceinline__ void bspline_w64(double t, double* w)
{
    double t3 = t * t * t, t2 = t * t;
    w[0] = (-1.0 / 6.0) * t3 + (3.0 / 6.0) * t2 + (-3.0 / 6.0) * t + (1.0 / 6.0);
    w[1] = (3.0 / 6.0) * t3 + (-6.0 / 6.0) * t2 + (0.0 / 6.0) * t + (4.0 / 6.0);
    w[2] = (-3.0 / 6.0) * t3 + (3.0 / 6.0) * t2 + (3.0 / 6.0) * t + (1.0 / 6.0);
    w[3] = (1.0 / 6.0) * t3 + (0.0 / 6.0) * t2 + (0.0 / 6.0) * t + (0.0 / 6.0);
}

// derivative of the basis with respect to the offset t
__device__ __forceinline__ void bspline_dw64(double t, double* w)
{
    double t2 = t * t;
    w[0] = (-3.0 / 6.0) * t2 + (6.0 / 6.0) * t + (-3.0 / 6.0);
    w[1] = (9.0 / 6.0) * t2 + (-12.0 / 6.0) * t + (0.0 / 6.0);
    w[2] = (-9.0 / 6.0) * t2 + (6.0 / 6.0) * t + (3.0 / 6.0);
    w[3] = (3.0 / 6.0) * t2 + (0.0 / 6.0) * t + (0.0 / 6.0);
}

// Cell index and fractional offset along axis d of a coordinate on or inside
// [a, b]; a NaN coordinate takes cell 0 (and a NaN offset).
__device__ __forceinline__ int spline_locate64(const SplineGrid& g, int d, double x, double* t)
{
    double u = (x - g.a[d]) * g.dinv[d];
    double fu = floor(u);
    int i;
    if (fu > (double)(g.n[d] - 2)) i = g.n[d] - 2;
    else if (!(fu >= 0.0)) i = 0;
    else i = (int)fu;
    *t = u - (double)i;
    return i;
}

// sum_a w0[a] sum_b w1[b] sum_c w2[c] C[it+a, ix+b, iy+c] of the interleaved
// (u, v) coefficient block
__device__ __forceinline__ void spline_sum_uv64(const SplineGrid& g, const double2* __restrict__ c,
                                                int it, int ix, int iy, const double* w0,
                                                const double* w1, const double* w2, double* u,
                                                double* v)
{
    double au = 0.0, av = 0.0;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        double su = 0.0, sv = 0.0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const size_t e = (size_t)(it + a) * g.st + (size_t)(ix + b) * g.sx + iy;
            const double2* row = c + e;
            double2 r0 = make_double2(0.0, 0.0), r1 = r0, r2 = r0, r3 = r0;
            if (NBCS_CHECKED(e + 3 < (size_t)g.st * (size_t)(g.n[0] + 2),
                             NBCS_CHECK_SPLINE_GATHER)) {
                r0 = __ldg(row);
                r1 = __ldg(row + 1);
                r2 = __ldg(row + 2);
                r3 = __ldg(row + 3);
            }
            double bu = w2[0] * r0.x + w2[1] * r1.x + w2[2] * r2.x + w2[3] * r3.x;
            double bv = w2[0] * r0.y + w2[1] * r1.y + w2[2] * r2.y + w2[3] * r3.y;
            su += w1[b] * bu;
            sv += w1[b] * bv;
        }
        au += w0[a] * su;
        av += w0[a] * sv;
    }
    *u = au;
    *v = av;
}

// Tricubic evaluation of (u, v) at (t, x, y) with extrapolation mode XM, the
// extrap_mode of the interpolation package's eval_spline that the reference
// passes through (flows.py:121):
//   0 "constant": 0 strictly outside the grid box;
//   1 "nearest":  each coordinate clamped into its axis' [a, b];
//   2 "linear":   the value at the clamped point plus, for each clamped axis
//                 (t, x, y in that order), the derivative along that axis at
//                 the clamped point times the distance beyond the box.
template <int XM>
__device__ __forceinline__ void spline_eval_uv64(const SplineGrid& g, const double2* __restrict__ c,
                                                 double t, double x, double y, double* u,
                                                 double* v)
{
    if (XM == 0 && (t < g.a[0] || t > g.b[0] || x < g.a[1] || x > g.b[1] || y < g.a[2] ||
                    y > g.b[2])) {
        *u = 0.0;
        *v = 0.0;
        return;
    }
    const double vv[3] = {t, x, y};
    double dl[3], f[3], w[3][4];
    int i[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double cl = vv[d];
        if (XM != 0) cl = vv[d] < g.a[d] ? g.a[d] : (vv[d] > g.b[d] ? g.b[d] : vv[d]);
        dl[d] = vv[d] - cl;
        i[d] = spline_locate64(g, d, cl, &f[d]);
        bspline_w64(f[d], w[d]);
    }
    double au, av;
    spline_sum_uv64(g, c, i[0], i[1], i[2], w[0], w[1], w[2], &au, &av);
    if (XM == 2) {
#pragma unroll 1
        for (int d = 0; d < 3; ++d) {
            if (dl[d] == 0.0 || isnan(dl[d])) continue;
            double dw[4], gu, gv;
            bspline_dw64(f[d], dw);
            spline_sum_uv64(g, c, i[0], i[1], i[2], d == 0 ? dw : w[0], d == 1 ? dw : w[1],
                            d == 2 ? dw : w[2], &gu, &gv);
            const double s = dl[d] * g.dinv[d];
            au = au + s * gu;
            av = av + s * gv;
        }
    }
    *u = au;
    *v = av;
}

// XM: extrapolation mode (0 constant, 1 nearest, 2 linear)
template <int SPH, int XM = 0>
struct FlowSpline64 {
    SplineGrid g;
    const double2* __restrict__ c;
    double r;

    __device__ __forceinline__ void operator()(double t, const double* y, double* dy,
                                               const Params& P) const
    {
        const double* p = P.v;
        double tt = p[0] * t;
        double u, v;
        if (SPH == 1 || SPH == 2) {
            double xx = SPH == 1 ? py_fmod(y[0] - 180.0, 360.0) - 180.0 : py_fmod(y[0], 360.0);
            double yy = y[1];
            spline_eval_uv64<XM>(g, c, tt, xx, yy, &u, &v);
            dy[0] = p[0] * u * 180.0 / (NBCS_PI * r * nbcs_cos_deg(yy));
            dy[1] = p[0] * v * 180.0 / (NBCS_PI * r);
        } else {
            spline_eval_uv64<XM>(g, c, tt, y[0], y[1], &u, &v);
            dy[0] = p[0] * u;
            dy[1] = p[0] * v;
        }
    }
};

}  // namespace nbcs
