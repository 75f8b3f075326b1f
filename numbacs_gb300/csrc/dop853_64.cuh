// FP64 DOP853 for one particle with a 2-D state.
//
// The method is the Dormand-Prince 8(5,3) pair with Hairer & Wanner's dop853
// step-size controller, which is what the reference's numbalsoda.dop853
// (called at integration.py:169-171) runs: HINIT initial step, error norm
// err5^2/(err5^2 + 0.01 err3^2) scaling, safe = 0.9, fac1 = 0.333, fac2 = 6,
// beta = 0, uround = 2.3e-16, no step-size increase right after a rejection.
// Stage sums keep the published operand order and skip the zero tableau
// entries; compiled with -fmad=false so results match the CPU oracle.
#pragma once

#include "detmath.h"
#include "dop853_tableau.h"
#include "nbcs_internal.cuh"

namespace nbcs {

// Comparison-based min/max (a NaN operand propagates the same way as in the
// CPU oracle; fmin/fmax would drop it).
__device__ __forceinline__ double dmin_(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double dmax_(double a, double b) { return a > b ? a : b; }

struct Dop853Stats {
    int accepted, rejected, nfcn;
};

template <class Flow>
__device__ __forceinline__ double dop853_hinit64(const Flow& fl, const Params& P, double x,
                                                 const double* y, double posneg,
                                                 const double* f0, double hmax, double rtol,
                                                 double atol)
{
    double dnf = 0.0, dny = 0.0, sk, sqr, h, der2, der12, h1, y1[2], f1[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        sk = atol + rtol * fabs(y[i]);
        sqr = f0[i] / sk;
        dnf += sqr * sqr;
        sqr = y[i] / sk;
        dny += sqr * sqr;
    }
    if (dnf <= 1.0e-10 || dny <= 1.0e-10) h = 1.0e-6;
    else h = sqrt(dny / dnf) * 0.01;
    h = dmin_(h, hmax);
    h = posneg >= 0.0 ? fabs(h) : -fabs(h);
#pragma unroll
    for (int i = 0; i < 2; ++i) y1[i] = y[i] + h * f0[i];
    fl(x + h, y1, f1, P);
    der2 = 0.0;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        sk = atol + rtol * fabs(y[i]);
        sqr = (f1[i] - f0[i]) / sk;
        der2 += sqr * sqr;
    }
    der2 = sqrt(der2) / h;
    der12 = dmax_(fabs(der2), sqrt(dnf));
    if (der12 <= 1.0e-15) h1 = dmax_(1.0e-6, fabs(h) * 1.0e-3);
    else h1 = nbcs_root8(0.01 / der12);
    h = dmin_(100.0 * fabs(h), dmin_(h1, hmax));
    return posneg >= 0.0 ? fabs(h) : -fabs(h);
}

// Integrate y over solver time [x, xend].  Returns an NBCS_PARTICLE_* code.
template <class Flow>
__device__ int dop853_solve64(const Flow& fl, const Params& P, double x, double xend, double* y,
                              double rtol, double atol, int nmax, Dop853Stats* st)
{
    const double uround = 2.3e-16, safe = 0.9, facc1 = 1.0 / 0.333, facc2 = 1.0 / 6.0;
    double k1[2], k2[2], k3[2], k4[2], k5[2], k6[2], k7[2], k8[2], k9[2], k10[2], yy1[2];
    double facold = 1.0e-4;
    double posneg = (xend - x) >= 0.0 ? 1.0 : -1.0;
    double hmax, h, hnew, xph, err, err2, deno, fac, fac11, sk, erri, sqr;
    bool last = false, reject = false;
    int nstep = 0, status = NBCS_PARTICLE_OK;
    st->accepted = st->rejected = st->nfcn = 0;
    if (xend == x) return NBCS_PARTICLE_OK;

    fl(x, y, k1, P);
    hmax = fabs(xend - x);
    h = dop853_hinit64(fl, P, x, y, posneg, k1, hmax, rtol, atol);
    st->nfcn += 2;

    for (;;) {
        if (nstep > nmax) { status = NBCS_PARTICLE_MAX_STEPS; break; }
        if (0.1 * fabs(h) <= fabs(x) * uround) { status = NBCS_PARTICLE_STEP_UNDERFLOW; break; }
        if ((x + 1.01 * h - xend) * posneg > 0.0) {
            h = xend - x;
            last = true;
        }
        nstep++;
#pragma unroll
        for (int i = 0; i < 2; ++i) yy1[i] = y[i] + h * DP853_A_2_1 * k1[i];
        fl(x + DP853_C_2 * h, yy1, k2, P);
#pragma unroll
        for (int i = 0; i < 2; ++i) yy1[i] = y[i] + h * (DP853_A_3_1 * k1[i] + DP853_A_3_2 * k2[i]);
        fl(x + DP853_C_3 * h, yy1, k3, P);
#pragma unroll
        for (int i = 0; i < 2; ++i) yy1[i] = y[i] + h * (DP853_A_4_1 * k1[i] + DP853_A_4_3 * k3[i]);
        fl(x + DP853_C_4 * h, yy1, k4, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy1[i] = y[i] + h * (DP853_A_5_1 * k1[i] + DP853_A_5_3 * k3[i] + DP853_A_5_4 * k4[i]);
        fl(x + DP853_C_5 * h, yy1, k5, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy1[i] = y[i] + h * (DP853_A_6_1 * k1[i] + DP853_A_6_4 * k4[i] + DP853_A_6_5 * k5[i]);
        fl(x + DP853_C_6 * h, yy1, k6, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy1[i] = y[i] + h * (DP853_A_7_1 * k1[i] + DP853_A_7_4 * k4[i] + DP853_A_7_5 * k5[i]
                                 + DP853_A_7_6 * k6[i]);
        fl(x + DP853_C_7 * h, yy1, k7, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy1[i] = y[i] + h * (DP853_A_8_1 * k1[i] + DP853_A_8_4 * k4[i] + DP853_A_8_5 * k5[i]
                                 + DP853_A_8_6 * k6[i] + DP853_A_8_7 * k7[i]);
        fl(x + DP853_C_8 * h, yy1, k8, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy1[i] = y[i] + h * (DP853_A_9_1 * k1[i] + DP853_A_9_4 * k4[i] + DP853_A_9_5 * k5[i]
                                 + DP853_A_9_6 * k6[i] + DP853_A_9_7 * k7[i] + DP853_A_9_8 * k8[i]);
        fl(x + DP853_C_9 * h, yy1, k9, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy1[i] = y[i] + h * (DP853_A_10_1 * k1[i] + DP853_A_10_4 * k4[i] + DP853_A_10_5 * k5[i]
                                 + DP853_A_10_6 * k6[i] + DP853_A_10_7 * k7[i] + DP853_A_10_8 * k8[i]
                                 + DP853_A_10_9 * k9[i]);
        fl(x + DP853_C_10 * h, yy1, k10, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy1[i] = y[i] + h * (DP853_A_11_1 * k1[i] + DP853_A_11_4 * k4[i] + DP853_A_11_5 * k5[i]
                                 + DP853_A_11_6 * k6[i] + DP853_A_11_7 * k7[i] + DP853_A_11_8 * k8[i]
                                 + DP853_A_11_9 * k9[i] + DP853_A_11_10 * k10[i]);
        fl(x + DP853_C_11 * h, yy1, k2, P);
        xph = x + h;
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy1[i] = y[i] + h * (DP853_A_12_1 * k1[i] + DP853_A_12_4 * k4[i] + DP853_A_12_5 * k5[i]
                                 + DP853_A_12_6 * k6[i] + DP853_A_12_7 * k7[i] + DP853_A_12_8 * k8[i]
                                 + DP853_A_12_9 * k9[i] + DP853_A_12_10 * k10[i]
                                 + DP853_A_12_11 * k2[i]);
        fl(xph, yy1, k3, P);
        st->nfcn += 11;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            k4[i] = DP853_B_1 * k1[i] + DP853_B_6 * k6[i] + DP853_B_7 * k7[i] + DP853_B_8 * k8[i]
                    + DP853_B_9 * k9[i] + DP853_B_10 * k10[i] + DP853_B_11 * k2[i]
                    + DP853_B_12 * k3[i];
            k5[i] = y[i] + h * k4[i];
        }
        err = 0.0;
        err2 = 0.0;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            sk = atol + rtol * dmax_(fabs(y[i]), fabs(k5[i]));
            erri = k4[i] - DP853_BHH1 * k1[i] - DP853_BHH2 * k9[i] - DP853_BHH3 * k3[i];
            sqr = erri / sk;
            err2 += sqr * sqr;
            erri = DP853_E5_1 * k1[i] + DP853_E5_6 * k6[i] + DP853_E5_7 * k7[i] + DP853_E5_8 * k8[i]
                   + DP853_E5_9 * k9[i] + DP853_E5_10 * k10[i] + DP853_E5_11 * k2[i]
                   + DP853_E5_12 * k3[i];
            sqr = erri / sk;
            err += sqr * sqr;
        }
        deno = err + 0.01 * err2;
        if (deno <= 0.0) deno = 1.0;
        err = fabs(h) * err * sqrt(1.0 / (deno * 2.0));
        if (isnan(err)) { status = NBCS_PARTICLE_NONFINITE; break; }
        fac11 = nbcs_root8(err);  // err^(1/8)
        fac = fac11;  // beta = 0: the Lund stabilisation factor facold^beta is 1
        fac = dmax_(facc2, dmin_(facc1, fac / safe));
        hnew = h / fac;
        if (err <= 1.0) {
            facold = dmax_(err, 1.0e-4);
            st->accepted++;
            fl(xph, k5, k4, P);
            st->nfcn++;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                k1[i] = k4[i];
                y[i] = k5[i];
            }
            x = xph;
            if (last) break;
            if (fabs(hnew) > hmax) hnew = posneg * hmax;
            if (reject) hnew = posneg * dmin_(fabs(hnew), fabs(h));
            reject = false;
        } else {
            hnew = h / dmin_(facc1, fac11 / safe);
            reject = true;
            if (st->accepted >= 1) st->rejected++;
            last = false;
        }
        h = hnew;
    }
    (void)facold;
    return status;
}

}  // namespace nbcs
