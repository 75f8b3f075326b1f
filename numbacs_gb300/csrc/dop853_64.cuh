// FP64 DOP853 for one particle with a 2-D state.
//
// The method is the Dormand-Prince 8(5,3) pair with Hairer & Wanner's dop853
// step-size controller, which is what the reference's numbalsoda.dop853
// (called at integration.py:169-171) runs: HINIT initial step, error norm
// err5^2/(err5^2 + 0.01 err3^2) scaling, safe = 0.9, fac1 = 0.333, fac2 = 6,
// beta = 0, uround = 2.3e-16, no step-size increase right after a rejection.
//
// Arithmetic: every stage sum keeps the published operand order (ascending
// stage index, zero tableau entries skipped, stage 2 as (h*a21)*k1) and the
// file is compiled with -fmad=false, so results match the CPU oracle bit for
// bit apart from the library transcendentals of the analytic flows.
//
// Code shape: the twelve stages run as one rolled loop (the right-hand side is
// instantiated once per solver, not twelve times -- the unrolled form was
// instruction-fetch bound); stage derivatives live in this thread's column of
// shared memory and the tableau in constant memory.  The derivative at the new
// point after an accepted step (FSAL) is the next step's stage 0.
#pragma once

#include "detmath.h"
#include "dop853_tableau.h"
#include "nbcs_internal.cuh"

namespace nbcs {

constexpr int kThreads64 = 128;

static __constant__ double kA64[12][12] = {
    {0.0},
    {DP853_A_2_1},
    {DP853_A_3_1, DP853_A_3_2},
    {DP853_A_4_1, DP853_A_4_2, DP853_A_4_3},
    {DP853_A_5_1, DP853_A_5_2, DP853_A_5_3, DP853_A_5_4},
    {DP853_A_6_1, DP853_A_6_2, DP853_A_6_3, DP853_A_6_4, DP853_A_6_5},
    {DP853_A_7_1, DP853_A_7_2, DP853_A_7_3, DP853_A_7_4, DP853_A_7_5, DP853_A_7_6},
    {DP853_A_8_1, DP853_A_8_2, DP853_A_8_3, DP853_A_8_4, DP853_A_8_5, DP853_A_8_6, DP853_A_8_7},
    {DP853_A_9_1, DP853_A_9_2, DP853_A_9_3, DP853_A_9_4, DP853_A_9_5, DP853_A_9_6, DP853_A_9_7,
     DP853_A_9_8},
    {DP853_A_10_1, DP853_A_10_2, DP853_A_10_3, DP853_A_10_4, DP853_A_10_5, DP853_A_10_6,
     DP853_A_10_7, DP853_A_10_8, DP853_A_10_9},
    {DP853_A_11_1, DP853_A_11_2, DP853_A_11_3, DP853_A_11_4, DP853_A_11_5, DP853_A_11_6,
     DP853_A_11_7, DP853_A_11_8, DP853_A_11_9, DP853_A_11_10},
    {DP853_A_12_1, DP853_A_12_2, DP853_A_12_3, DP853_A_12_4, DP853_A_12_5, DP853_A_12_6,
     DP853_A_12_7, DP853_A_12_8, DP853_A_12_9, DP853_A_12_10, DP853_A_12_11},
};
static __constant__ double kC64[12] ={0.0, DP853_C_2, DP853_C_3, DP853_C_4, DP853_C_5, DP853_C_6,
                                DP853_C_7, DP853_C_8, DP853_C_9, DP853_C_10, DP853_C_11, 1.0};
static __constant__ double kB64[12] ={DP853_B_1, DP853_B_2, DP853_B_3, DP853_B_4, DP853_B_5, DP853_B_6,
                                DP853_B_7, DP853_B_8, DP853_B_9, DP853_B_10, DP853_B_11,
                                DP853_B_12};
static __constant__ double kE5_64[12] ={DP853_E5_1, DP853_E5_2, DP853_E5_3, DP853_E5_4,
                                  DP853_E5_5, DP853_E5_6, DP853_E5_7, DP853_E5_8,
                                  DP853_E5_9, DP853_E5_10, DP853_E5_11, DP853_E5_12};

// Comparison-based min/max (a NaN operand propagates the same way as in the
// CPU oracle; fmin/fmax would drop it).
__device__ __forceinline__ double dmin_(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double dmax_(double a, double b) { return a > b ? a : b; }

struct Dop853Stats {
    int accepted, rejected, nfcn;
};

// Dense output (numbalsoda.dop853 with a t_eval grid: dop853's contd8 and its
// three extra stages) after the accepted step [xold, xold + h] from y0 to y1:
// stages k1, k6..k12 in slots 0, 5..11 of kc, the derivative at the end in
// slot 12; the extra stages go to slots 13..15.  Writes the interpolant at
// every due output time teval[*m] (up to the step's end) to dout[*m].
template <class Flow, int KS>
__device__ void dense_output64(const Flow& fl, const Params& P, double xold, double h,
                               const double* y0, const double* y1, double2* kc,
                               const double* __restrict__ teval, int n, int* m, double posneg,
                               double2* __restrict__ dout)
{
    double k[17][2];  // 1-based stages (only 1, 6..16 are used)
#pragma unroll
    for (int j = 6; j <= 13; ++j) {
        const double2 v = kc[(j - 1) * KS];
        k[j][0] = v.x;
        k[j][1] = v.y;
    }
    {
        const double2 v = kc[0];
        k[1][0] = v.x;
        k[1][1] = v.y;
    }
    double yy[2], kk[2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
        yy[i] = y0[i] + h * (DP853_A_14_1 * k[1][i] + DP853_A_14_7 * k[7][i]
                             + DP853_A_14_8 * k[8][i] + DP853_A_14_9 * k[9][i]
                             + DP853_A_14_10 * k[10][i] + DP853_A_14_11 * k[11][i]
                             + DP853_A_14_12 * k[12][i] + DP853_A_14_13 * k[13][i]);
    fl(xold + DP853_C_14 * h, yy, kk, P);
    k[14][0] = kk[0];
    k[14][1] = kk[1];
#pragma unroll
    for (int i = 0; i < 2; ++i)
        yy[i] = y0[i] + h * (DP853_A_15_1 * k[1][i] + DP853_A_15_6 * k[6][i]
                             + DP853_A_15_7 * k[7][i] + DP853_A_15_8 * k[8][i]
                             + DP853_A_15_11 * k[11][i] + DP853_A_15_12 * k[12][i]
                             + DP853_A_15_13 * k[13][i] + DP853_A_15_14 * k[14][i]);
    fl(xold + DP853_C_15 * h, yy, kk, P);
    k[15][0] = kk[0];
    k[15][1] = kk[1];
#pragma unroll
    for (int i = 0; i < 2; ++i)
        yy[i] = y0[i] + h * (DP853_A_16_1 * k[1][i] + DP853_A_16_6 * k[6][i]
                             + DP853_A_16_7 * k[7][i] + DP853_A_16_8 * k[8][i]
                             + DP853_A_16_9 * k[9][i] + DP853_A_16_13 * k[13][i]
                             + DP853_A_16_14 * k[14][i] + DP853_A_16_15 * k[15][i]);
    fl(xold + DP853_C_16 * h, yy, kk, P);
    k[16][0] = kk[0];
    k[16][1] = kk[1];
    double F[7][2];
#define NBCS_DENSE_ROW(r)                                                                      \
    (DP853_D_##r##_1 * k[1][i] + DP853_D_##r##_6 * k[6][i] + DP853_D_##r##_7 * k[7][i]       \
     + DP853_D_##r##_8 * k[8][i] + DP853_D_##r##_9 * k[9][i] + DP853_D_##r##_10 * k[10][i]   \
     + DP853_D_##r##_11 * k[11][i] + DP853_D_##r##_12 * k[12][i]                              \
     + DP853_D_##r##_13 * k[13][i] + DP853_D_##r##_14 * k[14][i]                              \
     + DP853_D_##r##_15 * k[15][i] + DP853_D_##r##_16 * k[16][i])
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const double d = y1[i] - y0[i];
        F[0][i] = d;
        F[1][i] = h * k[1][i] - d;
        F[2][i] = 2.0 * d - h * (k[13][i] + k[1][i]);
        F[3][i] = h * NBCS_DENSE_ROW(4);
        F[4][i] = h * NBCS_DENSE_ROW(5);
        F[5][i] = h * NBCS_DENSE_ROW(6);
        F[6][i] = h * NBCS_DENSE_ROW(7);
    }
#undef NBCS_DENSE_ROW
    while (*m < n && (teval[*m] - (xold + h)) * posneg <= 0.0) {
        const double th = (teval[*m] - xold) / h, th1 = 1.0 - th;
        double o[2];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            double v = F[6][i] * th;
            v = (F[5][i] + v) * th1;
            v = (F[4][i] + v) * th;
            v = (F[3][i] + v) * th1;
            v = (F[2][i] + v) * th;
            v = (F[1][i] + v) * th1;
            v = (F[0][i] + v) * th;
            o[i] = v + y0[i];
        }
        dout[*m] = make_double2(o[0], o[1]);
        ++*m;
    }
}

// Integrate y over solver time [x, xend]; `kc` is this thread's shared-memory
// column of stage derivatives (stride KS, the block size).  Returns NBCS_PARTICLE_*.
// DENSE: also the positions at the n output times teval (teval[0] = x,
// teval[n-1] = xend) into dout[0 .. n), by dense output; kc needs 16 slots.
// When an output falls in an accepted step, the derivative at its end is
// evaluated there (for the interpolant) and handed to the next step as its
// first stage, with the same arguments as that stage would have had, so the
// step sequence is the one without outputs.
template <class Flow, int KS = kThreads64, bool DENSE = false>
__device__ int dop853_solve64(const Flow& fl, const Params& P, double x, double xend, double* y,
                              double rtol, double atol, int nmax, double2* kc, Dop853Stats* st,
                              const double* __restrict__ teval = nullptr, int n = 0,
                              double2* __restrict__ dout = nullptr)
{
    const double uround = 2.3e-16, safe = 0.9, facc1 = 1.0 / 0.333, facc2 = 1.0 / 6.0;
    const double posneg = (xend - x) >= 0.0 ? 1.0 : -1.0;
    double yy[2], kk[2], h = 0.0, hnew, hmax, err, err2, deno, fac, fac11, sk, erri, sqr;
    bool last = false, reject = false;
    int nstep = 0, status = NBCS_PARTICLE_OK;
    int m = 1;  // next dense output
    st->accepted = st->rejected = st->nfcn = 0;
    if (DENSE) dout[0] = make_double2(y[0], y[1]);
    if (xend == x) {
        if (DENSE)
            for (; m < n; ++m) dout[m] = make_double2(y[0], y[1]);
        return NBCS_PARTICLE_OK;
    }
    hmax = fabs(xend - x);

    // HINIT (f0 = f(x, y) is also stage 0 of the first step); one RHS site
    double f0[2] = {0.0, 0.0}, dnf = 0.0, dny = 0.0;
#pragma unroll 1
    for (int e = 0; e < 2; ++e) {
#pragma unroll
        for (int i = 0; i < 2; ++i) yy[i] = e ? y[i] + h * f0[i] : y[i];
        fl(e ? x + h : x, yy, kk, P);
        if (e == 0) {
            f0[0] = kk[0];
            f0[1] = kk[1];
            kc[0] = make_double2(kk[0], kk[1]);
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
        } else {
            double der2 = 0.0, der12, h1;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                sk = atol + rtol * fabs(y[i]);
                sqr = (kk[i] - f0[i]) / sk;
                der2 += sqr * sqr;
            }
            der2 = sqrt(der2) / h;
            der12 = dmax_(fabs(der2), sqrt(dnf));
            if (der12 <= 1.0e-15) h1 = dmax_(1.0e-6, fabs(h) * 1.0e-3);
            else h1 = nbcs_root8(0.01 / der12);  // (0.01/der12)^(1/8)
            h = dmin_(100.0 * fabs(h), dmin_(h1, hmax));
            h = posneg >= 0.0 ? fabs(h) : -fabs(h);
        }
    }
    st->nfcn += 2;

    bool fsal = false;  // stage 0 (the derivative at the new point) still to evaluate
    for (;;) {
        if (nstep > nmax) { status = NBCS_PARTICLE_MAX_STEPS; break; }
        if (0.1 * fabs(h) <= fabs(x) * uround) { status = NBCS_PARTICLE_STEP_UNDERFLOW; break; }
        if ((x + 1.01 * h - xend) * posneg > 0.0) {
            h = xend - x;
            last = true;
        }
        nstep++;
#pragma unroll 1
        for (int s = fsal ? 0 : 1; s < 12; ++s) {
            if (s == 0) {
                yy[0] = y[0];
                yy[1] = y[1];
            } else if (s == 1) {
                const double2 k1 = kc[0];
                yy[0] = y[0] + h * DP853_A_2_1 * k1.x;
                yy[1] = y[1] + h * DP853_A_2_1 * k1.y;
            } else {
                double a0 = 0.0, a1 = 0.0;
#pragma unroll
                for (int j = 0; j < 11; ++j) {
                    if (j < s) {
                        const double c = kA64[s][j];
                        if (c != 0.0) {
                            const double2 kj = kc[j * KS];
                            a0 = a0 + c * kj.x;
                            a1 = a1 + c * kj.y;
                        }
                    }
                }
                yy[0] = y[0] + h * a0;
                yy[1] = y[1] + h * a1;
            }
            fl(x + kC64[s] * h, yy, kk, P);
            kc[s * KS] = make_double2(kk[0], kk[1]);
        }
        fsal = false;
        st->nfcn += 11;
        double b[2] = {0.0, 0.0}, e5[2] = {0.0, 0.0}, ynew[2];
#pragma unroll
        for (int j = 0; j < 12; ++j) {
            const double2 kj = kc[j * KS];
            if (kB64[j] != 0.0) {
                b[0] = b[0] + kB64[j] * kj.x;
                b[1] = b[1] + kB64[j] * kj.y;
            }
            if (kE5_64[j] != 0.0) {
                e5[0] = e5[0] + kE5_64[j] * kj.x;
                e5[1] = e5[1] + kE5_64[j] * kj.y;
            }
        }
        const double2 k1 = kc[0], k9 = kc[8 * KS], k12 = kc[11 * KS];
        const double k1v[2] = {k1.x, k1.y}, k9v[2] = {k9.x, k9.y}, k12v[2] = {k12.x, k12.y};
        err = 0.0;
        err2 = 0.0;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            ynew[i] = y[i] + h * b[i];
            sk = atol + rtol * dmax_(fabs(y[i]), fabs(ynew[i]));
            erri = b[i] - DP853_BHH1 * k1v[i] - DP853_BHH2 * k9v[i] - DP853_BHH3 * k12v[i];
            sqr = erri / sk;
            err2 += sqr * sqr;
            sqr = e5[i] / sk;
            err += sqr * sqr;
        }
        deno = err + 0.01 * err2;
        if (deno <= 0.0) deno = 1.0;
        err = fabs(h) * err * sqrt(1.0 / (deno * 2.0));
        if (isnan(err)) { status = NBCS_PARTICLE_NONFINITE; break; }
        fac11 = nbcs_root8(err);  // err^(1/8)
        fac = fac11;              // beta = 0: the Lund factor facold^beta is 1
        fac = dmax_(facc2, dmin_(facc1, fac / safe));
        hnew = h / fac;
        if (err <= 1.0) {
            st->accepted++;
            st->nfcn++;  // the derivative at the new point (next step's stage 0)
            bool have_end_derivative = false;
            if (DENSE && m < n && (teval[m] - (x + h)) * posneg <= 0.0) {
                fl(x + h, ynew, kk, P);
                kc[12 * KS] = make_double2(kk[0], kk[1]);
                dense_output64<Flow, KS>(fl, P, x, h, y, ynew, kc, teval, n, &m, posneg, dout);
                kc[0] = make_double2(kk[0], kk[1]);
                st->nfcn += 3;
                have_end_derivative = true;
            }
            y[0] = ynew[0];
            y[1] = ynew[1];
            x = x + h;
            fsal = !have_end_derivative;
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
    return status;
}

}  // namespace nbcs
