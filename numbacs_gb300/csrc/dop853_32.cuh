// Mixed-precision DOP853 for one particle (shared by the single-field and
// batched integrators).
//
// Same DOP853 method and dop853 step-size controller as the FP64 path
// (dop853_64.cuh), but the stages and the RHS run on the FP32 pipe.  Particle
// position and time are carried as compensated FP32 pairs (hi + lo, ~48-bit
// significand) so that accumulating many steps keeps FP64-class accuracy; a
// stage argument is handed to the RHS as the pair (hi, lo + h*sum) and the RHS
// forms what it needs from it (flows32.cuh).
//
// Code shape (from the profile of the fully unrolled version, which was
// instruction-fetch bound): the twelve stages run as one rolled loop so the
// right-hand side is instantiated once; the stage derivatives live in a
// shared-memory column of stride KS (one per thread, or one per particle whose
// lanes share it) and the tableau is a set of compile-time constants.
#pragma once

#include "detmath.h"
#include "dop853_tableau.h"
#include "flows32.cuh"
#include "nbcs_internal.cuh"

namespace nbcs {

#define F_(x) ((float)(x))
// DP853 tableau as compile-time FP32 values, 0-based stage index: stage s uses
// a(s, j) for j < s.  Being constants of the compiler (not of a memory bank),
// the zero entries (a_i2 for i > 3, a_i3 for i > 5, b_2..b_5, the error
// weights at stages 2-5) cost neither a load of k_j nor an FMA.
struct DP853F {
    __host__ __device__ static constexpr float a(int s, int j)
    {
        constexpr float t[12][12] = {
            {0.f},
            {F_(DP853_A_2_1)},
            {F_(DP853_A_3_1), F_(DP853_A_3_2)},
            {F_(DP853_A_4_1), F_(DP853_A_4_2), F_(DP853_A_4_3)},
            {F_(DP853_A_5_1), F_(DP853_A_5_2), F_(DP853_A_5_3), F_(DP853_A_5_4)},
            {F_(DP853_A_6_1), F_(DP853_A_6_2), F_(DP853_A_6_3), F_(DP853_A_6_4), F_(DP853_A_6_5)},
            {F_(DP853_A_7_1), F_(DP853_A_7_2), F_(DP853_A_7_3), F_(DP853_A_7_4), F_(DP853_A_7_5),
             F_(DP853_A_7_6)},
            {F_(DP853_A_8_1), F_(DP853_A_8_2), F_(DP853_A_8_3), F_(DP853_A_8_4), F_(DP853_A_8_5),
             F_(DP853_A_8_6), F_(DP853_A_8_7)},
            {F_(DP853_A_9_1), F_(DP853_A_9_2), F_(DP853_A_9_3), F_(DP853_A_9_4), F_(DP853_A_9_5),
             F_(DP853_A_9_6), F_(DP853_A_9_7), F_(DP853_A_9_8)},
            {F_(DP853_A_10_1), F_(DP853_A_10_2), F_(DP853_A_10_3), F_(DP853_A_10_4),
             F_(DP853_A_10_5), F_(DP853_A_10_6), F_(DP853_A_10_7), F_(DP853_A_10_8),
             F_(DP853_A_10_9)},
            {F_(DP853_A_11_1), F_(DP853_A_11_2), F_(DP853_A_11_3), F_(DP853_A_11_4),
             F_(DP853_A_11_5), F_(DP853_A_11_6), F_(DP853_A_11_7), F_(DP853_A_11_8),
             F_(DP853_A_11_9), F_(DP853_A_11_10)},
            {F_(DP853_A_12_1), F_(DP853_A_12_2), F_(DP853_A_12_3), F_(DP853_A_12_4),
             F_(DP853_A_12_5), F_(DP853_A_12_6), F_(DP853_A_12_7), F_(DP853_A_12_8),
             F_(DP853_A_12_9), F_(DP853_A_12_10), F_(DP853_A_12_11)},
        };
        return t[s][j];
    }
    __host__ __device__ static constexpr float b(int j)
    {
        constexpr float t[12] = {F_(DP853_B_1), F_(DP853_B_2), F_(DP853_B_3), F_(DP853_B_4),
                                 F_(DP853_B_5), F_(DP853_B_6), F_(DP853_B_7), F_(DP853_B_8),
                                 F_(DP853_B_9), F_(DP853_B_10), F_(DP853_B_11), F_(DP853_B_12)};
        return t[j];
    }
    // 5th-order error weights
    __host__ __device__ static constexpr float e5(int j)
    {
        constexpr float t[12] = {F_(DP853_E5_1), F_(DP853_E5_2), F_(DP853_E5_3), F_(DP853_E5_4),
                                 F_(DP853_E5_5), F_(DP853_E5_6), F_(DP853_E5_7), F_(DP853_E5_8),
                                 F_(DP853_E5_9), F_(DP853_E5_10), F_(DP853_E5_11),
                                 F_(DP853_E5_12)};
        return t[j];
    }
    // 3rd-order estimate weights b_j - bhh_j (bhh at stages 1, 9, 12)
    __host__ __device__ static constexpr float e3(int j)
    {
        constexpr float t[12] = {F_(DP853_B_1 - DP853_BHH1), F_(DP853_B_2), F_(DP853_B_3),
                                 F_(DP853_B_4), F_(DP853_B_5), F_(DP853_B_6), F_(DP853_B_7),
                                 F_(DP853_B_8), F_(DP853_B_9 - DP853_BHH2), F_(DP853_B_10),
                                 F_(DP853_B_11), F_(DP853_B_12 - DP853_BHH3)};
        return t[j];
    }
};
// stage times c_s
__host__ __device__ constexpr float dp853_c32(int s)
{
    constexpr float t[12] = {0.f, F_(DP853_C_2), F_(DP853_C_3), F_(DP853_C_4), F_(DP853_C_5),
                             F_(DP853_C_6), F_(DP853_C_7), F_(DP853_C_8), F_(DP853_C_9),
                             F_(DP853_C_10), F_(DP853_C_11), 1.0f};
    return t[s];
}
#undef F_

constexpr int kThreads32 = 128;

// unevaluated sum hi + lo
struct F2 {
    float hi, lo;
};

__device__ __forceinline__ F2 f2_from_double(double d)
{
    float h = (float)d;
    return {h, (float)(d - (double)h)};
}

__device__ __forceinline__ double f2_to_double(F2 a) { return (double)a.hi + (double)a.lo; }

// a + (p + e): Knuth two-sum of the hi parts, low parts added to the error.
__device__ __forceinline__ F2 f2_add(F2 a, float p, float e)
{
    float s = __fadd_rn(a.hi, p);
    float bb = __fsub_rn(s, a.hi);
    float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    err = __fadd_rn(err, __fadd_rn(a.lo, e));
    float h = __fadd_rn(s, err);
    return {h, __fsub_rn(err, __fsub_rn(h, s))};
}

// a + h*b with the product rounding error kept
__device__ __forceinline__ F2 f2_axpy(F2 a, float h, float b)
{
    float p = __fmul_rn(h, b);
    float e = fmaf(h, b, -p);
    return f2_add(a, p, e);
}

__device__ __forceinline__ float f2_minus(F2 a, F2 b)  // (a - b) rounded to float
{
    return (a.hi - b.hi) + (a.lo - b.lo);
}

// Terms j >= J of the stage argument combination sum_{j<S} a_Sj k_j: the
// nonzero ones only, in ascending j.  KS is the stride of the shared-memory
// column of stage derivatives (the block size).
// The (x, y) halves of k_j share the coefficient: one paired FMA per term
// (fma_pair, bit-identical to two fmaf).
template <int S, int KS, int J = 0>
__device__ __forceinline__ void stage_terms(const float2* kc, float2& xy)
{
    if constexpr (J < S) {
        constexpr float a = DP853F::a(S, J);
        if constexpr (a != 0.f) xy = fma_pair(a, kc[J * KS], xy);
        stage_terms<S, KS, J + 1>(kc, xy);
    }
}

// Stage argument combination and stage time c_S for a compile-time stage S.
template <int S, int KS>
__device__ __forceinline__ void stage_combo(const float2* kc, float* a0, float* a1, float* c)
{
    float2 xy = make_float2(0.f, 0.f);
    stage_terms<S, KS>(kc, xy);
    *a0 = xy.x;
    *a1 = xy.y;
    *c = dp853_c32(S);
}

// The step's solution increment sum b_j k_j and the two error estimates
// sum e5_j k_j, sum e3_j k_j, over the stages with a nonzero weight.
template <int KS, int J = 0>
__device__ __forceinline__ void step_sums(const float2* kc, float2& b, float2& e5, float2& e3)
{
    if constexpr (J < 12) {
        constexpr float wb = DP853F::b(J), w5 = DP853F::e5(J), w3 = DP853F::e3(J);
        if constexpr (wb != 0.f || w5 != 0.f || w3 != 0.f) {
            const float2 kj = kc[J * KS];
            if constexpr (wb != 0.f) b = fma_pair(wb, kj, b);
            if constexpr (w5 != 0.f) e5 = fma_pair(w5, kj, e5);
            if constexpr (w3 != 0.f) e3 = fma_pair(w3, kj, e3);
        }
        step_sums<KS, J + 1>(kc, b, e5, e3);
    }
}

// The same for a runtime stage s that is uniform across the warp (one branch
// of a jump table instead of eleven predicated terms per stage).
template <int KS>
__device__ __forceinline__ void stage_combo(int s, const float2* kc, float* a0, float* a1,
                                            float* c)
{
    switch (s) {
    case 0: *a0 = 0.f; *a1 = 0.f; *c = 0.f; break;
    case 1: stage_combo<1, KS>(kc, a0, a1, c); break;
    case 2: stage_combo<2, KS>(kc, a0, a1, c); break;
    case 3: stage_combo<3, KS>(kc, a0, a1, c); break;
    case 4: stage_combo<4, KS>(kc, a0, a1, c); break;
    case 5: stage_combo<5, KS>(kc, a0, a1, c); break;
    case 6: stage_combo<6, KS>(kc, a0, a1, c); break;
    case 7: stage_combo<7, KS>(kc, a0, a1, c); break;
    case 8: stage_combo<8, KS>(kc, a0, a1, c); break;
    case 9: stage_combo<9, KS>(kc, a0, a1, c); break;
    case 10: stage_combo<10, KS>(kc, a0, a1, c); break;
    default: stage_combo<11, KS>(kc, a0, a1, c); break;
    }
}

// Integrate one particle (y, as compensated pairs) over solver time [x, xend].
// `kc` is this thread's shared-memory column of stage derivatives (stride KS,
// the block size).  Returns an NBCS_PARTICLE_* code.
template <class Flow, int KS = kThreads32>
__device__ int dop853_solve32(const Flow& fl, const ParamsF& P, F2 x, F2 xend, F2* y, float rtol,
                              float atol, int nmax, float2* kc, int* acc, int* rej, int* nfcn)
{
    const float safe = 0.9f, facc1 = (float)(1.0 / 0.333), facc2 = (float)(1.0 / 6.0);
    const float span = f2_minus(xend, x);
    const float posneg = span >= 0.f ? 1.f : -1.f;
    const float hmax = fabsf(span);
    float yh[2], ys[2], kk[2];
    int nstep = 0, status = NBCS_PARTICLE_OK;
    bool last = false, reject = false;
    *acc = *rej = *nfcn = 0;
    if (span == 0.f) return NBCS_PARTICLE_OK;

    // HINIT: f0 = f(x, y), Euler probe f1 = f(x + h, y + h f0); one RHS site
    float h = 0.f, dnf = 0.f, dny = 0.f, f0[2] = {0.f, 0.f};
#pragma unroll 1
    for (int e = 0; e < 2; ++e) {
        yh[0] = y[0].hi;
        yh[1] = y[1].hi;
        ys[0] = e ? fmaf(h, f0[0], y[0].lo) : y[0].lo;
        ys[1] = e ? fmaf(h, f0[1], y[1].lo) : y[1].lo;
        fl(x.hi, e ? x.lo + h : x.lo, yh, ys, kk, P);
        if (e == 0) {
            f0[0] = kk[0];
            f0[1] = kk[1];
            kc[0] = make_float2(kk[0], kk[1]);
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                float yv = y[i].hi + y[i].lo;
                float sk = fmaf(rtol, fabsf(yv), atol);
                float a = f0[i] / sk, b = yv / sk;
                dnf = fmaf(a, a, dnf);
                dny = fmaf(b, b, dny);
            }
            h = (dnf <= 1.0e-10f || dny <= 1.0e-10f) ? 1.0e-6f : sqrtf(dny / dnf) * 0.01f;
            h = copysignf(fminf(h, hmax), posneg);
        } else {
            float der2 = 0.f;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                float sk = fmaf(rtol, fabsf(y[i].hi + y[i].lo), atol);
                float a = (kk[i] - f0[i]) / sk;
                der2 = fmaf(a, a, der2);
            }
            der2 = sqrtf(der2) / h;
            float der12 = fmaxf(fabsf(der2), sqrtf(dnf));
            float h1 = der12 <= 1.0e-15f ? fmaxf(1.0e-6f, fabsf(h) * 1.0e-3f)
                                         : nbcs_root8f(0.01f / der12);
            h = copysignf(fminf(100.0f * fabsf(h), fminf(h1, hmax)), posneg);
        }
    }
    *nfcn += 2;

    bool fsal = false;  // stage 0 (the derivative at the new point) still to evaluate
    for (;;) {
        if (nstep > nmax) { status = NBCS_PARTICLE_MAX_STEPS; break; }
        float rem = f2_minus(xend, x);
        // time is a compensated pair: a step below ~2^-48 |t| no longer advances it
        if (fabsf(h) <= fabsf(x.hi) * 3.6e-15f) { status = NBCS_PARTICLE_STEP_UNDERFLOW; break; }
        if ((1.01f * h - rem) * posneg > 0.f) {
            h = rem;
            last = true;
        }
        nstep++;
        yh[0] = y[0].hi;
        yh[1] = y[1].hi;
        // every lane counts the stages from 0 (a rejected step skips stage 0,
        // whose derivative is still valid) so the stage index is warp-uniform
#pragma unroll 1
        for (int s = 0; s < 12; ++s) {
            if (s == 0 && !fsal) continue;
            float a0, a1, cs;
            stage_combo<KS>(s, kc, &a0, &a1, &cs);
            ys[0] = fmaf(h, a0, y[0].lo);
            ys[1] = fmaf(h, a1, y[1].lo);
            fl(x.hi, fmaf(cs, h, x.lo), yh, ys, kk, P);
            kc[s * KS] = make_float2(kk[0], kk[1]);
        }
        fsal = false;
        *nfcn += 11;
        float2 b2 = make_float2(0.f, 0.f), e52 = b2, e32 = b2;
        step_sums<KS>(kc, b2, e52, e32);
        const float b[2] = {b2.x, b2.y}, e5[2] = {e52.x, e52.y}, e3[2] = {e32.x, e32.y};
        F2 ynew[2];
        float err = 0.f, err2 = 0.f;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            ynew[i] = f2_axpy(y[i], h, b[i]);
            float yo = y[i].hi + y[i].lo, yn = ynew[i].hi + ynew[i].lo;
            float sk = fmaf(rtol, fmaxf(fabsf(yo), fabsf(yn)), atol);
            const float rs = __frcp_rn(sk);
            float q3 = e3[i] * rs, q5 = e5[i] * rs;
            err2 = fmaf(q3, q3, err2);
            err = fmaf(q5, q5, err);
        }
        float deno = fmaf(0.01f, err2, err);
        if (deno <= 0.f) deno = 1.f;
        err = fabsf(h) * err * rsqrtf(deno * 2.0f);
        if (isnan(err)) { status = NBCS_PARTICLE_NONFINITE; break; }
        // err^(1/8) and the error ratios to a few ulp: step-size control needs
        // no more, and the IEEE divisions and square roots cost issue slots
        float fac11 = exp2f(0.125f * __log2f(err));  // err^(1/8)
        float fac = fmaxf(facc2, fminf(facc1, fac11 * (1.0f / safe)));
        float hnew = h / fac;
        if (err <= 1.0f) {
            ++*acc;
            ++*nfcn;  // the derivative at the new point (next step's stage 0)
            x = f2_add(x, h, 0.f);
            y[0] = ynew[0];
            y[1] = ynew[1];
            fsal = true;
            if (last) break;
            if (fabsf(hnew) > hmax) hnew = posneg * hmax;
            if (reject) hnew = posneg * fminf(fabsf(hnew), fabsf(h));
            reject = false;
        } else {
            hnew = h / fminf(facc1, fac11 * (1.0f / safe));
            reject = true;
            if (*acc >= 1) ++*rej;
            last = false;
        }
        h = hnew;
    }
    return status;
}

}  // namespace nbcs
