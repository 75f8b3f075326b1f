// Mixed-precision flow-map integration (NBCS_PREC_MIXED).
//
// Same DOP853 method and dop853 step-size controller as the FP64 path
// (dop853_64.cuh), but the 12 stages, the RHS and the spline interpolation
// run on the FP32 pipe.  Particle position and time are carried as
// compensated FP32 pairs (hi + lo, ~48-bit significand) so that the
// accumulation over many steps keeps FP64-class accuracy; stage arguments
// only need FP32 accuracy and are formed as hi + (lo + h*sum).
//
// Particles are mapped to threads in 16x8 tiles of the (x, y) grid so that a
// warp integrates a 4x8 patch: neighbouring trajectories read the same
// spline coefficients (L1 hits) and take similar step counts (less
// divergence).
#include "dop853_tableau.h"
#include "flowmap_common.cuh"
#include "flows32.cuh"

namespace nbcs {

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

// a + b with b = p + e given as an exact product pair (Knuth two-sum on hi).
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
    float p = h * b;
    float e = fmaf(h, b, -p);
    return f2_add(a, p, e);
}

__device__ __forceinline__ float f2_minus(F2 a, F2 b)  // (a - b) rounded to float
{
    return (a.hi - b.hi) + (a.lo - b.lo);
}

__device__ __forceinline__ float stage_pos(F2 y, float d) { return y.hi + (y.lo + d); }

template <class Flow>
__device__ __forceinline__ float hinit32(const Flow& fl, const ParamsF& P, float x, const float* y,
                                         float posneg, const float* f0, float hmax, float rtol,
                                         float atol)
{
    float dnf = 0.f, dny = 0.f, h, y1[2], f1[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        float sk = fmaf(rtol, fabsf(y[i]), atol);
        float a = f0[i] / sk, b = y[i] / sk;
        dnf = fmaf(a, a, dnf);
        dny = fmaf(b, b, dny);
    }
    if (dnf <= 1.0e-10f || dny <= 1.0e-10f) h = 1.0e-6f;
    else h = sqrtf(dny / dnf) * 0.01f;
    h = fminf(h, hmax);
    h = copysignf(h, posneg);
#pragma unroll
    for (int i = 0; i < 2; ++i) y1[i] = fmaf(h, f0[i], y[i]);
    fl(x + h, y1, f1, P);
    float der2 = 0.f;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        float sk = fmaf(rtol, fabsf(y[i]), atol);
        float a = (f1[i] - f0[i]) / sk;
        der2 = fmaf(a, a, der2);
    }
    der2 = sqrtf(der2) / h;
    float der12 = fmaxf(fabsf(der2), sqrtf(dnf));
    float h1 = der12 <= 1.0e-15f ? fmaxf(1.0e-6f, fabsf(h) * 1.0e-3f)
                                 : exp2f(0.125f * log2f(0.01f / der12));
    h = fminf(100.0f * fabsf(h), fminf(h1, hmax));
    return copysignf(h, posneg);
}

#define A_(s, j) ((float)DP853_A_##s##_##j)
#define C_(s) ((float)DP853_C_##s)

template <class Flow>
__device__ int dop853_solve32(const Flow& fl, const ParamsF& P, F2 x, F2 xend, F2* y, float rtol,
                              float atol, int nmax, int* acc, int* rej, int* nfcn)
{
    const float safe = 0.9f, facc1 = (float)(1.0 / 0.333), facc2 = (float)(1.0 / 6.0);
    float k1[2], k2[2], k3[2], k4[2], k5[2], k6[2], k7[2], k8[2], k9[2], k10[2], yy[2], yf[2];
    const float span = f2_minus(xend, x);
    const float posneg = span >= 0.f ? 1.f : -1.f;
    const float hmax = fabsf(span);
    int nstep = 0, status = NBCS_PARTICLE_OK;
    bool last = false, reject = false;
    *acc = *rej = *nfcn = 0;
    if (span == 0.f) return NBCS_PARTICLE_OK;

    yf[0] = y[0].hi + y[0].lo;
    yf[1] = y[1].hi + y[1].lo;
    float xf = x.hi + x.lo;
    fl(xf, yf, k1, P);
    float h = hinit32(fl, P, xf, yf, posneg, k1, hmax, rtol, atol);
    *nfcn += 2;

    for (;;) {
        if (nstep > nmax) { status = NBCS_PARTICLE_MAX_STEPS; break; }
        float rem = f2_minus(xend, x);
        xf = x.hi + x.lo;
        // time is a compensated pair: resolution ~2^-44 relative
        if (0.1f * fabsf(h) <= fabsf(xf) * 1.0e-13f) { status = NBCS_PARTICLE_STEP_UNDERFLOW; break; }
        if ((1.01f * h - rem) * posneg > 0.f) {
            h = rem;
            last = true;
        }
        nstep++;
#define STAGE_T(cc) (x.hi + fmaf((cc), h, x.lo))
#pragma unroll
        for (int i = 0; i < 2; ++i) yy[i] = stage_pos(y[i], h * (A_(2, 1) * k1[i]));
        fl(STAGE_T(C_(2)), yy, k2, P);
#pragma unroll
        for (int i = 0; i < 2; ++i) yy[i] = stage_pos(y[i], h * fmaf(A_(3, 1), k1[i], A_(3, 2) * k2[i]));
        fl(STAGE_T(C_(3)), yy, k3, P);
#pragma unroll
        for (int i = 0; i < 2; ++i) yy[i] = stage_pos(y[i], h * fmaf(A_(4, 1), k1[i], A_(4, 3) * k3[i]));
        fl(STAGE_T(C_(4)), yy, k4, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy[i] = stage_pos(y[i], h * fmaf(A_(5, 1), k1[i], fmaf(A_(5, 3), k3[i], A_(5, 4) * k4[i])));
        fl(STAGE_T(C_(5)), yy, k5, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy[i] = stage_pos(y[i], h * fmaf(A_(6, 1), k1[i], fmaf(A_(6, 4), k4[i], A_(6, 5) * k5[i])));
        fl(STAGE_T(C_(6)), yy, k6, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy[i] = stage_pos(y[i], h * fmaf(A_(7, 1), k1[i], fmaf(A_(7, 4), k4[i],
                                          fmaf(A_(7, 5), k5[i], A_(7, 6) * k6[i]))));
        fl(STAGE_T(C_(7)), yy, k7, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy[i] = stage_pos(y[i], h * fmaf(A_(8, 1), k1[i], fmaf(A_(8, 4), k4[i], fmaf(A_(8, 5), k5[i],
                                          fmaf(A_(8, 6), k6[i], A_(8, 7) * k7[i])))));
        fl(STAGE_T(C_(8)), yy, k8, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy[i] = stage_pos(y[i], h * fmaf(A_(9, 1), k1[i], fmaf(A_(9, 4), k4[i], fmaf(A_(9, 5), k5[i],
                                          fmaf(A_(9, 6), k6[i], fmaf(A_(9, 7), k7[i], A_(9, 8) * k8[i]))))));
        fl(STAGE_T(C_(9)), yy, k9, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy[i] = stage_pos(y[i], h * fmaf(A_(10, 1), k1[i], fmaf(A_(10, 4), k4[i],
                                          fmaf(A_(10, 5), k5[i], fmaf(A_(10, 6), k6[i],
                                          fmaf(A_(10, 7), k7[i], fmaf(A_(10, 8), k8[i], A_(10, 9) * k9[i])))))));
        fl(STAGE_T(C_(10)), yy, k10, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy[i] = stage_pos(y[i], h * fmaf(A_(11, 1), k1[i], fmaf(A_(11, 4), k4[i],
                                          fmaf(A_(11, 5), k5[i], fmaf(A_(11, 6), k6[i],
                                          fmaf(A_(11, 7), k7[i], fmaf(A_(11, 8), k8[i],
                                          fmaf(A_(11, 9), k9[i], A_(11, 10) * k10[i]))))))));
        fl(STAGE_T(C_(11)), yy, k2, P);
#pragma unroll
        for (int i = 0; i < 2; ++i)
            yy[i] = stage_pos(y[i], h * fmaf(A_(12, 1), k1[i], fmaf(A_(12, 4), k4[i],
                                          fmaf(A_(12, 5), k5[i], fmaf(A_(12, 6), k6[i],
                                          fmaf(A_(12, 7), k7[i], fmaf(A_(12, 8), k8[i],
                                          fmaf(A_(12, 9), k9[i], fmaf(A_(12, 10), k10[i],
                                               A_(12, 11) * k2[i])))))))));
        fl(STAGE_T(1.0f), yy, k3, P);
#undef STAGE_T
        *nfcn += 11;
        F2 ynew[2];
        float err = 0.f, err2 = 0.f;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            float bsum = fmaf((float)DP853_B_1, k1[i], fmaf((float)DP853_B_6, k6[i],
                         fmaf((float)DP853_B_7, k7[i], fmaf((float)DP853_B_8, k8[i],
                         fmaf((float)DP853_B_9, k9[i], fmaf((float)DP853_B_10, k10[i],
                         fmaf((float)DP853_B_11, k2[i], (float)DP853_B_12 * k3[i])))))));
            ynew[i] = f2_axpy(y[i], h, bsum);
            k4[i] = bsum;
            float yo = y[i].hi + y[i].lo, yn = ynew[i].hi + ynew[i].lo;
            float sk = fmaf(rtol, fmaxf(fabsf(yo), fabsf(yn)), atol);
            float e3 = bsum - fmaf((float)DP853_BHH1, k1[i], fmaf((float)DP853_BHH2, k9[i],
                                  (float)DP853_BHH3 * k3[i]));
            float e5 = fmaf((float)DP853_E5_1, k1[i], fmaf((float)DP853_E5_6, k6[i],
                       fmaf((float)DP853_E5_7, k7[i], fmaf((float)DP853_E5_8, k8[i],
                       fmaf((float)DP853_E5_9, k9[i], fmaf((float)DP853_E5_10, k10[i],
                       fmaf((float)DP853_E5_11, k2[i], (float)DP853_E5_12 * k3[i])))))));
            float q3 = e3 / sk, q5 = e5 / sk;
            err2 = fmaf(q3, q3, err2);
            err = fmaf(q5, q5, err);
        }
        float deno = fmaf(0.01f, err2, err);
        if (deno <= 0.f) deno = 1.f;
        err = fabsf(h) * err * rsqrtf(deno * 2.0f);
        if (isnan(err)) { status = NBCS_PARTICLE_NONFINITE; break; }
        float fac11 = exp2f(0.125f * log2f(err));
        float fac = fmaxf(facc2, fminf(facc1, fac11 / safe));
        float hnew = h / fac;
        if (err <= 1.0f) {
            ++*acc;
            x = f2_add(x, h, 0.f);
            yf[0] = ynew[0].hi + ynew[0].lo;
            yf[1] = ynew[1].hi + ynew[1].lo;
            fl(x.hi + x.lo, yf, k1, P);
            ++*nfcn;
            y[0] = ynew[0];
            y[1] = ynew[1];
            if (last) break;
            if (fabsf(hnew) > hmax) hnew = posneg * hmax;
            if (reject) hnew = posneg * fminf(fabsf(hnew), fabsf(h));
            reject = false;
        } else {
            hnew = h / fminf(facc1, fac11 / safe);
            reject = true;
            if (*acc >= 1) ++*rej;
            last = false;
        }
        h = hnew;
    }
    return status;
}
#undef A_
#undef C_

// Thread -> particle map in 16 (x) by 8 (y) tiles, tiles in row-major order.
__device__ __forceinline__ bool tile_particle(long t, int nx, int ny, int* i, int* j)
{
    const int TI = 16, TJ = 8;
    long tile = t >> 7;
    int r = (int)(t & 127);
    int tiles_j = (ny + TJ - 1) / TJ;
    long ti = tile / tiles_j;
    int tj = (int)(tile - ti * tiles_j);
    *i = (int)(ti * TI) + (r >> 3);
    *j = tj * TJ + (r & 7);
    return *i < nx && *j < ny;
}

template <class Flow>
__global__ void __launch_bounds__(128)
flowmap32_kernel(Flow fl, ParamsF P, double ts, double te, const double* __restrict__ x,
                 const double* __restrict__ y, int nx, int ny, const uint8_t* __restrict__ mask,
                 double* __restrict__ out, int32_t* __restrict__ status,
                 int32_t* __restrict__ stats, float rtol, float atol, int nmax, long nthreads)
{
    const F2 xs = f2_from_double(ts), xe = f2_from_double(te);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nthreads;
         t += (long)gridDim.x * blockDim.x) {
        int i, j;
        if (!tile_particle(t, nx, ny, &i, &j)) continue;
        long k = (long)i * ny + j;
        double r0 = 0.0, r1 = 0.0;
        int st = NBCS_PARTICLE_MASKED, a = 0, rj = 0, nf = 0;
        if (!(mask && mask[k])) {
            F2 yv[2] = {f2_from_double(x[i]), f2_from_double(y[j])};
            st = dop853_solve32(fl, P, xs, xe, yv, rtol, atol, nmax, &a, &rj, &nf);
            r0 = f2_to_double(yv[0]);
            r1 = f2_to_double(yv[1]);
        }
        reinterpret_cast<double2*>(out)[k] = make_double2(r0, r1);
        if (status) status[k] = st;
        if (stats) {
            stats[3 * k] = a;
            stats[3 * k + 1] = rj;
            stats[3 * k + 2] = nf;
        }
    }
}

template <class Flow>
__global__ void rhs32_kernel(Flow fl, ParamsF P, const double* __restrict__ ty, long n,
                             double* __restrict__ dy)
{
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long)gridDim.x * blockDim.x) {
        float yv[2] = {(float)ty[3 * k + 1], (float)ty[3 * k + 2]}, d[2];
        fl((float)ty[3 * k], yv, d, P);
        dy[2 * k] = d[0];
        dy[2 * k + 1] = d[1];
    }
}

static ParamsF to_float(const Params& P)
{
    ParamsF f;
    for (int i = 0; i < NBCS_MAX_PARAMS; ++i) f.v[i] = (float)P.v[i];
    return f;
}

template <class F>
static int dispatch32(const nbcs_flow* flow, const F& f)
{
    switch (flow->kind) {
    case NBCS_FLOW_DOUBLE_GYRE: return f(FlowDG32{});
    case NBCS_FLOW_BICKLEY: return f(FlowBickley32{});
    default: {
        SplineGridF g = make_grid_f(flow->grid);
        const float2* c = reinterpret_cast<const float2*>(flow->coef_uv32);
        float k = (float)(180.0 / (3.141592653589793 * flow->r));
        switch (flow->spherical) {
        case 1: return f(FlowSpline32<1>{g, c, k});
        case 2: return f(FlowSpline32<2>{g, c, k});
        default: return f(FlowSpline32<0>{g, c, k});
        }
    }
    }
}

struct Launch32 {
    const FlowmapArgs* a;
    template <class Flow>
    int operator()(const Flow& fl) const
    {
        const int threads = 128;
        long tiles = (long)((a->nx + 15) / 16) * ((a->ny + 7) / 8);
        long nthreads = tiles * 128;
        long blocks = nthreads / threads;
        if (blocks > (1L << 30)) blocks = 1L << 30;
        flowmap32_kernel<<<(unsigned)blocks, threads, 0, a->stream>>>(
            fl, to_float(a->P), a->ts, a->te, a->x, a->y, a->nx, a->ny, a->mask, a->out,
            a->status, a->stats, (float)a->rtol, (float)a->atol, a->nmax, nthreads);
        NBCS_LAUNCH_CHECK();
        return NBCS_OK;
    }
};

struct LaunchRhs32 {
    ParamsF P;
    const double* ty;
    long n;
    double* dy;
    cudaStream_t stream;
    template <class Flow>
    int operator()(const Flow& fl) const
    {
        long blocks = (n + 127) / 128;
        rhs32_kernel<<<(unsigned)blocks, 128, 0, stream>>>(fl, P, ty, n, dy);
        NBCS_LAUNCH_CHECK();
        return NBCS_OK;
    }
};

int launch_flowmap32(const nbcs_flow* flow, const FlowmapArgs& a)
{
    return dispatch32(flow, Launch32{&a});
}

int launch_rhs32(const nbcs_flow* flow, const Params& P, const double* ty, long n, double* dy,
                 cudaStream_t stream)
{
    return dispatch32(flow, LaunchRhs32{to_float(P), ty, n, dy, stream});
}

}  // namespace nbcs
