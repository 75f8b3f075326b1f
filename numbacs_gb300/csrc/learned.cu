// DOP853 with a learned step-size proposer (mixed precision, spline flows).
//
// Two uses of one warp-synchronous solver:
//   LOG      -- the plain dop853 controller runs; a hashed fraction of the
//               accepted steps writes (features at the step start, ideal log
//               step) as training data;
//   PROPOSE  -- the MLP of mlp.cuh proposes the step from the local features
//               and that proposal meets the controller's
//               (nbcs_opts.step_model_mode): at every fresh step start (modes
//               0-2, features from a gradient evaluation that is also the
//               step's first stage), or only at the first step and after a
//               rejection (modes 3, 4: the accepted steps run the plain
//               controller and first stage, features are evaluated only where
//               the network is asked).  The embedded error estimate still
//               accepts or rejects every step and rejected steps shrink with
//               the plain controller, so accuracy is the controller's; only
//               the step sequence changes.
//
// The MLP runs on the tensor cores for all 32 lanes of a warp at once, so the
// solver loop is warp-uniform: a lane whose particle is finished stays in the
// loop (idle) until the whole warp is done, and the inference block is entered
// by every lane whenever any lane needs a proposal.
//
// Features (direction-independent): lon, lat, t (model time), u, v, du/dx,
// du/dy, dv/dx, with the velocity and its Jacobian from the spline's value and
// basis derivatives at the step start (that evaluation is also the step's
// first stage).  Target: log(|h| * 0.9 * err^(-1/8)) -- the step the dop853
// controller would have chosen had it known this step's error.
#include "dop853_32.cuh"
#include "flowmap_common.cuh"
#include "mlp.cuh"

namespace nbcs {

struct LogSink {
    float* feats;
    float* targets;
    long long capacity;
    unsigned long long* count;
    float sample;
    unsigned seed;
};

__device__ __forceinline__ unsigned hash32(unsigned a, unsigned b)
{
    unsigned h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u + (a << 6) + (a >> 2));
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

// Features and stage-0 derivative at the step start; false when the particle
// is outside the velocity grid (zero velocity: no proposal, no training sample,
// the plain controller lets its steps grow to the end of the span).
template <class Flow>
__device__ __forceinline__ bool step_features(const Flow& fl, F2 x, const F2* y, const ParamsF& P,
                                              float* k0, float* f)
{
    float yh[2] = {y[0].hi, y[1].hi}, ys[2] = {y[0].lo, y[1].lo}, J[4];
    const bool inside = fl.eval_grad(x.hi, x.lo, yh, ys, k0, J, P);
    const float p0 = P.v[0];
    f[0] = yh[0] + ys[0];
    f[1] = yh[1] + ys[1];
    f[2] = p0 * (x.hi + x.lo);
    f[3] = p0 * k0[0];
    f[4] = p0 * k0[1];
    f[5] = p0 * J[0];
    f[6] = p0 * J[1];
    f[7] = p0 * J[2];
    return inside;
}

template <class Flow, bool LOG, bool PROPOSE>
__device__ void solve32_warp(const Flow& fl, const ParamsF& P, F2 x, F2 xend, F2* y, float rtol,
                             float atol, int nmax, float2* kc, bool active, const MlpBlob* W,
                             __nv_bfloat16* xs, float* outs, int mode, const LogSink& sink,
                             bool lead, unsigned pid, int* status_out, int* acc, int* rej,
                             int* nfcn)
{
    const unsigned FULL = 0xffffffffu;
    const float safe = 0.9f, facc1 = (float)(1.0 / 0.333), facc2 = (float)(1.0 / 6.0);
    const float span = f2_minus(xend, x);
    const float posneg = span >= 0.f ? 1.f : -1.f;
    const float hmax = fabsf(span);
    int status = NBCS_PARTICLE_OK, nstep = 0;
    bool last = false, reject = false, fresh = false, feat_ok = false;
    float feat[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float h = 0.f, yh[2], ys[2], kk[2];
    *acc = *rej = *nfcn = 0;
    if (span == 0.f) active = false;

    const bool sparse = PROPOSE && mode >= 3;  // ask the network at the start and after rejections
    if (active && PROPOSE && mode == 4) {
        // the proposal replaces HINIT: one feature evaluation (the first
        // stage), no probe; the controller's step stays at the span until the
        // proposal meets it below (a particle outside the grid keeps HINIT)
        float f0[2];
        feat_ok = step_features(fl, x, y, P, f0, feat);
        kc[0] = make_float2(f0[0], f0[1]);
        *nfcn += 1;
        fresh = feat_ok;
        h = posneg * hmax;
    }
    if (active && !(PROPOSE && mode == 4 && feat_ok)) {  // HINIT, with f0 from the feature evaluation
        float f0[2];
        if (!(PROPOSE && mode == 4)) feat_ok = step_features(fl, x, y, P, f0, feat);
        else f0[0] = kc[0].x, f0[1] = kc[0].y, *nfcn -= 1;
        kc[0] = make_float2(f0[0], f0[1]);
        float dnf = 0.f, dny = 0.f;
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
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            yh[i] = y[i].hi;
            ys[i] = fmaf(h, f0[i], y[i].lo);
        }
        fl(x.hi, x.lo + h, yh, ys, kk, P);
        float der2 = 0.f;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            float sk = fmaf(rtol, fabsf(y[i].hi + y[i].lo), atol);
            float a = (kk[i] - f0[i]) / sk;
            der2 = fmaf(a, a, der2);
        }
        der2 = sqrtf(der2) / h;
        float der12 = fmaxf(fabsf(der2), sqrtf(dnf));
        float h1 = der12 <= 1.0e-15f ? fmaxf(1.0e-6f, fabsf(h) * 1.0e-3f) : nbcs_root8f(0.01f / der12);
        h = copysignf(fminf(100.0f * fabsf(h), fminf(h1, hmax)), posneg);
        *nfcn += 2;
        fresh = feat_ok;
    }

    while (__any_sync(FULL, active)) {
        if (PROPOSE) {
            const bool want = active && fresh;
            if (__any_sync(FULL, want)) {
                const float lh = mlp_predict_groups<Flow::LP>(*W, feat, xs, outs);
                if (want) {
                    const float hm = __expf(lh), hc = fabsf(h);
                    // (mode 4's first proposal meets h = the span: it stands alone)
                    float hn = mode == 0 ? hm : (mode == 2 ? sqrtf(hm * hc) : fminf(hm, hc));
                    hn = fminf(hn, hmax);
                    if (hn > 0.f && hn < INFINITY) h = copysignf(hn, posneg);
                }
            }
        }
        if (!active) continue;
        fresh = false;
        if (nstep > nmax) {
            status = NBCS_PARTICLE_MAX_STEPS;
            active = false;
            continue;
        }
        const float rem = f2_minus(xend, x);
        if (fabsf(h) <= fabsf(x.hi) * 3.6e-15f) {
            status = NBCS_PARTICLE_STEP_UNDERFLOW;
            active = false;
            continue;
        }
        if ((1.01f * h - rem) * posneg > 0.f) {
            h = rem;
            last = true;
        }
        nstep++;
        yh[0] = y[0].hi;
        yh[1] = y[1].hi;
#pragma unroll 1
        for (int s = 1; s < 12; ++s) {
            float a0, a1, cs;
            stage_combo<kThreads32>(s, kc, &a0, &a1, &cs);
            ys[0] = fmaf(h, a0, y[0].lo);
            ys[1] = fmaf(h, a1, y[1].lo);
            fl(x.hi, fmaf(cs, h, x.lo), yh, ys, kk, P);
            kc[s * kThreads32] = make_float2(kk[0], kk[1]);
        }
        *nfcn += 11;
        float2 b2 = make_float2(0.f, 0.f), e52 = b2, e32 = b2;
        step_sums<kThreads32>(kc, b2, e52, e32);
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
        if (isnan(err)) {
            status = NBCS_PARTICLE_NONFINITE;
            active = false;
            continue;
        }
        const float fac11 = exp2f(0.125f * __log2f(err));  // err^(1/8)
        const float fac = fmaxf(facc2, fminf(facc1, fac11 * (1.0f / safe)));
        float hnew = h / fac;
        if (err <= 1.0f) {
            ++*acc;
            ++*nfcn;
            x = f2_add(x, h, 0.f);
            y[0] = ynew[0];
            y[1] = ynew[1];
            if (last) {  // the clipped last step says nothing about the ideal step
                active = false;
                continue;
            }
            float k0[2], fnext[8];
            bool ok_next = false;
            if (sparse) {  // plain first stage of the next step; no features, no proposal
                float yh2[2] = {y[0].hi, y[1].hi}, ys2[2] = {y[0].lo, y[1].lo};
                fl(x.hi, x.lo, yh2, ys2, k0, P);
            } else {
                ok_next = step_features(fl, x, y, P, k0, fnext);  // next step's stage 0
            }
            // Training samples: accepted steps that start and end inside the
            // velocity grid (a step across its edge meets the jump to zero
            // velocity, and its tiny "ideal" step would teach the network to
            // shorten steps everywhere).
            if (LOG && lead && feat_ok && ok_next) {
                const unsigned hv = hash32(pid ^ sink.seed, (unsigned)nstep);
                if ((float)(hv >> 8) * (1.0f / 16777216.0f) < sink.sample) {
                    unsigned long long k = atomicAdd(sink.count, 1ull);
                    if ((long long)k < sink.capacity) {
#pragma unroll
                        for (int i = 0; i < 8; ++i) sink.feats[k * 8 + i] = feat[i];
                        sink.targets[k] = __logf(fabsf(h) * safe / fmaxf(fac11, 1.0e-3f));
                    }
                }
            }
            if (!sparse) {
#pragma unroll
                for (int i = 0; i < 8; ++i) feat[i] = fnext[i];
            }
            feat_ok = ok_next;
            kc[0] = make_float2(k0[0], k0[1]);
            fresh = feat_ok;
            if (fabsf(hnew) > hmax) hnew = posneg * hmax;
            if (reject) hnew = posneg * fminf(fabsf(hnew), fabsf(h));
            reject = false;
        } else {
            hnew = h / fminf(facc1, fac11 * (1.0f / safe));
            reject = true;
            if (*acc >= 1) ++*rej;
            last = false;
            if (sparse) {  // features at the step start (its first stage is kept), then a proposal
                float k0[2];
                feat_ok = step_features(fl, x, y, P, k0, feat);
                ++*nfcn;
                fresh = feat_ok;
            }
        }
        h = hnew;
    }
    *status_out = status;
}

// No register cap: capping at 72 (7 blocks/SM) spills onto the L1 pipe that
// the spline gathers already saturate and measured 36% slower than the
// uncapped 96 registers.
template <class Flow, bool LOG, bool PROPOSE>
__global__ void __launch_bounds__(kThreads32)
learned_kernel(Flow fl, ParamsF P, double ts, double te, const double* __restrict__ x,
               const double* __restrict__ y, int nx, int ny, const uint8_t* __restrict__ mask,
               double* __restrict__ out, int32_t* __restrict__ status, int32_t* __restrict__ stats,
               float rtol, float atol, int nmax, long nthreads, const MlpBlob* __restrict__ Wg,
               int mode, LogSink sink)
{
    __shared__ float2 ks[12 * kThreads32];
    __shared__ MlpBlob W;
    __shared__ __align__(16) __nv_bfloat16 xs[kThreads32 / 32][32 * kMlpInPad];
    __shared__ float outs[kThreads32 / 32][32];
    if (PROPOSE) mlp_stage(Wg, &W);
    __syncthreads();
    float2* kc = ks + threadIdx.x;
    const int warp = threadIdx.x >> 5;
    const F2 xs0 = f2_from_double(ts), xe = f2_from_double(te);
    // uniform trip count: nthreads is a multiple of the block size
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nthreads;
         t += (long)gridDim.x * blockDim.x) {
        constexpr int LP = Flow::LP;  // lanes of a group hold the same particle
        int i, j;
        const bool valid = tile_particle<LP, kThreads32>(t, nx, ny, &i, &j);
        const bool lead = (threadIdx.x & (LP - 1)) == 0;
        const long k = valid ? (long)i * ny + j : 0;
        const bool live = valid && !(mask && mask[k]);
        F2 yv[2] = {f2_from_double(valid ? x[i] : 0.0), f2_from_double(valid ? y[j] : 0.0)};
        int st = NBCS_PARTICLE_MASKED, a = 0, rj = 0, nf = 0;
        solve32_warp<Flow, LOG, PROPOSE>(fl, P, xs0, xe, yv, rtol, atol, nmax, kc, live, &W,
                                         xs[warp], outs[warp], mode, sink, lead, (unsigned)k, &st,
                                         &a, &rj, &nf);
        if (!live) st = NBCS_PARTICLE_MASKED;
        if (valid && lead) {
            double2 res = live ? make_double2(f2_to_double(yv[0]), f2_to_double(yv[1]))
                               : make_double2(0.0, 0.0);
            if (out) reinterpret_cast<double2*>(out)[k] = res;
            if (status) status[k] = st;
            if (stats) {
                stats[3 * k] = a;
                stats[3 * k + 1] = rj;
                stats[3 * k + 2] = nf;
            }
        }
    }
}

static ParamsF to_float_p(const Params& P)
{
    ParamsF f;
    for (int i = 0; i < NBCS_MAX_PARAMS; ++i) f.v[i] = (float)P.v[i];
    return f;
}

template <bool LOG, bool PROPOSE>
static int launch_learned(const nbcs_flow* flow, const FlowmapArgs& a, const MlpBlob* W, int mode,
                          const LogSink& sink)
{
    if (flow->kind != NBCS_FLOW_SPLINE2D)
        return set_error(NBCS_ERR_UNSUPPORTED, "the learned step proposer needs a spline flow");
    if (flow->extrap != 0)
        return set_error(NBCS_ERR_UNSUPPORTED,
                         "the learned step proposer takes extrap_mode 'constant' only");
    SplineGridF g = make_grid_f(flow->grid);
    const float* c = flow->coef_uv32;
    float kd = (float)(180.0 / (3.141592653589793 * flow->r));
    // two lanes per particle (8 x 8 particle tiles per 128-thread block)
    constexpr int LPL = 2, TI = kThreads32 / LPL / 8;
    long tiles = (long)((a.nx + TI - 1) / TI) * ((a.ny + 7) / 8);
    long nthreads = tiles * kThreads32;
    long blocks = tiles;
    if (a.blocks_per_sm > 0 && blocks > (long)sm_count() * a.blocks_per_sm)
        blocks = (long)sm_count() * a.blocks_per_sm;
    ParamsF P = to_float_p(a.P);
#define NBCS_LAUNCH_LEARNED(SPH)                                                              \
    learned_kernel<FlowSpline32<SPH, LPL>, LOG, PROPOSE><<<(unsigned)blocks, kThreads32, 0, a.stream>>>( \
        FlowSpline32<SPH, LPL>{g, c, kd}, P, a.ts, a.te, a.x, a.y, a.nx, a.ny, a.mask, a.out,    \
        a.status, a.stats, (float)a.rtol, (float)a.atol, a.nmax, nthreads, W, mode, sink)
    switch (flow->spherical) {
    case 1: NBCS_LAUNCH_LEARNED(1); break;
    case 2: NBCS_LAUNCH_LEARNED(2); break;
    default: NBCS_LAUNCH_LEARNED(0); break;
    }
#undef NBCS_LAUNCH_LEARNED
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

int launch_flowmap32_learned(const nbcs_flow* flow, const FlowmapArgs& a, int mode)
{
    if ((reinterpret_cast<uintptr_t>(a.step_model) & 15))
        return set_error(NBCS_ERR_INVALID, "step_model blob must be 16-byte aligned");
    LogSink none = {nullptr, nullptr, 0, nullptr, 0.f, 0u};
    return launch_learned<false, true>(flow, a, static_cast<const MlpBlob*>(a.step_model), mode,
                                       none);
}

}  // namespace nbcs

using namespace nbcs;

extern "C" int nbcs_flowmap_log_steps(const nbcs_flow* flow, double t0, double T, const double* x,
                                      int32_t nx, const double* y, int32_t ny,
                                      const double* params, int32_t np, double rtol, double atol,
                                      float sample, uint32_t seed, float* feats, float* targets,
                                      int64_t capacity, unsigned long long* count, void* stream)
{
    NBCS_RANGE();
    int rc = validate_flow(flow, params, np, NBCS_PREC_MIXED);
    if (rc) return rc;
    if (nx < 0 || ny < 0 || !x || !y || !count || capacity < 0 || (capacity > 0 && (!feats || !targets)))
        return set_error(NBCS_ERR_INVALID, "log_steps: bad arguments");
    if ((long)nx * ny == 0) return NBCS_OK;
    FlowmapArgs a = {};
    for (int i = 0; i < NBCS_MAX_PARAMS; ++i) a.P.v[i] = i < np ? params[i] : 0.0;
    a.ts = params[0] * t0;
    a.te = params[0] * (t0 + T);
    a.x = x;
    a.y = y;
    a.nx = nx;
    a.ny = ny;
    a.rtol = rtol;
    a.atol = atol;
    a.nmax = 100000;
    a.stream = as_stream(stream);
    LogSink sink = {feats, targets, capacity, count, sample, seed};
    return launch_learned<true, false>(flow, a, nullptr, 0, sink);
}
