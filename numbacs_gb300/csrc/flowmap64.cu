// FP64 flow-map integration (the plain path) and the RHS probe entry point.
//
// Replaces flowmap_grid_2D (integration.py:123-182) with method="dop853":
// one thread per particle runs the FP64 DOP853 solver of dop853_64.cuh on a
// device-compiled right-hand side.  Compiled with -fmad=false.  The particle
// <-> thread map does not enter the arithmetic: results are the oracle's bit
// for bit whatever the tile shape.
#include "dop853_64.cuh"
#include "flows64.cuh"
#include "flowmap_common.cuh"

namespace nbcs {

// One 256-thread block per 32 x 8 tile of particles (warps of 4 x 8): as in
// the mixed kernel, the warps of a block follow neighbouring trajectories and
// share L1 lines (geophysical workload: 194 ms against 209 ms with one block
// per 128 consecutive particles of a row).
constexpr int kFm64Block = 256;

template <class Flow>
__global__ void __launch_bounds__(kFm64Block)
flowmap64_kernel(Flow fl, Params P, double ts, double te, const double* __restrict__ x,
                 const double* __restrict__ y, int nx, int nyv, AuxGrid aux,
                 const uint8_t* __restrict__ mask, double* __restrict__ out,
                 int32_t* __restrict__ status, int32_t* __restrict__ stats, double rtol,
                 double atol, int nmax)
{
    __shared__ double2 ks[12 * kFm64Block];
    double2* kc = ks + threadIdx.x;
    using S = TileShape<1, kFm64Block>;
    const long nthreads = (long)((nx + S::TI - 1) / S::TI) * ((nyv + S::TJ - 1) / S::TJ) * kFm64Block;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nthreads;
         t += (long)gridDim.x * blockDim.x) {
        int i, j;
        if (!tile_particle<1, kFm64Block>(t, nx, nyv, &i, &j)) continue;
        const long k = (long)i * nyv + j;
        if (!particle_exists(aux, k)) continue;
        double yv[2] = {0.0, 0.0}, x0, y0;
        int st = NBCS_PARTICLE_MASKED;
        Dop853Stats s = {0, 0, 0};
        if (particle_start(aux, x, y, mask, nx, i, j, &x0, &y0)) {
            yv[0] = x0;
            yv[1] = y0;
            st = dop853_solve64<Flow, kFm64Block>(fl, P, ts, te, yv, rtol, atol, nmax, kc, &s);
        }
        reinterpret_cast<double2*>(out)[k] = make_double2(yv[0], yv[1]);
        if (status) status[k] = st;
        if (stats) {
            stats[3 * k] = s.accepted;
            stats[3 * k + 1] = s.rejected;
            stats[3 * k + 2] = s.nfcn;
        }
    }
}

template <class Flow>
__global__ void rhs64_kernel(Flow fl, Params P, const double* __restrict__ ty, long n,
                             double* __restrict__ dy)
{
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long)gridDim.x * blockDim.x) {
        double yv[2] = {ty[3 * k + 1], ty[3 * k + 2]}, d[2];
        fl(ty[3 * k], yv, d, P);
        dy[2 * k] = d[0];
        dy[2 * k + 1] = d[1];
    }
}

struct Launch64 {
    const FlowmapArgs* a;
    template <class Flow>
    int operator()(const Flow& fl) const
    {
        using S = TileShape<1, kFm64Block>;
        const int threads = kFm64Block;
        long blocks = (long)((a->nx + S::TI - 1) / S::TI) * ((a->nyv() + S::TJ - 1) / S::TJ);
        if (a->blocks_per_sm > 0) {
            long cap = (long)sm_count() * a->blocks_per_sm;
            if (blocks > cap) blocks = cap;
        }
        if (blocks > (1L << 30)) blocks = 1L << 30;
        flowmap64_kernel<<<(unsigned)blocks, threads, 0, a->stream>>>(
            fl, a->P, a->ts, a->te, a->x, a->y, a->nx, a->nyv(), a->aux, a->mask, a->out,
            a->status, a->stats, a->rtol, a->atol, a->nmax);
        NBCS_LAUNCH_CHECK();
        return NBCS_OK;
    }
};

// flowmap_n / flowmap_n_grid_2D (integration.py:65-121, :468-534): one thread
// per point of a list, the positions at the n output times teval by dense
// output of one DOP853 run (16 stage slots per thread); masked points and the
// outputs past a failure stay 0.
constexpr int kDense64Block = 128;

template <class Flow>
__global__ void __launch_bounds__(kDense64Block)
flowmap64_n_kernel(Flow fl, Params P, const double* __restrict__ pts, long npts,
                   const double* __restrict__ teval, int n, const uint8_t* __restrict__ mask,
                   double2* __restrict__ out, int32_t* __restrict__ status, double rtol,
                   double atol, int nmax)
{
    __shared__ double2 ks[16 * kDense64Block];
    double2* kc = ks + threadIdx.x;
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npts) return;
    double2* o = out + k * n;
    for (int m = 0; m < n; ++m) o[m] = make_double2(0.0, 0.0);
    int st = NBCS_PARTICLE_MASKED;
    if (!(mask && mask[k])) {
        double yv[2] = {pts[2 * k], pts[2 * k + 1]};
        Dop853Stats s;
        st = dop853_solve64<Flow, kDense64Block, true>(fl, P, teval[0], teval[n - 1], yv, rtol,
                                                       atol, nmax, kc, &s, teval, n, o);
    }
    if (status) status[k] = st;
}

struct LaunchDense64 {
    Params P;
    const double* pts;
    long npts;
    const double* teval;
    int n;
    const uint8_t* mask;
    double* out;
    int32_t* status;
    double rtol, atol;
    int nmax;
    cudaStream_t stream;
    template <class Flow>
    int operator()(const Flow& fl) const
    {
        const long blocks = (npts + kDense64Block - 1) / kDense64Block;
        flowmap64_n_kernel<<<(unsigned)blocks, kDense64Block, 0, stream>>>(
            fl, P, pts, npts, teval, n, mask, reinterpret_cast<double2*>(out), status, rtol, atol,
            nmax);
        NBCS_LAUNCH_CHECK();
        return NBCS_OK;
    }
};

struct LaunchRhs64 {
    Params P;
    const double* ty;
    long n;
    double* dy;
    cudaStream_t stream;
    template <class Flow>
    int operator()(const Flow& fl) const
    {
        int threads = 128;
        long blocks = (n + threads - 1) / threads;
        if (blocks < 1) blocks = 1;
        rhs64_kernel<<<(unsigned)blocks, threads, 0, stream>>>(fl, P, ty, n, dy);
        NBCS_LAUNCH_CHECK();
        return NBCS_OK;
    }
};

template <class F>
static int dispatch64(const nbcs_flow* flow, const F& f)
{
    switch (flow->kind) {
    case NBCS_FLOW_DOUBLE_GYRE: return f(FlowDG64{});
    case NBCS_FLOW_BICKLEY: return f(FlowBickley64{});
    default: {
        SplineGrid g = make_grid(flow->grid);
        const double2* c = reinterpret_cast<const double2*>(flow->coef_uv);
        const double r = flow->r;
        switch (flow->spherical * 3 + flow->extrap) {  // validate_flow bounds both
        case 1: return f(FlowSpline64<0, 1>{g, c, r});
        case 2: return f(FlowSpline64<0, 2>{g, c, r});
        case 3: return f(FlowSpline64<1, 0>{g, c, r});
        case 4: return f(FlowSpline64<1, 1>{g, c, r});
        case 5: return f(FlowSpline64<1, 2>{g, c, r});
        case 6: return f(FlowSpline64<2, 0>{g, c, r});
        case 7: return f(FlowSpline64<2, 1>{g, c, r});
        case 8: return f(FlowSpline64<2, 2>{g, c, r});
        default: return f(FlowSpline64<0, 0>{g, c, r});
        }
    }
    }
}

int launch_flowmap64(const nbcs_flow* flow, const FlowmapArgs& a)
{
    return dispatch64(flow, Launch64{&a});
}

}  // namespace nbcs

using namespace nbcs;

extern "C" int nbcs_eval_rhs(const nbcs_flow* flow, const double* params, int32_t np,
                             const double* ty, int64_t n, double* dy, int32_t precision,
                             void* stream)
{
    NBCS_RANGE();
    int rc = validate_flow(flow, params, np, precision);
    if (rc) return rc;
    if (n < 0 || (n > 0 && (!ty || !dy))) return set_error(NBCS_ERR_INVALID, "eval_rhs: bad arrays");
    if (n == 0) return NBCS_OK;
    Params P = {};
    for (int i = 0; i < np; ++i) P.v[i] = params[i];
    if (precision == NBCS_PREC_MIXED) return launch_rhs32(flow, P, ty, n, dy, as_stream(stream));
    return dispatch64(flow, LaunchRhs64{P, ty, (long)n, dy, as_stream(stream)});
}

static int flowmap_particles(const nbcs_flow* flow, double t0, double T, const double* x,
                             int32_t nx, const double* y, int32_t ny, const double* params,
                             int32_t np, double rtol, double atol, const uint8_t* mask,
                             double* flowmap, int32_t* status, const nbcs_opts* opts,
                             void* stream, const AuxGrid& aux);

extern "C" int nbcs_flowmap_grid_2d(const nbcs_flow* flow, double t0, double T, const double* x,
                                    int32_t nx, const double* y, int32_t ny,
                                    const double* params, int32_t np, double rtol, double atol,
                                    const uint8_t* mask, double* flowmap, int32_t* status,
                                    const nbcs_opts* opts, void* stream)
{
    NBCS_RANGE();
    const AuxGrid plain = {0, ny, 1, 0.0, 0};
    return flowmap_particles(flow, t0, T, x, nx, y, ny, params, np, rtol, atol, mask, flowmap,
                             status, opts, stream, plain);
}

extern "C" int nbcs_flowmap_pts(const nbcs_flow* flow, double t0, double T, const double* pts,
                                int64_t npts, const double* params, int32_t np, double rtol,
                                double atol, const uint8_t* mask, double* flowmap, int32_t* status,
                                const nbcs_opts* opts, void* stream)
{
    NBCS_RANGE();
    if (npts < 0 || npts > 0x7fffffffL)
        return set_error(NBCS_ERR_INVALID, "flowmap_pts: npts must be in [0, 2^31)");
    if (opts && opts->step_model)
        return set_error(NBCS_ERR_UNSUPPORTED, "flowmap_pts: no step_model");
    const int W = kPointListColumns;
    const AuxGrid list = {kPointList, W, 0, 0.0, (long)npts};
    return flowmap_particles(flow, t0, T, pts, (int32_t)((npts + W - 1) / W), pts, W, params, np,
                             rtol, atol, mask, flowmap, status, opts, stream, list);
}

extern "C" int nbcs_flowmap_n_pts(const nbcs_flow* flow, const double* pts, int64_t npts,
                                  const double* teval, int32_t n, const double* params, int32_t np,
                                  double rtol, double atol, const uint8_t* mask, double* out,
                                  int32_t* status, const nbcs_opts* opts, void* stream)
{
    NBCS_RANGE();
    int rc = validate_flow(flow, params, np, NBCS_PREC_FP64);
    if (rc) return rc;
    if (opts && (opts->precision != NBCS_PREC_FP64 || opts->step_model))
        return set_error(NBCS_ERR_UNSUPPORTED, "flowmap_n: FP64 only, no step_model");
    if (npts < 0 || npts > (int64_t)1 << 30 || n < 1)
        return set_error(NBCS_ERR_INVALID, "flowmap_n: npts in [0, 2^30] and n >= 1");
    if (npts == 0) return NBCS_OK;
    if (!pts || !teval || !out || (reinterpret_cast<uintptr_t>(out) & 15))
        return set_error(NBCS_ERR_INVALID, "flowmap_n: NULL or misaligned array");
    if (!(rtol > 0.0) || !(atol > 0.0)) return set_error(NBCS_ERR_INVALID, "rtol/atol must be > 0");
    LaunchDense64 L;
    for (int i = 0; i < NBCS_MAX_PARAMS; ++i) L.P.v[i] = i < np ? params[i] : 0.0;
    L.pts = pts;
    L.npts = (long)npts;
    L.teval = teval;
    L.n = n;
    L.mask = mask;
    L.out = out;
    L.status = status;
    L.rtol = rtol;
    L.atol = atol;
    L.nmax = opts && opts->max_steps > 0 ? opts->max_steps : 100000;
    L.stream = as_stream(stream);
    return dispatch64(flow, L);
}

extern "C" int nbcs_flowmap_aux_grid_2d(const nbcs_flow* flow, double t0, double T,
                                        const double* x, int32_t nx, const double* y, int32_t ny,
                                        const double* params, int32_t np, double h,
                                        int32_t eig_main, int32_t compute_edge, double rtol,
                                        double atol, const uint8_t* mask, double* flowmap_aux,
                                        int32_t* status, const nbcs_opts* opts, void* stream)
{
    NBCS_RANGE();
    if (!(h > 0.0) && !(h < 0.0)) return set_error(NBCS_ERR_INVALID, "aux grid: h must be nonzero");
    if (opts && opts->step_model)
        return set_error(NBCS_ERR_UNSUPPORTED, "aux grid: no step_model");
    if ((long)nx * ny * (eig_main ? 5 : 4) > 0x7fffffffL)
        return set_error(NBCS_ERR_INVALID, "aux grid: too many particles");
    const AuxGrid aux = {eig_main ? 5 : 4, ny, compute_edge ? 1 : 0, h, 0};
    return flowmap_particles(flow, t0, T, x, nx, y, ny, params, np, rtol, atol, mask,
                             flowmap_aux, status, opts, stream, aux);
}

static int flowmap_particles(const nbcs_flow* flow, double t0, double T, const double* x,
                             int32_t nx, const double* y, int32_t ny, const double* params,
                             int32_t np, double rtol, double atol, const uint8_t* mask,
                             double* flowmap, int32_t* status, const nbcs_opts* opts,
                             void* stream, const AuxGrid& aux)
{
    nbcs_opts o = {};
    o.precision = NBCS_PREC_FP64;
    o.max_steps = 100000;
    if (opts) {
        o = *opts;
        if (o.max_steps <= 0) o.max_steps = 100000;
    }
    int rc = validate_flow(flow, params, np, o.precision);
    if (rc) return rc;
    if (nx < 0 || ny < 0) return set_error(NBCS_ERR_INVALID, "negative grid size");
    if ((long)nx * ny == 0) return NBCS_OK;
    if (!x || !y || !flowmap) return set_error(NBCS_ERR_INVALID, "flowmap_grid_2d: NULL array");
    if (reinterpret_cast<uintptr_t>(flowmap) & 15)
        return set_error(NBCS_ERR_INVALID, "flowmap_grid_2d: output must be 16-byte aligned");
    if (!(rtol > 0.0) || !(atol > 0.0)) return set_error(NBCS_ERR_INVALID, "rtol/atol must be > 0");
    FlowmapArgs a;
    for (int i = 0; i < NBCS_MAX_PARAMS; ++i) a.P.v[i] = i < np ? params[i] : 0.0;
    // t_eval = params[0] * linspace(t0, t0 + T, 2)   (integration.py:164)
    a.ts = params[0] * t0;
    a.te = params[0] * (t0 + T);
    a.x = x;
    a.y = y;
    a.nx = nx;
    a.ny = ny;
    a.aux = aux;
    a.mask = mask;
    a.out = flowmap;
    a.status = status;
    a.stats = o.stats;
    a.rtol = rtol;
    a.atol = atol;
    a.nmax = o.max_steps;
    a.threads = o.threads_per_block;
    a.blocks_per_sm = o.blocks_per_sm;
    a.lanes = o.lanes_per_particle;
    a.step_model = o.step_model;
    a.stream = as_stream(stream);
    if (o.step_model) {
        if (o.precision != NBCS_PREC_MIXED)
            return set_error(NBCS_ERR_UNSUPPORTED, "step_model needs precision NBCS_PREC_MIXED");
        if (o.step_model_mode < 0 || o.step_model_mode > 4)
            return set_error(NBCS_ERR_INVALID, "step_model_mode must be 0 .. 4");
        return launch_flowmap32_learned(flow, a, o.step_model_mode);
    }
    if (o.precision == NBCS_PREC_MIXED) return launch_flowmap32(flow, a);
    if (o.precision != NBCS_PREC_FP64) return set_error(NBCS_ERR_INVALID, "unknown precision");
    return launch_flowmap64(flow, a);
}
