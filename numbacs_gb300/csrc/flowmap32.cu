// Mixed-precision flow-map integration (NBCS_PREC_MIXED).
//
// Same DOP853 method and dop853 step-size controller as the FP64 path
// (dop853_64.cuh), but the stages, the RHS and the spline interpolation run
// on the FP32 pipe.  Particle position and time are carried as compensated
// FP32 pairs (hi + lo, ~48-bit significand) so that accumulating many steps
// keeps FP64-class accuracy; a stage argument is handed to the RHS as the
// pair (hi, lo + h*sum) and the RHS forms what it needs from it (flows32.cuh).
//
// Code shape (from the profile of the fully unrolled version, which was
// instruction-fetch bound): the twelve stages run as one rolled loop so the
// right-hand side is instantiated once; the stage derivatives live in shared
// memory (one column per particle, shared by its lanes) and the tableau is a
// set of compile-time constants (zero coefficients cost nothing).
//
// Work mapping: a group of LP lanes (1, 2 or 4) integrates one particle; the
// spline RHS splits its 4 time levels over the group.  Particles are taken in
// tiles of the (x, y) grid (8 along y) so neighbouring trajectories share
// coefficient cache lines and take similar step counts.
#include "dop853_32.cuh"
#include "flowmap_common.cuh"

namespace nbcs {

template <class Flow>
__global__ void __launch_bounds__(kFm32Block, kFm32MinBlocks)
flowmap32_kernel(Flow fl, ParamsF P, double ts, double te, const double* __restrict__ x,
                 const double* __restrict__ y, int nx, int nyv, AuxGrid aux,
                 const uint8_t* __restrict__ mask, double* __restrict__ out,
                 int32_t* __restrict__ status, int32_t* __restrict__ stats, float rtol,
                 float atol, int nmax, long nthreads)
{
    constexpr int LP = Flow::LP;
    // the LP lanes of a particle compute identical stage derivatives (the
    // split RHS ends in a butterfly sum): one shared column per particle, read
    // as a broadcast by its lanes
    constexpr int KS = kFm32Block / LP;
    __shared__ float2 ks[12 * KS];
    float2* kc = ks + threadIdx.x / LP;
    const F2 xs = f2_from_double(ts), xe = f2_from_double(te);
    // every lane of a group walks the same trip count (nthreads is a multiple of kFm32Block)
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nthreads;
         t += (long)gridDim.x * blockDim.x) {
        int i, j;
        if (!tile_particle<LP, kFm32Block, kFm32TileJ>(t, nx, nyv, &i, &j)) continue;
        long k = (long)i * nyv + j;
        if (!particle_exists(aux, k)) continue;  // uniform in a lane group
        double r0 = 0.0, r1 = 0.0, x0, y0;
        int st = NBCS_PARTICLE_MASKED, a = 0, rj = 0, nf = 0;
        if (particle_start(aux, x, y, mask, nx, i, j, &x0, &y0)) {
            F2 yv[2] = {f2_from_double(x0), f2_from_double(y0)};
            st = dop853_solve32<Flow, KS>(fl, P, xs, xe, yv, rtol, atol, nmax, kc, &a, &rj, &nf);
            r0 = f2_to_double(yv[0]);
            r1 = f2_to_double(yv[1]);
        }
        if (LP == 1 || (threadIdx.x & (LP - 1)) == 0) {
            reinterpret_cast<double2*>(out)[k] = make_double2(r0, r1);
            if (status) status[k] = st;
            if (stats) {
                stats[3 * k] = a;
                stats[3 * k + 1] = rj;
                stats[3 * k + 2] = nf;
            }
        }
    }
}

template <class Flow>
__global__ void __launch_bounds__(kThreads32)
rhs32_kernel(Flow fl, ParamsF P, const double* __restrict__ ty, long n, double* __restrict__ dy)
{
    constexpr int LP = Flow::LP;
    const long total = ((n * LP + kThreads32 - 1) / kThreads32) * kThreads32;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x) {
        long k = t / LP;
        long kk = k < n ? k : n - 1;  // idle lanes of the last group repeat a point
        F2 tt = f2_from_double(ty[3 * kk]), a = f2_from_double(ty[3 * kk + 1]),
           b = f2_from_double(ty[3 * kk + 2]);
        float yh[2] = {a.hi, b.hi}, ys[2] = {a.lo, b.lo}, d[2];
        fl(tt.hi, tt.lo, yh, ys, d, P);
        if (k < n && (t % LP) == 0) {
            dy[2 * k] = d[0];
            dy[2 * k + 1] = d[1];
        }
    }
}

static ParamsF to_float(const Params& P)
{
    ParamsF f;
    for (int i = 0; i < NBCS_MAX_PARAMS; ++i) f.v[i] = (float)P.v[i];
    return f;
}

template <int SPH, class F>
static int dispatch_lp(int lp, int xm, const SplineGridF& g, const float* c, float k, bool exact,
                       const F& f)
{
    // extrapolation beyond the grid box ("nearest", "linear"): the general
    // cell search only (fewer instantiations; the box test is the same)
    if (xm == 1) {
        switch (lp) {
        case 1: return f(FlowSpline32<SPH, 1, false, 1>{g, c, k});
        case 2: return f(FlowSpline32<SPH, 2, false, 1>{g, c, k});
        default: return f(FlowSpline32<SPH, 4, false, 1>{g, c, k});
        }
    }
    if (xm == 2) {
        switch (lp) {
        case 1: return f(FlowSpline32<SPH, 1, false, 2>{g, c, k});
        case 2: return f(FlowSpline32<SPH, 2, false, 2>{g, c, k});
        default: return f(FlowSpline32<SPH, 4, false, 2>{g, c, k});
        }
    }
    // grids whose nodes are floats on every axis (dyadic spacings) take the
    // cell search without compensated node sums: -3 % on the geophysical flow
    if (exact) {
        switch (lp) {
        case 1: return f(FlowSpline32<SPH, 1, true>{g, c, k});
        case 2: return f(FlowSpline32<SPH, 2, true>{g, c, k});
        default: return f(FlowSpline32<SPH, 4, true>{g, c, k});
        }
    }
    switch (lp) {
    case 1: return f(FlowSpline32<SPH, 1>{g, c, k});
    case 2: return f(FlowSpline32<SPH, 2>{g, c, k});
    default: return f(FlowSpline32<SPH, 4>{g, c, k});
    }
}

// lanes per particle for the spline RHS: explicit request, else enough groups
// to give every SM ~16 resident warps.
static int spline_lanes(int requested, long particles)
{
    if (requested == 1 || requested == 2 || requested == 4) return requested;
    long lanes_target = (long)sm_count() * 16 * 32;
    if (particles * 2 >= lanes_target) return 2;
    return 4;
}

template <class F>
static int dispatch32(const nbcs_flow* flow, int lp, const F& f)
{
    switch (flow->kind) {
    case NBCS_FLOW_DOUBLE_GYRE: return f(FlowDG32{});
    case NBCS_FLOW_BICKLEY: return f(FlowBickley32{});
    default: {
        SplineGridF g = make_grid_f(flow->grid);
        const float* c = flow->coef_uv32;
        float k = (float)(180.0 / (3.141592653589793 * flow->r));
        const bool ex = grid_nodes_exact_f(flow->grid);
        const int xm = flow->extrap;
        switch (flow->spherical) {
        case 1: return dispatch_lp<1>(lp, xm, g, c, k, ex, f);
        case 2: return dispatch_lp<2>(lp, xm, g, c, k, ex, f);
        default: return dispatch_lp<0>(lp, xm, g, c, k, ex, f);
        }
    }
    }
}

struct Launch32 {
    const FlowmapArgs* a;
    template <class Flow>
    int operator()(const Flow& fl) const
    {
        using S = TileShape<Flow::LP, kFm32Block, kFm32TileJ>;
        long tiles = (long)((a->nx + S::TI - 1) / S::TI) * ((a->nyv() + S::TJ - 1) / S::TJ);
        long nthreads = tiles * kFm32Block;
        long blocks = tiles;
        if (a->blocks_per_sm > 0) {
            long cap = (long)sm_count() * a->blocks_per_sm;
            if (blocks > cap) blocks = cap;
        }
        if (blocks > (1L << 30)) blocks = 1L << 30;
        flowmap32_kernel<<<(unsigned)blocks, kFm32Block, 0, a->stream>>>(
            fl, to_float(a->P), a->ts, a->te, a->x, a->y, a->nx, a->nyv(), a->aux, a->mask, a->out,
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
        long total = n * Flow::LP;
        long blocks = (total + kThreads32 - 1) / kThreads32;
        rhs32_kernel<<<(unsigned)blocks, kThreads32, 0, stream>>>(fl, P, ty, n, dy);
        NBCS_LAUNCH_CHECK();
        return NBCS_OK;
    }
};

int launch_flowmap32(const nbcs_flow* flow, const FlowmapArgs& a)
{
    int lp = spline_lanes(a.lanes, (long)a.nx * a.nyv());
    return dispatch32(flow, lp, Launch32{&a});
}

int launch_rhs32(const nbcs_flow* flow, const Params& P, const double* ty, long n, double* dy,
                 cudaStream_t stream)
{
    return dispatch32(flow, 4, LaunchRhs32{to_float(P), ty, n, dy, stream});
}

}  // namespace nbcs
