// Batched flow maps: many FTLE fields (different flows, t0, T, grid sizes) in
// one persistent launch, and the host side of nbcs_batch_prepare / _run.
//
// The reference computes a time series of FTLE fields with a Python loop that
// calls flowmap_grid_2D and ftle_grid_2D once per t0
// (examples/time_series/plot_dg_time_series.py, plot_dg_numbacs_vs_scipy.py).
// Here every particle of every field is one work item: warps of a persistent
// grid take 32-particle chunks from a shared atomic counter, so a field with
// long trajectories or a big grid spreads over the whole GPU instead of
// leaving SMs idle at the end of a per-field launch.  The counter is reset by
// a one-thread kernel at the start of every run, so a run is two or three
// kernel launches and can be captured in a CUDA graph.
#include <algorithm>
#include <vector>

#include "batch_common.cuh"
#include "dop853_32.cuh"
#include "flowmap_common.cuh"

namespace nbcs {

__global__ void batch_reset_kernel(BatchHeader* hdr) { hdr->counter = 0ull; }

// Integrate particle (i, j) of field F and write its flow map and status
// (the group's leader lane writes).  `lane` is the thread's lane in its warp;
// KS is the block size (the stride of the stage-derivative column kc).
template <int KS>
__device__ __forceinline__ void batch_solve32(const DevFlow32* __restrict__ flows,
                                              const DevField& F, int i, int j, int lane,
                                              float2* kc, int nmax)
{
    const long p = (long)i * F.ny + j;
    double r0 = 0.0, r1 = 0.0;
    int st = NBCS_PARTICLE_MASKED, a = 0, rj = 0, nf = 0;
    if (!(F.mask && F.mask[p])) {
        ParamsF P;
#pragma unroll
        for (int q = 0; q < NBCS_MAX_PARAMS; ++q) P.v[q] = (float)F.P.v[q];
        const F2 xs = f2_from_double(F.ts), xe = f2_from_double(F.te);
        const float rtol = (float)F.rtol, atol = (float)F.atol;
        F2 yv[2] = {f2_from_double(F.x[i]), f2_from_double(F.y[j])};
        const DevFlow32& fl = flows[F.flow];
        switch (fl.kind) {
        case NBCS_FLOW_DOUBLE_GYRE:
            st = dop853_solve32<FlowDG32, KS>(FlowDG32{}, P, xs, xe, yv, rtol, atol, nmax, kc, &a,
                                              &rj, &nf);
            break;
        case NBCS_FLOW_BICKLEY:
            st = dop853_solve32<FlowBickley32, KS>(FlowBickley32{}, P, xs, xe, yv, rtol, atol,
                                                   nmax, kc, &a, &rj, &nf);
            break;
        default:  // spline fields run two lanes per particle
#define NBCS_SPLINE_SOLVE(SPH, LP)                                                              \
    st = dop853_solve32<FlowSpline32<SPH, LP>, KS>(FlowSpline32<SPH, LP>{fl.g, fl.c,           \
                                                                        fl.deg_per_km},     \
                                                   P, xs, xe, yv, rtol, atol, nmax, kc, &a,   \
                                                   &rj, &nf)
            if (F.lp == 2) {
                if (fl.spherical == 1) NBCS_SPLINE_SOLVE(1, 2);
                else if (fl.spherical == 2) NBCS_SPLINE_SOLVE(2, 2);
                else NBCS_SPLINE_SOLVE(0, 2);
            } else {
                if (fl.spherical == 1) NBCS_SPLINE_SOLVE(1, 1);
                else if (fl.spherical == 2) NBCS_SPLINE_SOLVE(2, 1);
                else NBCS_SPLINE_SOLVE(0, 1);
            }
#undef NBCS_SPLINE_SOLVE
            break;
        }
        r0 = f2_to_double(yv[0]);
        r1 = f2_to_double(yv[1]);
    }
    if ((lane % F.lp) == 0) {
        reinterpret_cast<double2*>(F.out)[p] = make_double2(r0, r1);
        if (F.status) F.status[p] = st;
    }
}

// persistent schedule: warps take 32-particle chunks from the shared counter
__global__ void __launch_bounds__(kBatchThreads)
batch32_kernel(BatchHeader* hdr, const DevFlow32* __restrict__ flows,
               const DevField* __restrict__ fields, int nfields, int nmax)
{
    __shared__ float2 ks[12 * kThreads32];
    float2* kc = ks + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const long long total = hdr->total_chunks;
    for (;;) {
        unsigned long long c = 0ull;
        if (lane == 0) c = atomicAdd(&hdr->counter, 1ull);
        c = __shfl_sync(0xffffffffu, c, 0);
        if ((long long)c >= total) break;
        const int f = batch_find<kByChunk>(fields, nfields, (long long)c);
        const DevField& F = fields[f];
        int i, j;
        if (!batch_particle(F, (long long)c, lane, &i, &j)) continue;  // whole lane group
        batch_solve32<kThreads32>(flows, F, i, j, lane, kc, nmax);
    }
}

// Tile schedule, one launch per flow class: block b integrates tile b of the
// class's fields (field table ordered longest first), with the single-field
// integrator's block (256 threads), tile map (16 x 8 particles at two lanes
// a particle, 32 x 8 at one) and register budget (3 resident blocks).  The
// kernel is instantiated for one right-hand side, so it keeps the
// single-field kernel's 80 registers where one kernel for every flow kind
// took 128 (2 blocks per SM); each particle's arithmetic is the single-field
// kernel's, so the results are bit-identical to it.
// The right-hand side of a field: the kernel argument when every field of the
// class uses one flow (UNIFORM: the single-field kernel's form, read from the
// constant bank), else rebuilt from the flow table.
template <class Flow>
struct FlowFromDev {
    __device__ static Flow make(const DevFlow32&) { return Flow{}; }
};
template <int SPH, int LP, bool EX>
struct FlowFromDev<FlowSpline32<SPH, LP, EX>> {
    __device__ static FlowSpline32<SPH, LP, EX> make(const DevFlow32& f)
    {
        return FlowSpline32<SPH, LP, EX>{f.g, f.c, f.deg_per_km};
    }
};

template <class Flow, bool UNIFORM>
__global__ void __launch_bounds__(kFm32Block, kFm32MinBlocks)
batch32_class_kernel(Flow fl0, const DevFlow32* __restrict__ flows,
                     const DevField* __restrict__ fields, int nfields, int nmax)
{
    constexpr int LP = Flow::LP;
    constexpr int KS = kFm32Block / LP;  // one stage column per particle, shared by its lanes
    __shared__ float2 ks[12 * KS];
    __shared__ ParamsF sP;  // the block's field is uniform: its parameters once per block
    float2* kc = ks + threadIdx.x / LP;
    const long long b = blockIdx.x;
    const DevField& F = fields[batch_find<kByTile>(fields, nfields, b)];
    if (threadIdx.x < NBCS_MAX_PARAMS) sP.v[threadIdx.x] = (float)F.P.v[threadIdx.x];
    __syncthreads();
    const long t = (long)(b - F.tile0) * kFm32Block + threadIdx.x;
    int i, j;
    // the lanes of a group share the particle: they leave together
    if (!tile_particle<LP, kFm32Block, kFm32TileJ>(t, F.nx, F.ny, &i, &j)) return;
    const long p = (long)i * F.ny + j;
    double r0 = 0.0, r1 = 0.0;
    int st = NBCS_PARTICLE_MASKED, a = 0, rj = 0, nf = 0;
    if (!(F.mask && F.mask[p])) {
        F2 yv[2] = {f2_from_double(F.x[i]), f2_from_double(F.y[j])};
        st = dop853_solve32<Flow, KS>(UNIFORM ? fl0 : FlowFromDev<Flow>::make(flows[F.flow]), sP,
                                      f2_from_double(F.ts), f2_from_double(F.te), yv,
                                      (float)F.rtol, (float)F.atol, nmax, kc, &a, &rj, &nf);
        r0 = f2_to_double(yv[0]);
        r1 = f2_to_double(yv[1]);
    }
    if (LP == 1 || (threadIdx.x & (LP - 1)) == 0) {
        reinterpret_cast<double2*>(F.out)[p] = make_double2(r0, r1);
        if (F.status) F.status[p] = st;
    }
}

template <class Flow>
static int launch_class(const nbcs_batch_class& c, const Flow& fl, const DevFlow32* flows,
                        const DevField* fields, int nmax, cudaStream_t s)
{
    if (c.flow >= 0)
        batch32_class_kernel<Flow, true><<<(unsigned)c.tiles, kFm32Block, 0, s>>>(
            fl, flows, fields + c.field0, c.nfields, nmax);
    else
        batch32_class_kernel<Flow, false><<<(unsigned)c.tiles, kFm32Block, 0, s>>>(
            fl, flows, fields + c.field0, c.nfields, nmax);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

template <int SPH, bool EX>
static int launch_spline_class(const nbcs_batch_class& c, const DevFlow32* flows,
                               const DevField* fields, int nmax, cudaStream_t s)
{
    FlowSpline32<SPH, 2, EX> fl{};
    if (c.flow >= 0)
        fl = FlowSpline32<SPH, 2, EX>{make_grid_f(c.grid), c.coef_uv32,
                                      (float)(180.0 / (3.141592653589793 * c.r))};
    return launch_class(c, fl, flows, fields, nmax, s);
}

int launch_batch32_class(const nbcs_batch_class& c, const DevFlow32* flows,
                         const DevField* fields, int nmax, cudaStream_t s)
{
    if (c.tiles <= 0) return NBCS_OK;
    if (c.tiles > 0x7fffffffLL) return set_error(NBCS_ERR_UNSUPPORTED, "batch: too many tiles");
    switch (c.kind) {
    case NBCS_FLOW_DOUBLE_GYRE: return launch_class(c, FlowDG32{}, flows, fields, nmax, s);
    case NBCS_FLOW_BICKLEY: return launch_class(c, FlowBickley32{}, flows, fields, nmax, s);
    default:
        switch (c.spherical * 2 + (c.exact_nodes ? 1 : 0)) {
        case 1: return launch_spline_class<0, true>(c, flows, fields, nmax, s);
        case 2: return launch_spline_class<1, false>(c, flows, fields, nmax, s);
        case 3: return launch_spline_class<1, true>(c, flows, fields, nmax, s);
        case 4: return launch_spline_class<2, false>(c, flows, fields, nmax, s);
        case 5: return launch_spline_class<2, true>(c, flows, fields, nmax, s);
        default: return launch_spline_class<0, false>(c, flows, fields, nmax, s);
        }
    }
}

static int persistent_blocks(const void* kernel, int threads, int blocks_per_sm)
{
    int per_sm = blocks_per_sm;
    if (per_sm <= 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess ||
            per_sm <= 0)
            per_sm = 4;
    }
    return per_sm * sm_count();
}

int launch_batch32(const BatchHeader* dev_hdr, const DevFlow32* flows, const DevField* fields,
                   int nfields, int blocks_per_sm, int nmax, cudaStream_t s)
{
    BatchHeader* hdr = const_cast<BatchHeader*>(dev_hdr);
    batch_reset_kernel<<<1, 1, 0, s>>>(hdr);
    NBCS_LAUNCH_CHECK();
    int blocks = persistent_blocks((const void*)batch32_kernel, kBatchThreads, blocks_per_sm);
    batch32_kernel<<<blocks, kBatchThreads, 0, s>>>(hdr, flows, fields, nfields, nmax);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

int batch_blocks_for(const void* kernel, int blocks_per_sm)
{
    return persistent_blocks(kernel, kBatchThreads, blocks_per_sm);
}

}  // namespace nbcs

using namespace nbcs;

extern "C" size_t nbcs_batch_scratch_bytes(int32_t nflows, int32_t nfields)
{
    if (nflows < 1 || nfields < 1) return 0;
    return batch_layout(nflows, nfields).total;
}

extern "C" int nbcs_batch_prepare(const nbcs_flow* flows, int32_t nflows, const nbcs_field* fields,
                                  int32_t nfields, int32_t precision, void* scratch,
                                  size_t scratch_bytes, nbcs_batch* plan, void* stream)
{
    NBCS_RANGE();
    if (!flows || !fields || !plan || nflows < 1 || nfields < 1)
        return set_error(NBCS_ERR_INVALID, "batch_prepare: need >= 1 flow and >= 1 field");
    if (precision != NBCS_PREC_FP64 && precision != NBCS_PREC_MIXED)
        return set_error(NBCS_ERR_INVALID, "batch_prepare: unknown precision %d", precision);
    const BatchLayout lay = batch_layout(nflows, nfields);
    if (!scratch || scratch_bytes < lay.total || (reinterpret_cast<uintptr_t>(scratch) & 255))
        return set_error(NBCS_ERR_SCRATCH, "batch_prepare: scratch needs %zu bytes, 256-aligned",
                         lay.total);
    std::vector<unsigned char> host(lay.total, 0);
    BatchHeader* hdr = reinterpret_cast<BatchHeader*>(host.data());
    DevFlow32* f32 = reinterpret_cast<DevFlow32*>(host.data() + lay.off_f32);
    DevFlow64* f64 = reinterpret_cast<DevFlow64*>(host.data() + lay.off_f64);
    DevField* df = reinterpret_cast<DevField*>(host.data() + lay.off_fields);
    for (int k = 0; k < nflows; ++k) {
        const nbcs_flow& fl = flows[k];
        f32[k].kind = f64[k].kind = fl.kind;
        f32[k].spherical = f64[k].spherical = fl.spherical;
        if (fl.kind == NBCS_FLOW_SPLINE2D) {
            f32[k].g = make_grid_f(fl.grid);
            f64[k].g = make_grid(fl.grid);
        }
        f32[k].c = fl.coef_uv32;
        f64[k].c = reinterpret_cast<const double2*>(fl.coef_uv);
        f32[k].deg_per_km = (float)(180.0 / (3.141592653589793 * fl.r));
        f64[k].r = fl.r;
    }
    // validate, then classify: fields that share one integrator
    // instantiation (flow kind; for splines the spherical mode and float
    // nodes) form a class, launched as one tile kernel
    std::vector<int> cls(nfields);
    int nclasses = 0;
    nbcs_batch_class classes[NBCS_BATCH_MAX_CLASSES] = {};
    for (int k = 0; k < nfields; ++k) {
        const nbcs_field& F = fields[k];
        if (F.flow < 0 || F.flow >= nflows)
            return set_error(NBCS_ERR_INVALID, "batch field %d: flow index %d out of range", k, F.flow);
        int rc = validate_flow(&flows[F.flow], F.params, F.np, precision);
        if (rc) return rc;
        if (flows[F.flow].kind == NBCS_FLOW_SPLINE2D && flows[F.flow].extrap != 0)
            return set_error(NBCS_ERR_UNSUPPORTED,
                             "batch field %d: the batched kernels take extrap_mode 'constant' "
                             "only; run such fields through nbcs_flowmap_grid_2d", k);
        if (F.nx < 0 || F.ny < 0 || ((long)F.nx * F.ny > 0 && (!F.x || !F.y || !F.flowmap)))
            return set_error(NBCS_ERR_INVALID, "batch field %d: bad grid or NULL array", k);
        if (!(F.rtol > 0.0) || !(F.atol > 0.0))
            return set_error(NBCS_ERR_INVALID, "batch field %d: rtol/atol must be > 0", k);
        if ((reinterpret_cast<uintptr_t>(F.flowmap) | reinterpret_cast<uintptr_t>(F.evec_max)) & 15)
            return set_error(NBCS_ERR_INVALID, "batch field %d: outputs must be 16-byte aligned", k);
        if (F.ftle && !F.evec_max)
            return set_error(NBCS_ERR_INVALID, "batch field %d: ftle needs evec_max", k);
        const nbcs_flow& fl = flows[F.flow];
        const bool spline = fl.kind == NBCS_FLOW_SPLINE2D;
        nbcs_batch_class key = {};
        key.kind = fl.kind;
        key.spherical = spline ? fl.spherical : 0;
        key.exact_nodes = spline && grid_nodes_exact_f(fl.grid) ? 1 : 0;
        key.lanes = (precision == NBCS_PREC_MIXED && spline) ? 2 : 1;
        int c = 0;
        while (c < nclasses && !(classes[c].kind == key.kind &&
                                 classes[c].spherical == key.spherical &&
                                 classes[c].exact_nodes == key.exact_nodes))
            ++c;
        if (c == nclasses) {
            if (nclasses == NBCS_BATCH_MAX_CLASSES)
                return set_error(NBCS_ERR_UNSUPPORTED, "batch: more than %d flow classes",
                                 NBCS_BATCH_MAX_CLASSES);
            key.flow = F.flow;
            key.r = fl.r;
            for (int q = 0; q < 9; ++q) key.grid[q] = fl.grid[q];
            key.coef_uv32 = fl.coef_uv32;
            classes[nclasses++] = key;
        } else if (classes[c].flow != F.flow) {
            classes[c].flow = -1;  // fields of several flows: each block reads its own
        }
        cls[k] = c;
    }
    // field table order: by class, then longest first (|T|, then particles),
    // so each class's tiles run longest first and the last tiles are short
    std::vector<int> order(nfields);
    for (int k = 0; k < nfields; ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int p, int q) {
        if (cls[p] != cls[q]) return cls[p] < cls[q];
        const double tp = fabs(fields[p].T), tq = fabs(fields[q].T);
        if (tp != tq) return tp > tq;
        return (long)fields[p].nx * fields[p].ny > (long)fields[q].nx * fields[q].ny;
    });
    long long chunks = 0, blocks = 0, tiles = 0, class_tiles = 0;
    for (int k = 0; k < nfields; ++k) {
        const nbcs_field& F = fields[order[k]];
        nbcs_batch_class& C = classes[cls[order[k]]];
        if (C.nfields == 0) {  // classes are contiguous in `order`
            C.field0 = k;
            class_tiles = 0;
        }
        C.nfields++;
        DevField& D = df[k];
        D.flow = F.flow;
        D.nx = F.nx;
        D.ny = F.ny;
        D.has_ftle = F.ftle != nullptr;
        for (int q = 0; q < NBCS_MAX_PARAMS; ++q) D.P.v[q] = q < F.np ? F.params[q] : 0.0;
        D.ts = F.params[0] * F.t0;  // t_eval = params[0] * linspace(t0, t0 + T, 2)
        D.te = F.params[0] * (F.t0 + F.T);
        D.rtol = F.rtol;
        D.atol = F.atol;
        D.den = 2.0 * fabs(F.T);
        D.dx = F.dx;
        D.dy = F.dy;
        // the fused FTLE stencil's reciprocals, as nbcs_ftle_evec_2d forms them
        D.rden = 1.0 / (2.0 * fabs(F.T));
        D.rdx = 1.0 / (2.0 * F.dx);
        D.rdy = 1.0 / (2.0 * F.dy);
        D.x = F.x;
        D.y = F.y;
        D.mask = F.mask;
        D.out = F.flowmap;
        D.status = F.status;
        D.ftle = F.ftle;
        D.evec = F.evec_max;
        D.lp = C.lanes;
        D.chunk0 = chunks;
        D.block0 = blocks;
        D.tile0 = class_tiles;  // tiles are counted within the class
        long n = (long)F.nx * F.ny;
        const int tj = batch_tile_j(D.lp);
        chunks += (long long)((F.nx + kBatchTileI - 1) / kBatchTileI) * ((F.ny + tj - 1) / tj);
        if (F.ftle) blocks += (n + kFtleBlock - 1) / kFtleBlock;
        // block tile of the class kernels: (ti x tj) particles
        const int ti = D.lp == 2 ? TileShape<2, kFm32Block>::TI : TileShape<1, kFm32Block>::TI;
        const int tjt = D.lp == 2 ? TileShape<2, kFm32Block>::TJ : TileShape<1, kFm32Block>::TJ;
        const long long ft = (long long)((F.nx + ti - 1) / ti) * ((F.ny + tjt - 1) / tjt);
        class_tiles += ft;
        C.tiles += ft;
        tiles += ft;
    }
    hdr->counter = 0;
    hdr->total_chunks = chunks;
    hdr->nfields = nfields;
    hdr->nflows = nflows;
    NBCS_CUDA_TRY(cudaMemcpyAsync(scratch, host.data(), lay.total, cudaMemcpyHostToDevice,
                                  as_stream(stream)));
    // pageable source: the call returns once the bytes are staged, so `host` may go
    plan->scratch = scratch;
    plan->nflows = nflows;
    plan->nfields = nfields;
    plan->precision = precision;
    plan->reserved = 0;
    plan->total_chunks = chunks;
    plan->ftle_blocks = blocks;
    plan->tiles = tiles;
    plan->nclasses = nclasses;
    plan->reserved2 = 0;
    for (int c = 0; c < NBCS_BATCH_MAX_CLASSES; ++c)
        plan->classes[c] = c < nclasses ? classes[c] : nbcs_batch_class{};
    return NBCS_OK;
}

static const DevField* plan_fields(const nbcs_batch* plan)
{
    const BatchLayout lay = batch_layout(plan->nflows, plan->nfields);
    return reinterpret_cast<const DevField*>(static_cast<unsigned char*>(plan->scratch) +
                                             lay.off_fields);
}

extern "C" int nbcs_batch_run_class(const nbcs_batch* plan, int32_t k, const nbcs_opts* opts,
                                    void* stream)
{
    NBCS_RANGE();
    if (!plan || !plan->scratch) return set_error(NBCS_ERR_INVALID, "batch_run_class: no plan");
    if (plan->precision != NBCS_PREC_MIXED)
        return set_error(NBCS_ERR_UNSUPPORTED, "batch_run_class: mixed-precision plans only");
    if (k < 0 || k >= plan->nclasses)
        return set_error(NBCS_ERR_INVALID, "batch_run_class: class %d of %d", k, plan->nclasses);
    const BatchLayout lay = batch_layout(plan->nflows, plan->nfields);
    const DevFlow32* f32 = reinterpret_cast<const DevFlow32*>(
        static_cast<unsigned char*>(plan->scratch) + lay.off_f32);
    const int nmax = (opts && opts->max_steps > 0) ? opts->max_steps : 100000;
    return launch_batch32_class(plan->classes[k], f32, plan_fields(plan), nmax, as_stream(stream));
}

extern "C" int nbcs_batch_run_ftle(const nbcs_batch* plan, void* stream)
{
    NBCS_RANGE();
    if (!plan || !plan->scratch) return set_error(NBCS_ERR_INVALID, "batch_run_ftle: no plan");
    if (plan->ftle_blocks <= 0) return NBCS_OK;
    return launch_ftle_batch(plan_fields(plan), plan->nfields, plan->ftle_blocks,
                             as_stream(stream));
}

extern "C" int nbcs_batch_run(const nbcs_batch* plan, const nbcs_opts* opts, void* stream)
{
    NBCS_RANGE();
    if (!plan || !plan->scratch) return set_error(NBCS_ERR_INVALID, "batch_run: no plan");
    const BatchLayout lay = batch_layout(plan->nflows, plan->nfields);
    unsigned char* base = static_cast<unsigned char*>(plan->scratch);
    const BatchHeader* hdr = reinterpret_cast<const BatchHeader*>(base);
    const DevField* fields = plan_fields(plan);
    const int bps = opts ? opts->blocks_per_sm : 0;
    const int nmax = (opts && opts->max_steps > 0) ? opts->max_steps : 100000;
    cudaStream_t s = as_stream(stream);
    int rc;
    if (plan->total_chunks > 0) {
        const DevFlow32* f32 = reinterpret_cast<const DevFlow32*>(base + lay.off_f32);
        if (plan->precision == NBCS_PREC_MIXED && bps < 0) {
            for (int c = 0; c < plan->nclasses; ++c) {
                rc = launch_batch32_class(plan->classes[c], f32, fields, nmax, s);
                if (rc) return rc;
            }
            rc = NBCS_OK;
        } else if (plan->precision == NBCS_PREC_MIXED) {
            rc = launch_batch32(hdr, f32, fields, plan->nfields, bps, nmax, s);
        } else {
            rc = launch_batch64(hdr, reinterpret_cast<const DevFlow64*>(base + lay.off_f64), fields,
                                plan->nfields, bps, nmax, s);
        }
        if (rc) return rc;
    }
    if (plan->ftle_blocks > 0) return launch_ftle_batch(fields, plan->nfields, plan->ftle_blocks, s);
    return NBCS_OK;
}
