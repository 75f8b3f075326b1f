// Batched flow maps, plain FP64 path: the persistent work-stealing kernel of
// batch32.cu with the FP64 solver of dop853_64.cuh (compiled with
// -fmad=false, bit-compatible with the single-field FP64 kernel).
#include "batch_common.cuh"
#include "dop853_64.cuh"
#include "flows64.cuh"

namespace nbcs {

__global__ void batch64_reset_kernel(BatchHeader* hdr) { hdr->counter = 0ull; }

__global__ void __launch_bounds__(kBatchThreads)
batch64_kernel(BatchHeader* hdr, const DevFlow64* __restrict__ flows,
               const DevField* __restrict__ fields, int nfields, int nmax)
{
    __shared__ double2 ks[12 * kThreads64];
    double2* kc = ks + threadIdx.x;
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
        if (!batch_particle(F, (long long)c, lane, &i, &j)) continue;
        const long p = (long)i * F.ny + j;
        double yv[2] = {0.0, 0.0};
        int st = NBCS_PARTICLE_MASKED;
        Dop853Stats s = {0, 0, 0};
        if (!(F.mask && F.mask[p])) {
            yv[0] = F.x[i];
            yv[1] = F.y[j];
            const DevFlow64& fl = flows[F.flow];
            switch (fl.kind) {
            case NBCS_FLOW_DOUBLE_GYRE:
                st = dop853_solve64(FlowDG64{}, F.P, F.ts, F.te, yv, F.rtol, F.atol, nmax, kc, &s);
                break;
            case NBCS_FLOW_BICKLEY:
                st = dop853_solve64(FlowBickley64{}, F.P, F.ts, F.te, yv, F.rtol, F.atol, nmax, kc,
                                    &s);
                break;
            default:
                if (fl.spherical == 1)
                    st = dop853_solve64(FlowSpline64<1>{fl.g, fl.c, fl.r}, F.P, F.ts, F.te, yv,
                                        F.rtol, F.atol, nmax, kc, &s);
                else if (fl.spherical == 2)
                    st = dop853_solve64(FlowSpline64<2>{fl.g, fl.c, fl.r}, F.P, F.ts, F.te, yv,
                                        F.rtol, F.atol, nmax, kc, &s);
                else
                    st = dop853_solve64(FlowSpline64<0>{fl.g, fl.c, fl.r}, F.P, F.ts, F.te, yv,
                                        F.rtol, F.atol, nmax, kc, &s);
                break;
            }
        }
        reinterpret_cast<double2*>(F.out)[p] = make_double2(yv[0], yv[1]);
        if (F.status) F.status[p] = st;
    }
}

int launch_batch64(const BatchHeader* dev_hdr, const DevFlow64* flows, const DevField* fields,
                   int nfields, int blocks_per_sm, int nmax, cudaStream_t s)
{
    BatchHeader* hdr = const_cast<BatchHeader*>(dev_hdr);
    batch64_reset_kernel<<<1, 1, 0, s>>>(hdr);
    NBCS_LAUNCH_CHECK();
    int per_sm = blocks_per_sm;
    if (per_sm <= 0 &&
        (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch64_kernel, kBatchThreads, 0) !=
             cudaSuccess ||
         per_sm <= 0))
        per_sm = 4;
    batch64_kernel<<<per_sm * sm_count(), kBatchThreads, 0, s>>>(hdr, flows, fields, nfields, nmax);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

}  // namespace nbcs
