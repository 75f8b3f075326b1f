// Measurement helpers: a launch counter and FP32 / FP64 FMA throughput probes
// used as the compute roofline of the integrators.  No counterpart in the
// reference (it has no GPU path).
#include <atomic>

#include "nbcs_internal.cuh"

namespace nbcs {

static std::atomic<unsigned long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

template <class T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T* out, long iters, T a, T b)
{
    // 8 independent dependency chains per thread keep the FMA pipe full
    T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    T x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (long i = 0; i < iters; ++i) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == (T)-1.2345) out[blockIdx.x] = s;  // never true; keeps the chains alive
}

}  // namespace nbcs

using namespace nbcs;

extern "C" unsigned long long nbcs_launch_count(void) { return g_launches.load(); }

extern "C" int nbcs_probe_fma(int32_t precision, int64_t iters, void* sink, double* flops,
                              void* stream)
{
    NBCS_RANGE();
    if (iters < 1 || !sink || !flops) return set_error(NBCS_ERR_INVALID, "probe_fma: bad arguments");
    const int threads = 256;
    const long blocks = (long)sm_count() * 8;
    *flops = 2.0 * 8.0 * (double)iters * (double)threads * (double)blocks;
    if (precision == NBCS_PREC_FP64)
        fma_probe_kernel<double><<<(unsigned)blocks, threads, 0, as_stream(stream)>>>(
            static_cast<double*>(sink), iters, 0.999999, 1e-7);
    else
        fma_probe_kernel<float><<<(unsigned)blocks, threads, 0, as_stream(stream)>>>(
            static_cast<float*>(sink), iters, 0.999999f, 1e-7f);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}
