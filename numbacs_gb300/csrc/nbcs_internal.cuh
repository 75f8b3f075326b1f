// Internal helpers shared by the libnbcs translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include "../../include/nbcs.h"

namespace nbcs {

// Record a message for nbcs_last_error() (thread-local) and return `code`.
int set_error(int code, const char* fmt, ...);

#define NBCS_CUDA_TRY(expr)                                                        \
    do {                                                                           \
        cudaError_t e_ = (expr);                                                   \
        if (e_ != cudaSuccess)                                                     \
            return ::nbcs::set_error(NBCS_ERR_CUDA, "%s: %s (%s:%d)", #expr,         \
                                     cudaGetErrorString(e_), __FILE__, __LINE__);  \
    } while (0)

// Count one kernel launch (nbcs_launch_count) and surface launch errors.
void count_launch();
#define NBCS_LAUNCH_CHECK()                  \
    do {                                     \
        ::nbcs::count_launch();              \
        NBCS_CUDA_TRY(cudaGetLastError());   \
    } while (0)

// NVTX range over one C-ABI call, so that a timeline (Nsight Systems, or ncu
// with --nvtx) shows which entry point issued which kernels.  NVTX3 is
// header-only: without an attached tool each push/pop is a load and a branch.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
#define NBCS_RANGE() ::nbcs::NvtxRange nbcs_range_(__func__)

// Bounds-checked build (compiled with -DNBCS_CHECK; `python -m
// numbacs_gb300.build --check` builds it beside the normal library).  Every
// checked access (the data-dependent ones: spline gathers, composition
// gathers, labelling links) tests its index against the extent of its buffer;
// a failed test sets its bit (NBCS_CHECK_* in nbcs.h) in this translation
// unit's word and the access is skipped, so a bad index is reported by
// nbcs_check_bits instead of faulting the GPU.  In the normal build the test
// compiles to nothing.
#ifdef NBCS_CHECK
static __device__ unsigned int g_nbcs_check_word;
#define NBCS_CHECKED(cond, bit) \
    ((cond) ? true : (atomicOr(&g_nbcs_check_word, (unsigned)(bit)), false))
// each unit registers a reader of its own word with the library (capi.cu)
int register_check_reader(int (*read)(unsigned int* bits, int reset));
namespace {
int read_check_word(unsigned int* bits, int reset)
{
    unsigned int w = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&w, g_nbcs_check_word, sizeof(w));
    if (e != cudaSuccess) return (int)e;
    *bits |= w;
    if (reset) {
        const unsigned int zero = 0;
        e = cudaMemcpyToSymbol(g_nbcs_check_word, &zero, sizeof(zero));
    }
    return (int)e;
}
const int g_check_reader_registered = register_check_reader(&read_check_word);
}  // namespace
#else
#define NBCS_CHECKED(cond, bit) true
#endif

// Number of SMs of the current device (cached per device).
int sm_count();

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Flow parameters passed by value to kernels (params[0] is the integration
// direction, as in the reference's @cfunc right-hand sides).
struct Params {
    double v[NBCS_MAX_PARAMS];
};

// Uniform grid of a tricubic spline, with the per-axis reciprocal spacing
// (n-1)/(b-a) precomputed on the host exactly as the device would.
struct SplineGrid {
    double a[3], b[3], dinv[3];
    int n[3];
    int sx, st;  // node strides of the (nt+2, nx+2, ny+2) coefficient block
};

inline SplineGrid make_grid(const double* g)
{
    SplineGrid s;
    for (int d = 0; d < 3; ++d) {
        s.a[d] = g[3 * d];
        s.b[d] = g[3 * d + 1];
        s.n[d] = (int)g[3 * d + 2];
        s.dinv[d] = (double)(s.n[d] - 1) / (s.b[d] - s.a[d]);
    }
    s.sx = s.n[2] + 2;
    s.st = (s.n[1] + 2) * (s.n[2] + 2);
    return s;
}

int validate_flow(const nbcs_flow* flow, const double* params, int32_t np, int precision);

}  // namespace nbcs
