// Host-side helpers of the C ABI: error reporting, device queries, flow checks.
#include <stdarg.h>
#include <stdio.h>

#include <mutex>

#include "nbcs_internal.cuh"

namespace nbcs {

static thread_local char g_err[512] = "";

int set_error(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int sm_count()
{
    static std::mutex mu;
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    std::lock_guard<std::mutex> lk(mu);
    if (cache[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 148;
        cache[dev] = n;
    }
    return cache[dev];
}

int validate_flow(const nbcs_flow* flow, const double* params, int32_t np, int precision)
{
    if (!flow) return set_error(NBCS_ERR_INVALID, "flow is NULL");
    if (np < 1 || np > NBCS_MAX_PARAMS || !params)
        return set_error(NBCS_ERR_INVALID, "params: need 1..%d values, got %d", NBCS_MAX_PARAMS, np);
    switch (flow->kind) {
    case NBCS_FLOW_DOUBLE_GYRE:
        if (np < 6) return set_error(NBCS_ERR_INVALID, "double gyre needs 6 params, got %d", np);
        break;
    case NBCS_FLOW_BICKLEY:
        if (np < 12) return set_error(NBCS_ERR_INVALID, "Bickley jet needs 12 params, got %d", np);
        break;
    case NBCS_FLOW_SPLINE2D: {
        if (flow->spherical < 0 || flow->spherical > 2)
            return set_error(NBCS_ERR_INVALID, "spherical must be 0, 1 or 2");
        if (flow->extrap < 0 || flow->extrap > 2)
            return set_error(NBCS_ERR_INVALID,
                             "extrap must be 0 (constant), 1 (nearest) or 2 (linear), got %d",
                             flow->extrap);
        for (int d = 0; d < 3; ++d) {
            double n = flow->grid[3 * d + 2];
            if (!(n >= 2.0) || !(flow->grid[3 * d + 1] > flow->grid[3 * d]))
                return set_error(NBCS_ERR_INVALID, "spline grid axis %d needs n >= 2 and b > a", d);
        }
        if (!flow->coef_uv) return set_error(NBCS_ERR_INVALID, "spline flow without coefficients");
        if (precision == NBCS_PREC_MIXED && !flow->coef_uv32)
            return set_error(NBCS_ERR_INVALID, "mixed precision needs the FP32 coefficient copy");
        if (precision == NBCS_PREC_MIXED && (reinterpret_cast<uintptr_t>(flow->coef_uv32) & 31))
            return set_error(NBCS_ERR_INVALID, "the FP32 coefficient copy must be 32-byte aligned");
        // the mixed path indexes quad entries with 32-bit integers
        if (precision == NBCS_PREC_MIXED &&
            (flow->grid[2] + 2.0) * (flow->grid[5] + 2.0) * (flow->grid[8] + 2.0) >= 4294967296.0)
            return set_error(NBCS_ERR_UNSUPPORTED,
                             "mixed precision: spline grids of 2^32 nodes or more (with the "
                             "2-node border) are not supported; use precision fp64");
        // the FP32 cell search takes the cell index from the float mantissa
        for (int d = 0; d < 3 && precision == NBCS_PREC_MIXED; ++d)
            if (flow->grid[3 * d + 2] > 8388608.0)
                return set_error(NBCS_ERR_UNSUPPORTED,
                                 "mixed precision: spline grid axis %d has more than 2^23 nodes; "
                                 "use precision fp64", d);
        break;
    }
    default:
        return set_error(NBCS_ERR_INVALID, "unknown flow kind %d", flow->kind);
    }
    return NBCS_OK;
}

}  // namespace nbcs

namespace nbcs {

#ifdef NBCS_CHECK
static int (*g_check_readers[32])(unsigned int*, int);
static int g_check_nreaders = 0;

int register_check_reader(int (*read)(unsigned int*, int))
{
    // static initialisers of the library's units, run once at load
    if (g_check_nreaders < 32) g_check_readers[g_check_nreaders++] = read;
    return g_check_nreaders;
}
#endif

}  // namespace nbcs

extern "C" int nbcs_check_enabled(void)
{
#ifdef NBCS_CHECK
    return 1;
#else
    return 0;
#endif
}

extern "C" int nbcs_check_bits(uint32_t* bits, int32_t reset)
{
    if (!bits) return nbcs::set_error(NBCS_ERR_INVALID, "check_bits: NULL");
    *bits = 0;
#ifdef NBCS_CHECK
    for (int k = 0; k < nbcs::g_check_nreaders; ++k) {
        unsigned int b = 0;
        int e = nbcs::g_check_readers[k](&b, reset);
        if (e) return nbcs::set_error(NBCS_ERR_CUDA, "check_bits: %s",
                                      cudaGetErrorString((cudaError_t)e));
        *bits |= b;
    }
#else
    (void)reset;
#endif
    return NBCS_OK;
}

extern "C" int nbcs_abi_version(void) { return NBCS_ABI_VERSION; }

extern "C" const char* nbcs_last_error(void) { return nbcs::g_err; }
