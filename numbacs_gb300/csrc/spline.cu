// Cubic B-spline prefilter and coefficient packing.
//
// get_interp_arrays_2D (flows.py:9-46) calls interpolation.splines.prefilter
// with k=3: natural boundary conditions (zero second derivative at both ends),
// n+2 coefficients per axis, applied separably along t, x and y.  Each axis
// is a (1,4,1) tridiagonal solve per grid line; one thread solves one line
// (adjacent threads take adjacent lines, so the strided axes are coalesced).
// The forward-elimination pivots depend only on the line length, so each
// block tabulates them once in shared memory.  Compiled with -fmad=false, in
// the same operation order as the CPU oracle.
#include "nbcs_internal.cuh"

namespace nbcs {

struct LineSet {
    long n_outer, n_inner;
    long in_os, in_is, out_os, out_is;  // base offsets per outer / inner index
    long s_in, s_out;                   // element strides along the line
};

__global__ void prefilter_lines_kernel(const double* __restrict__ f, double* __restrict__ c, int n,
                                       LineSet L)
{
    extern __shared__ double piv[];  // piv[k] = modified diagonal of unknown k
    const int m = n - 2;
    if (threadIdx.x == 0 && m > 0) {
        piv[0] = 4.0;
        for (int k = 1; k < m; ++k) piv[k] = 4.0 - 1.0 / piv[k - 1];
    }
    __syncthreads();
    const long lines = L.n_outer * L.n_inner;
    for (long l = (long)blockIdx.x * blockDim.x + threadIdx.x; l < lines;
         l += (long)gridDim.x * blockDim.x) {
        long o = l / L.n_inner, q = l - o * L.n_inner;
        const double* fl = f + o * L.in_os + q * L.in_is;
        double* cl = c + o * L.out_os + q * L.out_is;
        const long fs = L.s_in, cs = L.s_out;
        if (n == 1) {
            double v = fl[0];
            cl[0] = v;
            cl[cs] = v;
            cl[2 * cs] = v;
            continue;
        }
        double c0 = fl[0], cn1 = fl[(long)(n - 1) * fs];
        // forward elimination; the modified rhs is parked in the output slots
        double rprev = 0.0;
        for (int k = 0; k < m; ++k) {
            double rhs = 6.0 * fl[(long)(k + 1) * fs];
            if (k == 0) rhs -= c0;
            if (k == m - 1) rhs -= cn1;
            double r;
            if (k == 0) {
                r = rhs;
            } else {
                double w = 1.0 / piv[k - 1];
                r = rhs - w * rprev;
            }
            cl[(long)(k + 2) * cs] = r;
            rprev = r;
        }
        double next = 0.0;
        for (int k = m - 1; k >= 0; --k) {
            double r = cl[(long)(k + 2) * cs];
            double v = (k == m - 1) ? r / piv[k] : (r - next) / piv[k];
            cl[(long)(k + 2) * cs] = v;
            next = v;
        }
        cl[cs] = c0;
        cl[(long)n * cs] = cn1;
        double c1 = (n > 2) ? cl[2 * cs] : cn1;
        double cn2 = (n > 2) ? cl[(long)(n - 1) * cs] : c0;
        cl[0] = 2.0 * c0 - c1;
        cl[(long)(n + 1) * cs] = 2.0 * cn1 - cn2;
    }
}

// FP64 (u, v) per node, and the FP32 "quad" layout: entry k = (u_j, v_j) for
// j = k .. k+3 (32 bytes; zeros past the end) so a 4-tap stencil row is one
// aligned 32-byte load.
__global__ void pack_uv_kernel(const double* __restrict__ cu, const double* __restrict__ cv, long n,
                               double2* __restrict__ uv, float4* __restrict__ uv32)
{
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long)gridDim.x * blockDim.x) {
        double u = cu[k], v = cv[k];
        uv[k] = make_double2(u, v);
        if (uv32) {
            float q[8];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                q[2 * j] = k + j < n ? (float)cu[k + j] : 0.f;
                q[2 * j + 1] = k + j < n ? (float)cv[k + j] : 0.f;
            }
            uv32[2 * k] = make_float4(q[0], q[1], q[2], q[3]);
            uv32[2 * k + 1] = make_float4(q[4], q[5], q[6], q[7]);
        }
    }
}

static const int kMaxLine = 12000;  // pivot table fits in 96 KB of shared memory

static int run_pass(const double* f, double* c, int n, const LineSet& L, cudaStream_t s)
{
    long lines = L.n_outer * L.n_inner;
    if (lines == 0) return NBCS_OK;
    int threads = 128;
    long blocks = (lines + threads - 1) / threads;
    long cap = (long)sm_count() * 8;
    if (blocks > cap) blocks = cap;
    size_t smem = sizeof(double) * (size_t)(n > 2 ? n - 2 : 1);
    if (smem > 48 * 1024)
        NBCS_CUDA_TRY(cudaFuncSetAttribute(prefilter_lines_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    prefilter_lines_kernel<<<(unsigned)blocks, threads, smem, s>>>(f, c, n, L);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

}  // namespace nbcs

using namespace nbcs;

extern "C" size_t nbcs_spline_prefilter_scratch_bytes(int32_t nt, int32_t nx, int32_t ny)
{
    if (nt < 1 || nx < 1 || ny < 1) return 0;
    size_t NT = (size_t)nt + 2, NX = (size_t)nx + 2;
    return sizeof(double) * (NT * nx * ny + NT * NX * ny);
}

extern "C" int nbcs_spline_prefilter_3d(const double* f, int32_t nt, int32_t nx, int32_t ny,
                                        double* coef, void* scratch, size_t scratch_bytes,
                                        void* stream)
{
    NBCS_RANGE();
    if (nt < 1 || nx < 1 || ny < 1 || !f || !coef)
        return set_error(NBCS_ERR_INVALID, "prefilter: bad sizes or NULL arrays");
    if (nt > kMaxLine || nx > kMaxLine || ny > kMaxLine)
        return set_error(NBCS_ERR_UNSUPPORTED, "prefilter: axis longer than %d", kMaxLine);
    size_t need = nbcs_spline_prefilter_scratch_bytes(nt, nx, ny);
    if (!scratch || scratch_bytes < need)
        return set_error(NBCS_ERR_SCRATCH, "prefilter: scratch needs %zu bytes", need);
    cudaStream_t s = as_stream(stream);
    const long NT = nt + 2, NX = nx + 2, NY = ny + 2;
    double* tmp = static_cast<double*>(scratch);          // (NT, nx, ny)
    double* tmp2 = tmp + (size_t)NT * nx * ny;            // (NT, NX, ny)
    LineSet Lt = {nx, ny, ny, 1, ny, 1, (long)nx * ny, (long)nx * ny};
    LineSet Lx = {NT, ny, (long)nx * ny, 1, NX * ny, 1, ny, ny};
    LineSet Ly = {NT, NX, NX * ny, ny, NX * NY, NY, 1, 1};
    int rc = run_pass(f, tmp, nt, Lt, s);
    if (!rc) rc = run_pass(tmp, tmp2, nx, Lx, s);
    if (!rc) rc = run_pass(tmp2, coef, ny, Ly, s);
    return rc;
}

extern "C" int nbcs_spline_pack_uv(const double* cu, const double* cv, int64_t n, double* coef_uv,
                                   float* coef_uv32, void* stream)
{
    NBCS_RANGE();
    if (n < 0 || (n > 0 && (!cu || !cv || !coef_uv)))
        return set_error(NBCS_ERR_INVALID, "pack_uv: bad arguments");
    if ((reinterpret_cast<uintptr_t>(coef_uv) & 15) || (reinterpret_cast<uintptr_t>(coef_uv32) & 31))
        return set_error(NBCS_ERR_INVALID,
                         "pack_uv: coef_uv must be 16-byte and coef_uv32 32-byte aligned");
    if (n == 0) return NBCS_OK;
    long blocks = (n + 255) / 256;
    long cap = (long)sm_count() * 16;
    if (blocks > cap) blocks = cap;
    pack_uv_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(
        cu, cv, n, reinterpret_cast<double2*>(coef_uv), reinterpret_cast<float4*>(coef_uv32));
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}
