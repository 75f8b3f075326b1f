// Cauchy-Green / FTLE stencil kernels (HBM-bound).
//
//   ftle_grid_2D   diagnostics.py:21-65 (+ utils.gradF_stencil_2D :41-44,
//                  utils.eigvalsh_max_2D :185-189)
//   C_eig_2D       diagnostics.py:200-244
//   ftle_from_eig  diagnostics.py:247-269
//
// One thread per grid point; the flow map is read as double2 (16 B per point)
// and each thread's four neighbours come from the same or adjacent rows, which
// the L1/L2 caches serve, so DRAM sees ~16 B read + 8 B (FTLE) or +16 B
// (eigenvector) written per point.  Compiled with -fmad=false: the arithmetic
// is the reference's, operation for operation.
#include "batch_common.cuh"
#include "nbcs_internal.cuh"

namespace nbcs {

struct Grad {
    double dxdx, dxdy, dydx, dydy;
};

__device__ __forceinline__ Grad grad_stencil(const double2* __restrict__ F, long k, int ny,
                                             double dx, double dy)
{
    // interior points only: k - ny >= 0 and k + ny < nx * ny by the caller's test
    double2 ip = __ldg(F + k + ny), im = __ldg(F + k - ny);
    double2 jp = __ldg(F + k + 1), jm = __ldg(F + k - 1);
    Grad g;
    g.dxdx = (ip.x - im.x) / (2.0 * dx);
    g.dxdy = (jp.x - jm.x) / (2.0 * dy);
    g.dydx = (ip.y - im.y) / (2.0 * dx);
    g.dydy = (jp.y - jm.y) / (2.0 * dy);
    return g;
}

// Symmetric 2x2 eigen-decomposition [[a, b], [b, d]]: the larger eigenvalue by
// the eigvalsh_max_2D closed form, the smaller one in LAPACK dlaev2's
// cancellation-free product form, the unit eigenvector of the larger one from
// the better-conditioned of its two expressions, sign normalised to ex >= 0.
__device__ __forceinline__ void sym2_eig(double a, double b, double d, double* lmin, double* lmax,
                                         double* vx, double* vy)
{
    double tr = a + d;
    double disc = sqrt((a - d) * (a - d) + 4.0 * (b * b));
    double l1 = 0.5 * (tr + disc);
    double acmx = fabs(a) > fabs(d) ? a : d;
    double acmn = fabs(a) > fabs(d) ? d : a;
    double l2 = (l1 != 0.0) ? (acmx / l1) * acmn - (b / l1) * b : 0.5 * (tr - disc);
    double ex, ey;
    if (b == 0.0) {
        if (a >= d) { ex = 1.0; ey = 0.0; }
        else { ex = 0.0; ey = 1.0; }
    } else if (a >= d) {
        ex = l1 - d;
        ey = b;
    } else {
        ex = b;
        ey = l1 - a;
    }
    double nrm = sqrt(ex * ex + ey * ey);
    ex /= nrm;
    ey /= nrm;
    if (ex < 0.0 || (ex == 0.0 && ey < 0.0)) { ex = -ex; ey = -ey; }
    *lmin = l2;
    *lmax = l1;
    *vx = ex;
    *vy = ey;
}

__device__ __forceinline__ bool interior(long k, int nx, int ny, int* i, int* j)
{
    *i = (int)(k / ny);
    *j = (int)(k - (long)(*i) * ny);
    return *i >= 1 && *i < nx - 1 && *j >= 1 && *j < ny - 1;
}

__global__ void ftle_kernel(const double2* __restrict__ F, int nx, int ny, double scaling,
                            double dx, double dy, const uint8_t* __restrict__ mask,
                            double* __restrict__ ftle)
{
    const long n = (long)nx * ny;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long)gridDim.x * blockDim.x) {
        int i, j;
        double out = 0.0;
        if (interior(k, nx, ny, &i, &j) && !(mask && mask[k])) {
            Grad g = grad_stencil(F, k, ny, dx, dy);
            double off = g.dxdx * g.dxdy + g.dydx * g.dydy;
            double a = g.dxdx * g.dxdx + g.dydx * g.dydx;
            double d = g.dxdy * g.dxdy + g.dydy * g.dydy;
            double tr = a + d;
            double disc = sqrt((a - d) * (a - d) + 4.0 * (off * off));
            double lmax = 0.5 * (tr + disc);
            if (lmax > 1.0) out = scaling * log(lmax);
        }
        ftle[k] = out;
    }
}

__global__ void ceig_kernel(const double2* __restrict__ F, int nx, int ny, double dx, double dy,
                            const uint8_t* __restrict__ mask, double2* __restrict__ evals,
                            double2* __restrict__ evecs)
{
    const long n = (long)nx * ny;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long)gridDim.x * blockDim.x) {
        int i, j;
        double2 ev = make_double2(0.0, 0.0);
        double2 v0 = make_double2(0.0, 0.0), v1 = make_double2(0.0, 0.0);
        if (interior(k, nx, ny, &i, &j) && !(mask && mask[k])) {
            Grad g = grad_stencil(F, k, ny, dx, dy);
            double off = g.dxdx * g.dxdy + g.dydx * g.dydy;
            double a = g.dxdx * g.dxdx + g.dydx * g.dydx;
            double d = g.dxdy * g.dxdy + g.dydy * g.dydy;
            double l0, l1, vx, vy;
            sym2_eig(a, off, d, &l0, &l1, &vx, &vy);
            ev = make_double2(l0, l1);
            v0 = make_double2(-vy, vx);  // row 0: columns v_min, v_max
            v1 = make_double2(vx, vy);   // row 1
        }
        evals[k] = ev;
        evecs[2 * k] = v0;
        evecs[2 * k + 1] = v1;
    }
}

// C_tensor_2D (diagnostics.py:69-111) with utils.gradF_aux_stencil_2D
// (:50-84): C11, C12, C22 of the tensor of the +-h particles (the first four
// of the na per point) for 2 <= i < nx-2, 2 <= j < ny-2 unless masked, 0
// elsewhere -- the stencil of ceig_aux_kernel without the eigen-solve.
__global__ void ctensor_aux_kernel(const double2* __restrict__ F, int nx, int ny, int na,
                                   double h, const uint8_t* __restrict__ mask,
                                   double* __restrict__ C)
{
    const long n = (long)nx * ny;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long)gridDim.x * blockDim.x) {
        const int i = (int)(k / ny), j = (int)(k - (long)i * ny);
        double c11 = 0.0, c12 = 0.0, c22 = 0.0;
        if (i >= 2 && i < nx - 2 && j >= 2 && j < ny - 2 && !(mask && mask[k])) {
            const double2* A = F + k * na;
            const double dxdx = (A[0].x - A[1].x) / (2.0 * h);
            const double dxdy = (A[2].x - A[3].x) / (2.0 * h);
            const double dydx = (A[0].y - A[1].y) / (2.0 * h);
            const double dydy = (A[2].y - A[3].y) / (2.0 * h);
            c11 = dxdx * dxdx + dydx * dydx;
            c12 = dxdx * dxdy + dydx * dydy;
            c22 = dxdy * dxdy + dydy * dydy;
        }
        C[3 * k] = c11;
        C[3 * k + 1] = c12;
        C[3 * k + 2] = c22;
    }
}

// C_eig_aux_2D (diagnostics.py:113-197) with utils.gradF_aux_stencil_2D
// (:50-84) and gradF_main_stencil_2D (:88-124): F is (nx, ny, na, 2).
// eig_main (na = 5): eigenvectors from the aux-particle tensor, eigenvalues
// from the main-grid tensor of the centre particles, for 2 <= i < nx-2,
// 2 <= j < ny-2; otherwise (na = 4) both from the aux tensor, 1-wide border.
__global__ void ceig_aux_kernel(const double2* __restrict__ F, int nx, int ny, int eig_main,
                                double dx, double dy, double h, const uint8_t* __restrict__ mask,
                                double2* __restrict__ evals, double2* __restrict__ evecs)
{
    const long n = (long)nx * ny;
    const int na = eig_main ? 5 : 4, b = eig_main ? 2 : 1;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long)gridDim.x * blockDim.x) {
        const int i = (int)(k / ny), j = (int)(k - (long)i * ny);
        double2 ev = make_double2(0.0, 0.0);
        double2 v0 = make_double2(0.0, 0.0), v1 = make_double2(0.0, 0.0);
        if (i >= b && i < nx - b && j >= b && j < ny - b && !(mask && mask[k])) {
            const double2* A = F + k * na;
            double dxdx = (A[0].x - A[1].x) / (2.0 * h);
            double dxdy = (A[2].x - A[3].x) / (2.0 * h);
            double dydx = (A[0].y - A[1].y) / (2.0 * h);
            double dydy = (A[2].y - A[3].y) / (2.0 * h);
            double off = dxdx * dxdy + dydx * dydy;
            double l0, l1, vx, vy;
            sym2_eig(dxdx * dxdx + dydx * dydx, off, dxdy * dxdy + dydy * dydy, &l0, &l1, &vx, &vy);
            if (eig_main) {
                const double2 xp = F[(k + ny) * na + 4], xm = F[(k - ny) * na + 4];
                const double2 yp = F[(k + 1) * na + 4], ym = F[(k - 1) * na + 4];
                double mxdx = (xp.x - xm.x) / (2.0 * dx);
                double mxdy = (yp.x - ym.x) / (2.0 * dy);
                double mydx = (xp.y - xm.y) / (2.0 * dx);
                double mydy = (yp.y - ym.y) / (2.0 * dy);
                double moff = mxdx * mxdy + mydx * mydy;
                double wx, wy;
                sym2_eig(mxdx * mxdx + mydx * mydx, moff, mxdy * mxdy + mydy * mydy, &l0, &l1,
                         &wx, &wy);
            }
            ev = make_double2(l0, l1);
            v0 = make_double2(-vy, vx);
            v1 = make_double2(vx, vy);
        }
        evals[k] = ev;
        evecs[2 * k] = v0;
        evecs[2 * k + 1] = v1;
    }
}

// FTLE and eigvec_max of one point for the fused ftle_evec_2D entry point:
// the stencil, tensor and larger eigenvalue of ftle_grid_2D / C_eig_2D, with
// the divisions that only scale -- the central differences' 1 / (2 dx),
// 1 / (2 dy) and the FTLE's 1 / (2 |T|) -- taken as products with reciprocals
// computed once on the host, and the eigenvector normalised by a reciprocal
// square root.  The smaller eigenvalue, which this entry point does not
// return, is not formed, and the log of the FTLE takes its mantissa part on
// the FP32 pipe (below).  The eigenvector is within a few ulp of C_eig_2D's
// and the FTLE within ~3e-7 relative of ftle_from_eig's where
// lambda_max > 1 + 1e-6; the FP64 divisions and log of the bit-exact kernels
// were most of this stencil's FP64 work.
__device__ __forceinline__ void ftle_evec_point(const double2* __restrict__ F, long k, int ny,
                                                double rdx, double rdy, double rden, double* f,
                                                double2* v)
{
    double2 ip = __ldg(F + k + ny), im = __ldg(F + k - ny);
    double2 jp = __ldg(F + k + 1), jm = __ldg(F + k - 1);
    const double dxdx = (ip.x - im.x) * rdx, dxdy = (jp.x - jm.x) * rdy;
    const double dydx = (ip.y - im.y) * rdx, dydy = (jp.y - jm.y) * rdy;
    const double b = dxdx * dxdy + dydx * dydy;
    const double a = dxdx * dxdx + dydx * dydx;
    const double d = dxdy * dxdy + dydy * dydy;
    const double l1 = 0.5 * ((a + d) + sqrt((a - d) * (a - d) + 4.0 * (b * b)));
    double ex, ey;
    if (b == 0.0) {
        ex = a >= d ? 1.0 : 0.0;
        ey = a >= d ? 0.0 : 1.0;
    } else if (a >= d) {
        ex = l1 - d;
        ey = b;
    } else {
        ex = b;
        ey = l1 - a;
    }
    const double r = rsqrt(ex * ex + ey * ey);
    ex *= r;
    ey *= r;
    if (ex < 0.0 || (ex == 0.0 && ey < 0.0)) {
        ex = -ex;
        ey = -ey;
    }
    // FTLE = log(lambda) / (2|T|) to ~3e-7 relative (the contract is 1e-5):
    // lambda = 2^e m with m in [1, 2), log(lambda) = e ln 2 + log1p(m - 1); the
    // exponent term in FP64 and m - 1 exact, its log1p on the FP32 pipe (the
    // FP64 log was the largest FP64 cost left once the divisions were gone)
    double fv = 0.0;
    if (l1 > 1.0) {
        const long long bits = __double_as_longlong(l1);
        const int e = (int)((bits >> 52) & 0x7ff) - 1023;
        if (e == 1024) {
            fv = l1 * rden;  // +inf
        } else {
            const double m =
                __longlong_as_double((bits & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
            fv = ((double)e * 0.6931471805599453 + (double)log1pf((float)(m - 1.0))) * rden;
        }
    }
    *f = fv;
    *v = make_double2(ex, ey);
}

__global__ void ftle_evec_kernel(const double2* __restrict__ F, int nx, int ny, double rden,
                                 double rdx, double rdy, const uint8_t* __restrict__ mask,
                                 double* __restrict__ ftle, double2* __restrict__ evec)
{
    const long n = (long)nx * ny;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long)gridDim.x * blockDim.x) {
        int i, j;
        double f = 0.0;
        double2 v = make_double2(0.0, 0.0);
        if (interior(k, nx, ny, &i, &j) && !(mask && mask[k])) ftle_evec_point(F, k, ny, rdx, rdy, rden, &f, &v);
        ftle[k] = f;
        evec[k] = v;
    }
}

__global__ void ftle_from_eig_kernel(const double* __restrict__ ev, long n, long stride,
                                     double den, double* __restrict__ ftle)
{
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long)gridDim.x * blockDim.x) {
        double e = ev[k * stride];
        ftle[k] = e > 1.0 ? log(e) / den : 0.0;
    }
}

// FTLE + eigvec_max of every field of a batch (fields without FTLE own no
// blocks); one 256-thread block per 256-point unit of a field.
__global__ void __launch_bounds__(kFtleBlock)
ftle_batch_kernel(const DevField* __restrict__ fields, int nfields, long long total_blocks)
{
    for (long long b = blockIdx.x; b < total_blocks; b += gridDim.x) {
        const int f = batch_find<kByFtleBlock>(fields, nfields, b);
        const DevField& F = fields[f];
        const long n = (long)F.nx * F.ny;
        const long k = (long)(b - F.block0) * kFtleBlock + threadIdx.x;
        if (k >= n) continue;
        int i, j;
        double fv = 0.0;
        double2 v = make_double2(0.0, 0.0);
        if (interior(k, F.nx, F.ny, &i, &j) && !(F.mask && F.mask[k]))
            ftle_evec_point(reinterpret_cast<const double2*>(F.out), k, F.ny, F.rdx, F.rdy,
                            F.rden, &fv, &v);
        F.ftle[k] = fv;
        reinterpret_cast<double2*>(F.evec)[k] = v;
    }
}

int launch_ftle_batch(const DevField* fields, int nfields, long long blocks, cudaStream_t s)
{
    long long g = blocks;
    long long cap = (long long)sm_count() * 32;
    if (g > cap) g = cap;
    ftle_batch_kernel<<<(unsigned)g, kFtleBlock, 0, s>>>(fields, nfields, blocks);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

static unsigned grid_for(long n, int threads)
{
    long b = (n + threads - 1) / threads;
    long cap = (long)sm_count() * 16;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (unsigned)b;
}

}  // namespace nbcs

using namespace nbcs;

static int check_fm(const double* fm, int32_t nx, int32_t ny)
{
    if (nx < 0 || ny < 0) return set_error(NBCS_ERR_INVALID, "negative grid size");
    if ((long)nx * ny > 0 && !fm) return set_error(NBCS_ERR_INVALID, "flowmap is NULL");
    if (fm && (reinterpret_cast<uintptr_t>(fm) & 15))
        return set_error(NBCS_ERR_INVALID, "flowmap must be 16-byte aligned");
    return NBCS_OK;
}

extern "C" int nbcs_ftle_grid_2d(const double* flowmap, int32_t nx, int32_t ny, double T,
                                 double dx, double dy, const uint8_t* mask, double* ftle,
                                 void* stream)
{
    NBCS_RANGE();
    int rc = check_fm(flowmap, nx, ny);
    if (rc) return rc;
    long n = (long)nx * ny;
    if (n == 0) return NBCS_OK;
    if (!ftle) return set_error(NBCS_ERR_INVALID, "ftle is NULL");
    double scaling = 1.0 / (2.0 * fabs(T));
    ftle_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(flowmap), nx, ny, scaling, dx, dy, mask, ftle);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

extern "C" int nbcs_c_eig_2d(const double* flowmap, int32_t nx, int32_t ny, double dx, double dy,
                             const uint8_t* mask, double* evals, double* evecs, void* stream)
{
    NBCS_RANGE();
    int rc = check_fm(flowmap, nx, ny);
    if (rc) return rc;
    long n = (long)nx * ny;
    if (n == 0) return NBCS_OK;
    if (!evals || !evecs || ((reinterpret_cast<uintptr_t>(evecs) | reinterpret_cast<uintptr_t>(evals)) & 15))
        return set_error(NBCS_ERR_INVALID, "evals/evecs NULL or not 16-byte aligned");
    ceig_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(flowmap), nx, ny, dx, dy, mask,
        reinterpret_cast<double2*>(evals), reinterpret_cast<double2*>(evecs));
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

extern "C" int nbcs_c_eig_aux_2d(const double* flowmap_aux, int32_t nx, int32_t ny,
                                 int32_t eig_main, double dx, double dy, double h,
                                 const uint8_t* mask, double* evals, double* evecs, void* stream)
{
    NBCS_RANGE();
    if (nx < 0 || ny < 0) return set_error(NBCS_ERR_INVALID, "c_eig_aux: negative grid size");
    long n = (long)nx * ny;
    if (n == 0) return NBCS_OK;
    if (!flowmap_aux || !evals || !evecs ||
        ((reinterpret_cast<uintptr_t>(flowmap_aux) | reinterpret_cast<uintptr_t>(evals) |
          reinterpret_cast<uintptr_t>(evecs)) & 15))
        return set_error(NBCS_ERR_INVALID, "c_eig_aux: NULL or misaligned array");
    ceig_aux_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(flowmap_aux), nx, ny, eig_main ? 1 : 0, dx, dy, h, mask,
        reinterpret_cast<double2*>(evals), reinterpret_cast<double2*>(evecs));
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

extern "C" int nbcs_c_tensor_2d(const double* flowmap_aux, int32_t nx, int32_t ny, int32_t naux,
                                double h, const uint8_t* mask, double* C, void* stream)
{
    NBCS_RANGE();
    if (nx < 0 || ny < 0 || naux < 4)
        return set_error(NBCS_ERR_INVALID, "c_tensor: negative grid size or fewer than 4 aux particles");
    long n = (long)nx * ny;
    if (n == 0) return NBCS_OK;
    if (!flowmap_aux || !C || (reinterpret_cast<uintptr_t>(flowmap_aux) & 15))
        return set_error(NBCS_ERR_INVALID, "c_tensor: NULL or misaligned array");
    ctensor_aux_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(flowmap_aux), nx, ny, naux, h, mask, C);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

extern "C" int nbcs_ftle_evec_2d(const double* flowmap, int32_t nx, int32_t ny, double T,
                                 double dx, double dy, const uint8_t* mask, double* ftle,
                                 double* evec_max, void* stream)
{
    NBCS_RANGE();
    int rc = check_fm(flowmap, nx, ny);
    if (rc) return rc;
    long n = (long)nx * ny;
    if (n == 0) return NBCS_OK;
    if (!ftle || !evec_max || (reinterpret_cast<uintptr_t>(evec_max) & 15))
        return set_error(NBCS_ERR_INVALID, "ftle/evec_max NULL or misaligned");
    ftle_evec_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(flowmap), nx, ny, 1.0 / (2.0 * fabs(T)),
        1.0 / (2.0 * dx), 1.0 / (2.0 * dy), mask, ftle, reinterpret_cast<double2*>(evec_max));
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

extern "C" int nbcs_ftle_from_eig(const double* eigval, int64_t n, int64_t stride, double T,
                                  double* ftle, void* stream)
{
    NBCS_RANGE();
    if (n < 0 || stride < 1) return set_error(NBCS_ERR_INVALID, "ftle_from_eig: bad n/stride");
    if (n == 0) return NBCS_OK;
    if (!eigval || !ftle) return set_error(NBCS_ERR_INVALID, "ftle_from_eig: NULL array");
    ftle_from_eig_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(eigval, n, stride,
                                                                          2.0 * fabs(T), ftle);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}
