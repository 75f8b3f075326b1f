// Flow-map composition (integration.py:609-737): a long-T flow map built from
// nT short ones, each particle carried through the maps by bilinear
// interpolation on the particle grid.  Compiled with -fmad=false (the oracle's
// operation order).
//
// One thread per particle walks the nT maps in sequence: per map it gathers the
// 2 x 2 cell around its current point (two 32-byte rows of double2) and
// interpolates both components.  The maps are read in ring order from
// `first`, so a time series that advances by one short map needs no copy of
// the other nT - 1 (the reference shifts the whole stack every step).
//
// Interpolation is the interpolation package's eval_linear on a UCGrid with
// extrapolation CONSTANT: 0 strictly outside the grid box (pinned by the
// reference's composition fixtures: wall points that a map leaves 1 ulp
// outside [0, 2] compose to 0).  Arithmetic: cell offsets from the host-side
// inverse spacing (n - 1) / (b - a) (GB300's FP64 pipe is narrow and a divide
// is a multi-instruction sequence) and three explicit-FMA lerps per component,
// the same operations as the oracle.
#include "nbcs_internal.cuh"

namespace nbcs {

struct UGrid2 {
    double x0, x1, y0, y1, dinvx, dinvy;  // dinv = (n - 1) / (b - a)
    int nx, ny;
};

// cell and offset of a point inside [a, b] on the uniform axis (a, b, n)
__device__ __forceinline__ int lin_locate(double a, double dinv, int n, double x, double* lam)
{
    double u = (x - a) * dinv;
    int i = (int)floor(u);
    if (i > n - 2) i = n - 2;
    if (i < 0) i = 0;
    *lam = u - (double)i;
    return i;
}

__device__ __forceinline__ double2 bilinear2(const double2* __restrict__ f, const UGrid2& g,
                                             double px, double py)
{
    if (px < g.x0 || px > g.x1 || py < g.y0 || py > g.y1) return make_double2(0.0, 0.0);
    if (px != px || py != py) return make_double2(px + py, px + py);  // NaN in, NaN out
    double l0, l1;
    const int i = lin_locate(g.x0, g.dinvx, g.nx, px, &l0);
    const int j = lin_locate(g.y0, g.dinvy, g.ny, py, &l1);
    if (!NBCS_CHECKED(i >= 0 && i <= g.nx - 2 && j >= 0 && j <= g.ny - 2,
                      NBCS_CHECK_COMPOSE_GATHER))
        return make_double2(0.0, 0.0);
    const double2* r0 = f + (long)i * g.ny + j;
    const double2* r1 = r0 + g.ny;
    const double2 f00 = __ldg(r0), f01 = __ldg(r0 + 1), f10 = __ldg(r1), f11 = __ldg(r1 + 1);
    double2 v;
    const double ax = __fma_rn(l1, f01.x - f00.x, f00.x), bx = __fma_rn(l1, f11.x - f10.x, f10.x);
    const double ay = __fma_rn(l1, f01.y - f00.y, f00.y), by = __fma_rn(l1, f11.y - f10.y, f10.y);
    v.x = __fma_rn(l0, bx - ax, ax);
    v.y = __fma_rn(l0, by - ay, ay);
    return v;
}

__global__ void compose_kernel(const double2* __restrict__ fms, int nT, int first, UGrid2 g,
                               double2* __restrict__ out)
{
    const long m = (long)g.nx * g.ny;
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < m;
         p += (long)gridDim.x * blockDim.x) {
        double2 pt = fms[(long)(first % nT) * m + p];
        for (int k = 1; k < nT - 1; ++k)
            pt = bilinear2(fms + (long)((first + k) % nT) * m, g, pt.x, pt.y);
        out[p] = bilinear2(fms + (long)((first + nT - 1) % nT) * m, g, pt.x, pt.y);
    }
}

}  // namespace nbcs

using namespace nbcs;

extern "C" int nbcs_flowmap_compose(const double* flowmaps, int32_t nT, int32_t first,
                                    const double* grid, double* out, void* stream)
{
    NBCS_RANGE();
    if (!grid) return set_error(NBCS_ERR_INVALID, "compose: NULL grid");
    const double gnx = grid[2], gny = grid[5];
    if (!(gnx >= 2.0 && gny >= 2.0 && gnx <= 2147483647.0 && gny <= 2147483647.0) ||
        gnx != (double)(long)gnx || gny != (double)(long)gny)
        return set_error(NBCS_ERR_INVALID, "compose: grid needs integer n >= 2 on both axes");
    if (!(grid[1] > grid[0]) || !(grid[4] > grid[3]))
        return set_error(NBCS_ERR_INVALID, "compose: grid needs b > a on both axes");
    if (nT < 1 || first < 0 || first >= nT)
        return set_error(NBCS_ERR_INVALID, "compose: need nT >= 1 and 0 <= first < nT");
    const UGrid2 g = {grid[0], grid[1], grid[3], grid[4], (gnx - 1.0) / (grid[1] - grid[0]),
                      (gny - 1.0) / (grid[4] - grid[3]), (int)gnx, (int)gny};
    const long m = (long)g.nx * g.ny;
    if (m > (1L << 40)) return set_error(NBCS_ERR_INVALID, "compose: grid too large");
    if (!flowmaps || !out ||
        ((reinterpret_cast<uintptr_t>(flowmaps) | reinterpret_cast<uintptr_t>(out)) & 15))
        return set_error(NBCS_ERR_INVALID, "compose: NULL or misaligned array");
    long blocks = (m + 255) / 256;
    const long cap = (long)sm_count() * 32;
    if (blocks > cap) blocks = cap;
    compose_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const double2*>(flowmaps), nT, first, g, reinterpret_cast<double2*>(out));
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}
