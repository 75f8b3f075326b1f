// Arguments shared by the FP64 and mixed-precision flow-map launchers.
#pragma once

#include "nbcs_internal.cuh"

namespace nbcs {

// The particle set of one launch: the grid (x_i, y_j) of flowmap_grid_2D, or
// the auxiliary grid of flowmap_aux_grid_2D (integration.py:249-464) -- n = 5
// (eig_main) or 4 particles per grid point, started at (x_i, y_j) + (h, 0),
// (-h, 0), (0, h), (0, -h) [, (0, 0)] -- laid out as a virtual (nx, ny * n)
// grid, so that the (nx, ny, n, 2) result is that grid's flow map and the
// near-identical trajectories of one point sit in neighbouring lanes; or
// (n = kPointList) the point list of flowmap (integration.py:8-62), npts
// rows (x, y) of x, laid out as a virtual (ceil(npts / ny), ny) grid in list
// order, so that consecutive points share a particle tile and the flat index
// of entry (i, j) is the point index i * ny + j (entries past npts do not
// exist: they are neither integrated nor written).
constexpr int kPointList = -1;
constexpr int kPointListColumns = 8;  // columns of the virtual grid of a point list

struct AuxGrid {
    int n;             // 0: plain grid; 4 or 5 particles per grid point; kPointList
    int ny;            // columns of the real grid (of the virtual grid for a point list)
    int compute_edge;  // integrate the edge points (only their centre particle when n = 5)
    double h;
    long npts;         // kPointList: number of points
};

// False for the padding entries of a point list's virtual grid.
__device__ __forceinline__ bool particle_exists(const AuxGrid& A, long k)
{
    return A.n != kPointList || k < A.npts;
}

// Start point of particle (i, jv) of the virtual grid; false when it is masked
// or skipped (its result stays 0 with status MASKED, as the reference leaves
// those entries of its zero-initialised output).
__device__ __forceinline__ bool particle_start(const AuxGrid& A, const double* __restrict__ x,
                                               const double* __restrict__ y,
                                               const uint8_t* __restrict__ mask, int nx, int i,
                                               int jv, double* x0, double* y0)
{
    if (A.n == 0) {
        if (mask && mask[(long)i * A.ny + jv]) return false;
        *x0 = x[i];
        *y0 = y[jv];
        return true;
    }
    if (A.n == kPointList) {  // pts[k, :], k < npts (particle_exists)
        const long k = (long)i * A.ny + jv;
        if (mask && mask[k]) return false;
        *x0 = x[2 * k];
        *y0 = x[2 * k + 1];
        return true;
    }
    const int j = jv / A.n, k = jv - j * A.n;
    if (mask && mask[(long)i * A.ny + j]) return false;
    const bool edge = i == 0 || i == nx - 1 || j == 0 || j == A.ny - 1;
    if (edge && !(A.compute_edge && (A.n == 4 || k == 4))) return false;
    // np.array([x[i], y[j]]) + aux_grid[k, :]
    *x0 = x[i] + (k == 0 ? A.h : k == 1 ? -A.h : 0.0);
    *y0 = y[j] + (k == 2 ? A.h : k == 3 ? -A.h : 0.0);
    return true;
}

struct FlowmapArgs {
    Params P;
    double ts, te;  // solver-time span params[0] * [t0, t0 + T]
    const double* x;
    const double* y;
    int nx, ny;  // real grid
    AuxGrid aux;
    const uint8_t* mask;
    double* out;
    int32_t* status;
    int32_t* stats;
    double rtol, atol;
    int nmax;
    int threads, blocks_per_sm, lanes;
    const void* step_model;
    cudaStream_t stream;
    // columns of the virtual particle grid
    int nyv() const { return aux.n > 0 ? ny * aux.n : ny; }
};

// Threads per block of the single-field integrator, and the width in y of the
// particle tile a block integrates: at LP = 2 a block takes a 16 x 8 tile of
// the grid (8 warps, each a 4 x 4 sub-tile).  Measured on the geophysical
// spline workload (676 x 251 particles): 128-thread 8 x 8 tiles 5.52 ms,
// 256-thread 16 x 8 tiles 5.24 ms, 8 x 16 tiles 5.36 ms, 32 x 4 tiles 5.43
// ms; warps of one block share L1 lines of neighbouring trajectories, and the
// flow is mostly zonal.  The minimum of 3 resident blocks gives the compiler
// 85 registers a thread; it takes 80 with no spills (24 warps per SM), 5.08
// ms; a 64-register cap with 4 blocks spilled and took 5.40 ms.
constexpr int kFm32Block = 256;
constexpr int kFm32TileJ = 8;
constexpr int kFm32MinBlocks = 3;

int launch_flowmap64(const nbcs_flow* flow, const FlowmapArgs& a);
int launch_flowmap32(const nbcs_flow* flow, const FlowmapArgs& a);
int launch_flowmap32_learned(const nbcs_flow* flow, const FlowmapArgs& a, int mode);
int launch_rhs32(const nbcs_flow* flow, const Params& P, const double* ty, long n, double* dy,
                 cudaStream_t stream);

// Thread -> (particle group, lane) map for blocks of BT threads.  A block
// holds BT/LP particles laid out as a (TI x TJ) tile of the grid; tiles run in
// row-major order.  Inside the tile each warp takes a compact (WI x WJ)
// sub-tile (4 x 8, 4 x 4, 2 x 4 particles at LP = 1, 2, 4): the fewer spline
// cells a warp's particles sit in, the more of its stencil gathers hit the
// same 32-byte entries.  Blocks of two or more warps use tiles TJW wide in y
// (8 unless given; never narrower than a warp's sub-tile).
template <int LP, int BT, int TJW = 8>
struct TileShape {
    static constexpr int PW = 32 / LP;                   // particles per warp
    static constexpr int WJ = LP == 1 ? 8 : 4, WI = PW / WJ;
    static constexpr int PB = BT / LP;                   // particles per block
    static constexpr int TJ = BT >= 64 && TJW > WJ ? TJW : WJ, TI = PB / TJ;
    static constexpr int WPJ = TJ / WJ;                  // warps along j
    static_assert(BT % 32 == 0 && TJ % WJ == 0 && PB % TJ == 0, "tile shape");
};

template <int LP, int BT, int TJW = 8>
__device__ __forceinline__ bool tile_particle(long t, int nx, int ny, int* i, int* j)
{
    using S = TileShape<LP, BT, TJW>;
    long tile = t / BT;
    int r = (int)(t - tile * BT) / LP;
    int w = r / S::PW, q = r - w * S::PW;
    int tiles_j = (ny + S::TJ - 1) / S::TJ;
    long ti = tile / tiles_j;
    int tj = (int)(tile - ti * tiles_j);
    *i = (int)(ti * S::TI) + (w / S::WPJ) * S::WI + q / S::WJ;
    *j = tj * S::TJ + (w % S::WPJ) * S::WJ + q % S::WJ;
    return *i < nx && *j < ny;
}

}  // namespace nbcs
