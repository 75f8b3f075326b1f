// Device-side description of a batched launch (nbcs_batch_prepare / _run).
//
// Scratch layout (each part 256-byte aligned):
//   BatchHeader | DevFlow32[nflows] | DevFlow64[nflows] | DevField[nfields]
// Fields are listed with the prefix of their 32-particle chunks (chunk0) and
// of their 256-point FTLE blocks (block0), so a work unit finds its field by
// binary search.
#pragma once

#include "flows32.cuh"
#include "nbcs_internal.cuh"

namespace nbcs {

// A work unit is one warp's worth of particles taken as a 2-D tile of the
// field's grid: 4 x 8 particles at one lane per particle, 4 x 4 at two lanes
// per particle (the spline right-hand side of the mixed path).
constexpr int kBatchTileI = 4;
constexpr int kBatchThreads = 128;

__host__ __device__ __forceinline__ int batch_tile_j(int lp) { return lp == 1 ? 8 : 4; }
constexpr int kFtleBlock = 256;        // points per FTLE work unit

struct BatchHeader {
    unsigned long long counter;  // next chunk to hand out
    long long total_chunks;
    int nfields, nflows;
};

struct DevFlow32 {
    int kind, spherical;
    SplineGridF g;
    const float* c;  // quad layout
    float deg_per_km;
};

struct DevFlow64 {
    int kind, spherical;
    SplineGrid g;
    const double2* c;
    double r;
};

struct DevField {
    int flow, nx, ny, has_ftle;
    int lp, pad_;  // lanes per particle of this field's work units
    double ts, te, rtol, atol;
    double den, dx, dy;  // FTLE: 2|T| and grid spacing
    double rden, rdx, rdy;  // their reciprocals 1/(2|T|), 1/(2 dx), 1/(2 dy)
    Params P;
    const double* x;
    const double* y;
    const uint8_t* mask;
    double* out;
    int32_t* status;
    double* ftle;
    double* evec;
    long long chunk0, block0, tile0;  // prefixes of chunks, FTLE blocks, block tiles
};

inline size_t batch_align(size_t b) { return (b + 255) & ~(size_t)255; }

struct BatchLayout {
    size_t off_f32, off_f64, off_fields, total;
};

inline BatchLayout batch_layout(int nflows, int nfields)
{
    BatchLayout L;
    L.off_f32 = batch_align(sizeof(BatchHeader));
    L.off_f64 = L.off_f32 + batch_align(sizeof(DevFlow32) * (size_t)nflows);
    L.off_fields = L.off_f64 + batch_align(sizeof(DevFlow64) * (size_t)nflows);
    L.total = L.off_fields + batch_align(sizeof(DevField) * (size_t)nfields);
    return L;
}

enum BatchKey { kByChunk, kByFtleBlock, kByTile };

// index of the last field whose prefix value (chunk0, block0 or tile0) is <= c
template <BatchKey KEY>
__device__ __forceinline__ int batch_find(const DevField* __restrict__ fields, int nf, long long c)
{
    int lo = 0, hi = nf - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        long long v = KEY == kByChunk ? fields[mid].chunk0
                    : KEY == kByFtleBlock ? fields[mid].block0 : fields[mid].tile0;
        if (v <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Particle (i, j) of lane `lane` in work unit c of field F; false past the grid edge.
__device__ __forceinline__ bool batch_particle(const DevField& F, long long c, int lane, int* i,
                                               int* j)
{
    const int lp = F.lp, tj = batch_tile_j(lp);
    const long r = (long)(c - F.chunk0);
    const int tiles_j = (F.ny + tj - 1) / tj;
    const long tI = r / tiles_j;
    const int tJ = (int)(r - tI * tiles_j);
    const int p = lane / lp;
    *i = (int)(tI * kBatchTileI) + p / tj;
    *j = tJ * tj + p % tj;
    return *i < F.nx && *j < F.ny;
}

int launch_batch32_tiles(const DevFlow32* flows, const DevField* fields, int nfields,
                         long long tiles, int nmax, cudaStream_t s);
int launch_batch32(const BatchHeader* dev_hdr, const DevFlow32* flows, const DevField* fields,
                   int nfields, int blocks_per_sm, int nmax, cudaStream_t s);
int launch_batch64(const BatchHeader* dev_hdr, const DevFlow64* flows, const DevField* fields,
                   int nfields, int blocks_per_sm, int nmax, cudaStream_t s);
int launch_ftle_batch(const DevField* fields, int nfields, long long blocks, cudaStream_t s);

}  // namespace nbcs
