// FTLE ridge extraction: exact percentile selection, ridge stencil and
// order-preserving compaction.
//
//   ftle_ridge_pts   extraction/ridges.py:9-76
//   _ftle_ridges     extraction/ridges.py:79-154 (the mask)
//   np.percentile    ridges.py:48-51, evaluated by numba inside the jitted
//                    function: rank = 1 + (n-1)*q/100, value
//                    lower*(1-m) + upper*m of the order statistics around it.
//
// Percentile: radix selection of the k-th smallest double on order-preserving
// 64-bit keys, 11 bits per pass (6 passes).  Each pass is one launch; the last
// block to finish (atomic ticket, no spinning) picks the digit and resets the
// histogram for the next pass, so no host round trip is needed.  The last
// pass also takes the smallest key above the final group (keys that differ
// from the k-th in a higher digit), so that its last block finds the
// (k+1)-th order statistic -- the next nonzero bin of its own histogram, or
// that minimum -- and writes the percentile without another pass.  The
// selection state starts from a memset of the scratch.
//
// Ridge points: pass 1 evaluates the stencil and writes the mask (and, when
// the caller asks for it, the full point array) and one count per block of
// points (and per group of 64 blocks); pass 2 ranks the flagged points of each
// block in row-major order (warp ballots; each block adds up the counts before
// it from the group sums and its own group's block counts) and
// writes them compacted, gathering them from the full array when there is
// one, else re-evaluating the stencil at the flagged points only.
// Compiled with -fmad=false: the stencil arithmetic is the reference's.
#include <math.h>

#include <mutex>

#include "nbcs_internal.cuh"

namespace nbcs {

// ------------------------------------------------------------ percentile

constexpr int kDigitBits = 11;
constexpr int kBins = 1 << kDigitBits;
constexpr int kSelThreads = 512;

struct SelState {
    unsigned long long prefix;  // key bits chosen so far
    unsigned long long pmask;   // which key bits are chosen
    unsigned long long above_inv; // ~(smallest key above the final group); 0: none
    long long rank;             // rank still to find inside the prefix group
    long long eq;               // elements equal to the k-th key (after the last pass)
    unsigned int done;          // ticket of finished blocks in the current pass
    unsigned int nan_count;
    unsigned int pinf, ninf;
    double result;
};

struct SelScratch {
    unsigned int hist[kBins];
    SelState st;
};

// order-preserving unsigned key of a double's bit pattern
__device__ __forceinline__ unsigned long long dkey(unsigned long long u)
{
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// NaN / +-inf tests on the bit pattern: the same answers as isnan() and
// == +-INFINITY without FP64 compares, which issue on GB300's narrow FP64 pipe
// (the selection passes are otherwise integer work)
__device__ __forceinline__ bool bits_nan(unsigned long long u)
{
    return (u & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}

__device__ __forceinline__ double dkey_decode(unsigned long long k)
{
    unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)u);
}

// one radix pass: histogram the digit at `shift` of the keys in the current
// prefix group; the last block selects the digit holding rank `rank`.
// How the last pass turns the k-th and (k+1)-th order statistics into the
// percentile (numba's rules, ridges.py:48-51).
struct SelFinish {
    int mode;  // 0: interpolate; 1: q == 100 (maximum); 2: q == 0 (minimum)
    double m;  // interpolation weight of the upper statistic
    double* out;
};

__device__ void sel_finish(SelScratch* s, long n, unsigned long long kk, unsigned long long up,
                           const SelFinish& fin)
{
    const long long nan_count = (long long)__ldcg(&s->st.nan_count);
    const long long pinf = (long long)__ldcg(&s->st.pinf), ninf = (long long)__ldcg(&s->st.ninf);
    double lower = dkey_decode(kk), val;
    if (nan_count > 0) {
        val = NAN;
    } else if (n == 1) {
        val = lower;
    } else if (fin.mode == 1) {  // q == 100: maximum
        val = lower;
        if ((pinf + ninf) > 0 && !isfinite(val)) val = NAN;
    } else if (fin.mode == 2) {  // q == 0: minimum, with numba's infinity rules
        val = lower;
        if (pinf + ninf > 0) {
            long long finite = n - (pinf + ninf);
            if (finite == 0) val = NAN;
            if (pinf == 1 && n == 2) val = NAN;
            if (ninf > 1) val = NAN;
            if (finite == 1 && pinf > 1 && ninf != 1) val = NAN;
        }
    } else {
        double upper = (up == ~0ull) ? lower : dkey_decode(up);
        val = lower * (1.0 - fin.m) + upper * fin.m;
    }
    s->st.result = val;
    if (fin.out) *fin.out = val;
}

__global__ void __launch_bounds__(kSelThreads)
sel_pass_kernel(const double* __restrict__ f, long n, SelScratch* s, int shift, int bits, int first,
                long long k, SelFinish fin)
{
    __shared__ unsigned int h[kBins];
    __shared__ unsigned int cnt[3];
    __shared__ unsigned long long wmax[kSelThreads / 32];
    __shared__ bool is_last;
    __shared__ int sel_b, sel_same, next_bin;
    __shared__ unsigned long long sel_kk;
    for (int b = threadIdx.x; b < kBins; b += blockDim.x) h[b] = 0;
    if (threadIdx.x < 3) cnt[threadIdx.x] = 0;
    __syncthreads();
    // the first pass starts from the zeroed scratch: empty prefix, rank k
    const unsigned long long prefix = first ? 0ull : s->st.prefix;
    const unsigned long long pmask = first ? 0ull : s->st.pmask;
    const bool last_pass = shift == 0;
    const unsigned int dmask = (1u << bits) - 1u;
    unsigned int nn = 0, np = 0, nm = 0;
    unsigned long long ainv = 0ull;  // ~(smallest key above the group), last pass
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        const unsigned long long u = (unsigned long long)__double_as_longlong(f[i]);
        if (bits_nan(u)) { ++nn; continue; }
        if (first) {
            if (u == 0x7ff0000000000000ull) ++np;
            else if (u == 0xfff0000000000000ull) ++nm;
        }
        const unsigned long long key = dkey(u);
        if ((key & pmask) != prefix) {
            if (last_pass && (key & pmask) > prefix && ~key > ainv) ainv = ~key;
            continue;
        }
        atomicAdd(&h[(unsigned)(key >> shift) & dmask], 1u);
    }
    if (first) {
        if (nn) atomicAdd(&cnt[0], nn);
        if (np) atomicAdd(&cnt[1], np);
        if (nm) atomicAdd(&cnt[2], nm);
    }
    if (last_pass) {
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, ainv, o);
            ainv = other > ainv ? other : ainv;
        }
        if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = ainv;
    }
    __syncthreads();
    if (last_pass && threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) ainv = wmax[w] > ainv ? wmax[w] : ainv;
        if (ainv) atomicMax(&s->st.above_inv, ainv);
    }
    for (int b = threadIdx.x; b <= (int)dmask; b += blockDim.x)
        if (h[b]) atomicAdd(&s->hist[b], h[b]);
    if (first && threadIdx.x == 0) {
        if (cnt[0]) atomicAdd(&s->st.nan_count, cnt[0]);
        if (cnt[1]) atomicAdd(&s->st.pinf, cnt[1]);
        if (cnt[2]) atomicAdd(&s->st.ninf, cnt[2]);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = (atomicAdd(&s->st.done, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    // last block: find the digit whose cumulative count passes `rank`.  Each
    // thread sums `per` consecutive bins, a block-wide scan of those sums
    // finds the one thread whose range holds the rank, and that thread walks
    // its own bins (no serial loop over the whole block).
    __shared__ long long wsum[kSelThreads / 32];
    const long long rank = first ? k : s->st.rank;
    const int nb = (int)dmask + 1;
    const int per = (nb + blockDim.x - 1) / blockDim.x;
    long long local = 0;
    for (int q = 0; q < per; ++q) {
        int b = threadIdx.x * per + q;
        if (b < nb) local += __ldcg(&s->hist[b]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    long long incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        long long v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        long long w = lane < nw ? wsum[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            long long v = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += v;
        }
        if (lane < nw) wsum[lane] = w;
    }
    __syncthreads();
    if (warp) incl += wsum[warp - 1];
    const long long excl = incl - local, total = wsum[nw - 1];
    const bool beyond = rank >= total;  // unreachable for a valid rank
    if ((excl <= rank && rank < incl) || (beyond && threadIdx.x == blockDim.x - 1)) {
        long long cum = beyond ? total : excl;
        int b = beyond ? nb : (int)threadIdx.x * per;
        unsigned int hb = 0;
        for (; b < nb; ++b) {
            hb = __ldcg(&s->hist[b]);
            if (cum + (long long)hb > rank) break;
            cum += hb;
        }
        if (b >= nb) b = nb - 1;
        const unsigned long long kk = prefix | ((unsigned long long)b << shift);
        s->st.rank = rank - cum;
        s->st.prefix = kk;
        s->st.pmask = pmask | ((unsigned long long)dmask << shift);
        s->st.eq = hb;
        s->st.done = 0;
        sel_b = b;
        sel_kk = kk;
        sel_same = (rank - cum + 1 < (long long)hb) ? 1 : 0;
    }
    __syncthreads();
    if (last_pass) {
        // the (k+1)-th statistic: the k-th key again while equal keys remain,
        // else the next nonzero bin of this group (a block-wide min over the
        // bins above the selected one), else the smallest key above the group
        if (threadIdx.x == 0) next_bin = nb;
        __syncthreads();
        if (!sel_same) {
            for (int c = sel_b + 1 + (int)threadIdx.x; c < nb; c += blockDim.x)
                if (__ldcg(&s->hist[c])) {
                    atomicMin(&next_bin, c);
                    break;
                }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long up = ~0ull;
            if (sel_same) {
                up = sel_kk;
            } else if (next_bin < nb) {
                up = prefix | (unsigned long long)next_bin;
            } else {
                const unsigned long long a = __ldcg(&s->st.above_inv);
                if (a) up = ~a;
            }
            sel_finish(s, n, sel_kk, up, fin);
        }
        __syncthreads();
    }
    for (int b = threadIdx.x; b < kBins; b += blockDim.x) s->hist[b] = 0;
}

static unsigned sel_grid(long n)
{
    // two keys per thread before the grid reaches 4 blocks per SM
    long b = (n + kSelThreads * 2 - 1) / (kSelThreads * 2);
    long cap = (long)sm_count() * 4;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (unsigned)b;
}

// enqueue the selection; the result lands in s->st.result (and *out if given)
static int percentile_enqueue(const double* f, long n, double q, double* out, SelScratch* s,
                              cudaStream_t st)
{
    int mode = 0;
    long long k = 0;
    double m = 0.0;
    if (n == 1) {
        k = 0;
    } else if (q == 100.0) {
        mode = 1;
        k = n - 1;
    } else if (q == 0.0) {
        mode = 2;
        k = 0;
    } else {
        double rank = 1.0 + (double)(n - 1) * (q / 100.0);
        double fl = floor(rank);
        m = rank - fl;
        k = (long long)(fl - 1.0);
    }
    // zeroed scratch: empty histogram and counters, no key above the group
    NBCS_CUDA_TRY(cudaMemsetAsync(s, 0, sizeof(SelScratch), st));
    const SelFinish fin = {mode, m, out};
    unsigned g = sel_grid(n);
    int shift = 64;
    for (int pass = 0; shift > 0; ++pass) {
        int bits = shift >= kDigitBits ? kDigitBits : shift;
        shift -= bits;
        sel_pass_kernel<<<g, kSelThreads, 0, st>>>(f, n, s, shift, bits, pass == 0, k, fin);
        NBCS_LAUNCH_CHECK();
    }
    return NBCS_OK;
}

// ------------------------------------------------------------ ridges

constexpr int kRidgeThreads = 256;
constexpr int kRidgeRounds = 8;                            // most rounds per block
constexpr int kRidgeTile = kRidgeThreads * kRidgeRounds;  // most points per block
constexpr long kRidgeFillBlocks = 1216;                    // 8 blocks on each of 152 SMs

// Rounds of kRidgeThreads points per block: fewer on small fields, so that the
// grid still fills the GPU (a 676 x 251 field at 8 rounds would be 83 blocks,
// each running 8 dependent rounds of the FP64 stencil).
static inline int ridge_rounds(long n)
{
    long r = (n + kRidgeFillBlocks * kRidgeThreads - 1) / (kRidgeFillBlocks * kRidgeThreads);
    return r < 1 ? 1 : (r > kRidgeRounds ? kRidgeRounds : (int)r);
}

struct RidgeIn {
    const double* f;
    const double2* ev;
    const double* x;
    const double* y;
    int nx, ny;
    double sdd;
    const double* fmin_ptr;  // device threshold (percentile) or NULL
    double fmin_val;         // threshold when fmin_ptr is NULL
    double dx, dy;           // grid spacing; NaN: x[1] - x[0], y[1] - y[0] (ridges.py:39-40)
    int rounds;              // rounds of kRidgeThreads points per block (ridge_rounds)
};

__device__ __forceinline__ void ridge_spacing(const RidgeIn& R, double* dx, double* dy)
{
    *dx = R.dx == R.dx ? R.dx : R.x[1] - R.x[0];
    *dy = R.dy == R.dy ? R.dy : R.y[1] - R.y[0];
}

// a > b for doubles given as bit patterns, by integer comparison (IEEE
// semantics: false when either is NaN, -0 == +0); the ridge threshold test runs
// on every point and an FP64 compare would issue on the narrow FP64 pipe
__device__ __forceinline__ bool gt_bits(unsigned long long a, unsigned long long b)
{
    if (bits_nan(a) || bits_nan(b)) return false;
    if ((a << 1) == 0) a = 0;  // -0 -> +0
    if ((b << 1) == 0) b = 0;
    return dkey(a) > dkey(b);
}

// Ridge test at point k = i*ny + j (ridges.py:52-74).  Returns true and the
// sub-pixel point when (i, j) is a ridge point.
__device__ __forceinline__ bool ridge_at(const RidgeIn& R, double fmin, double dx, double dy, long k,
                                         double* px, double* py)
{
    const int ny = R.ny;
    int i = (int)(k / ny), j = (int)(k - (long)i * ny);
    if (i < 2 || i >= R.nx - 2 || j < 2 || j >= ny - 2) return false;
    const double* f = R.f;
    double f0 = f[k];
    if (!gt_bits((unsigned long long)__double_as_longlong(f0),
                 (unsigned long long)__double_as_longlong(fmin)))
        return false;
    double fip = f[k + ny], fim = f[k - ny], fjp = f[k + 1], fjm = f[k - 1];
    double fx = (fip - fim) / (2.0 * dx);
    double fy = (fjp - fjm) / (2.0 * dy);
    double fxx = (fip - 2.0 * f0 + fim) / (dx * dx);
    double fyy = (fjp - 2.0 * f0 + fjm) / (dy * dy);
    double fxy = (f[k + ny + 1] - f[k + ny - 1] - f[k - ny + 1] + f[k - ny - 1]) / (4.0 * dx * dy);
    double2 e = R.ev[k];
    double ex = e.x, ey = e.y;
    double c2 = ex * (fxx * ex + fxy * ey) + ey * (fxy * ex + fyy * ey);
    if (!(c2 < -R.sdd)) return false;
    double t = -(fx * ex + fy * ey) / c2;
    if (fabs(t * ex) <= dx / 2.0 && fabs(t * ey) <= dy / 2.0) {
        *px = R.x[i] + t * ex;
        *py = R.y[j] + t * ey;
        return true;
    }
    return false;
}

// Blocks per group of the two-level count prefix: a compaction block adds
// the group sums before its own group and the counts before it in its group.
constexpr int kRidgeGroup = 64;

__global__ void __launch_bounds__(kRidgeThreads)
ridge_flag_kernel(RidgeIn R, uint8_t* __restrict__ mask, double2* __restrict__ rpts,
                  unsigned int* __restrict__ block_count, unsigned int* __restrict__ group_count)
{
    const long n = (long)R.nx * R.ny;
    double dx, dy;
    ridge_spacing(R, &dx, &dy);
    const double fmin = R.fmin_ptr ? *R.fmin_ptr : R.fmin_val;
    const long base = (long)blockIdx.x * R.rounds * kRidgeThreads;
    unsigned int c = 0;
#pragma unroll 1
    for (int r = 0; r < R.rounds; ++r) {
        long k = base + (long)r * kRidgeThreads + threadIdx.x;
        if (k >= n) break;
        double px = 0.0, py = 0.0;
        bool on = ridge_at(R, fmin, dx, dy, k, &px, &py);
        mask[k] = on ? 1 : 0;
        if (rpts) rpts[k] = on ? make_double2(px, py) : make_double2(0.0, 0.0);
        c += on;
    }
    __shared__ unsigned int tot;
    if (threadIdx.x == 0) tot = 0;
    __syncthreads();
    if (c) atomicAdd(&tot, c);
    __syncthreads();
    if (threadIdx.x == 0) {
        block_count[blockIdx.x] = tot;
        if (tot) atomicAdd(&group_count[blockIdx.x / kRidgeGroup], tot);
    }
}

// The block's first output slot is the sum of the counts of the blocks before
// it: the group sums of the groups before its own plus the counts before it in
// its group (a few hundred loads at most on a 4001 x 4001 field: no separate
// scan launch); the last block also writes the total.
__global__ void __launch_bounds__(kRidgeThreads)
ridge_compact_kernel(RidgeIn R, const uint8_t* __restrict__ mask,
                     const unsigned int* __restrict__ block_count,
                     const unsigned int* __restrict__ group_count, const double2* __restrict__ full,
                     double2* __restrict__ out, int64_t* __restrict__ n_out)
{
    __shared__ unsigned int wsum[kRidgeThreads / 32];
    __shared__ unsigned long long wpre[kRidgeThreads / 32];
    const long n = (long)R.nx * R.ny;
    double dx, dy;
    ridge_spacing(R, &dx, &dy);
    const double fmin = R.fmin_ptr ? *R.fmin_ptr : R.fmin_val;
    const long base = (long)blockIdx.x * R.rounds * kRidgeThreads;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long pre = 0;
    const unsigned g0 = blockIdx.x / kRidgeGroup;
    for (unsigned q = threadIdx.x; q < g0; q += blockDim.x) pre += group_count[q];
    for (unsigned b = g0 * kRidgeGroup + threadIdx.x; b < blockIdx.x; b += blockDim.x)
        pre += block_count[b];
    for (int o = 16; o > 0; o >>= 1) pre += __shfl_xor_sync(0xffffffffu, pre, o);
    if (lane == 0) wpre[warp] = pre;
    __syncthreads();
    unsigned long long run = 0;
    for (int w = 0; w < kRidgeThreads / 32; ++w) run += wpre[w];
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
        *n_out = (int64_t)(run + block_count[blockIdx.x]);
#pragma unroll 1
    for (int r = 0; r < R.rounds; ++r) {
        long k = base + (long)r * kRidgeThreads + threadIdx.x;
        bool on = k < n && mask[k];
        unsigned int bal = __ballot_sync(0xffffffffu, on);
        if (lane == 0) wsum[warp] = __popc(bal);
        __syncthreads();
        unsigned int before = 0, total = 0;
        for (int w = 0; w < kRidgeThreads / 32; ++w) {
            unsigned int v = wsum[w];
            before += (w < warp) ? v : 0;
            total += v;
        }
        if (on) {
            double px = 0.0, py = 0.0;
            if (full) {  // the flag pass stored every point: gather it
                const double2 v = full[k];
                px = v.x;
                py = v.y;
            } else {  // re-evaluate the stencil at the ridge point only
                ridge_at(R, fmin, dx, dy, k, &px, &py);
            }
            unsigned int rank = before + __popc(bal & ((1u << lane) - 1u));
            out[run + rank] = make_double2(px, py);
        }
        run += total;
        __syncthreads();
    }
}

}  // namespace nbcs

using namespace nbcs;

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

extern "C" size_t nbcs_percentile_scratch_bytes(int64_t n)
{
    (void)n;
    return align256(sizeof(SelScratch));
}

extern "C" int nbcs_percentile(const double* f, int64_t n, double q, double* out, void* scratch,
                               size_t scratch_bytes, void* stream)
{
    NBCS_RANGE();
    if (n < 1 || !f || !out) return set_error(NBCS_ERR_INVALID, "percentile: empty input or NULL");
    if (!(q >= 0.0 && q <= 100.0)) return set_error(NBCS_ERR_INVALID, "percentile: q outside [0, 100]");
    if (!scratch || scratch_bytes < sizeof(SelScratch))
        return set_error(NBCS_ERR_SCRATCH, "percentile: scratch needs %zu bytes", sizeof(SelScratch));
    return percentile_enqueue(f, n, q, out, static_cast<SelScratch*>(scratch), as_stream(stream));
}

static long ridge_blocks(int32_t nx, int32_t ny)
{
    long n = (long)nx * ny;
    long per = (long)ridge_rounds(n) * kRidgeThreads;
    return (n + per - 1) / per;
}

extern "C" size_t nbcs_ridge_scratch_bytes(int32_t nx, int32_t ny)
{
    if (nx < 0 || ny < 0) return 0;
    long nb = ridge_blocks(nx, ny);
    const long ng = (nb + kRidgeGroup - 1) / kRidgeGroup;
    return align256(sizeof(SelScratch)) + align256(sizeof(unsigned int) * (size_t)nb) +
           align256(sizeof(unsigned int) * (size_t)ng) + align256((size_t)nx * ny);
}

// Ridge flags, points and compaction with the threshold f_min either taken
// from the percentile selection (use_percentile, percentile != 0) or given.
static int ridge_run(const double* f, const double* evec_max, const double* x, int32_t nx,
                     const double* y, int32_t ny, double dx, double dy, double sdd_thresh,
                     bool use_percentile, double percentile, double f_min, uint8_t* mask_out,
                     double* rpts_full, double* pts_out, int64_t* n_out, void* scratch,
                     size_t scratch_bytes, void* stream)
{
    if (nx < 2 || ny < 2) return set_error(NBCS_ERR_INVALID, "ridge_pts: need nx, ny >= 2");
    if (!f || !evec_max || !x || !y || !pts_out || !n_out)
        return set_error(NBCS_ERR_INVALID, "ridge_pts: NULL array");
    if ((reinterpret_cast<uintptr_t>(evec_max) | reinterpret_cast<uintptr_t>(pts_out) |
         reinterpret_cast<uintptr_t>(rpts_full)) & 15)
        return set_error(NBCS_ERR_INVALID, "ridge_pts: evec/pts arrays must be 16-byte aligned");
    if (use_percentile && !(percentile >= 0.0 && percentile <= 100.0))
        return set_error(NBCS_ERR_INVALID, "ridge_pts: percentile outside [0, 100]");
    size_t need = nbcs_ridge_scratch_bytes(nx, ny);
    if (!scratch || scratch_bytes < need)
        return set_error(NBCS_ERR_SCRATCH, "ridge_pts: scratch needs %zu bytes", need);
    cudaStream_t st = as_stream(stream);
    const long n = (long)nx * ny, nb = ridge_blocks(nx, ny);
    char* p = static_cast<char*>(scratch);
    SelScratch* sel = reinterpret_cast<SelScratch*>(p);
    p += align256(sizeof(SelScratch));
    unsigned int* cnt = reinterpret_cast<unsigned int*>(p);
    p += align256(sizeof(unsigned int) * (size_t)nb);
    const long ng = (nb + kRidgeGroup - 1) / kRidgeGroup;
    unsigned int* gcnt = reinterpret_cast<unsigned int*>(p);
    p += align256(sizeof(unsigned int) * (size_t)ng);
    uint8_t* mask = mask_out ? mask_out : reinterpret_cast<uint8_t*>(p);

    RidgeIn R;
    R.f = f;
    R.ev = reinterpret_cast<const double2*>(evec_max);
    R.x = x;
    R.y = y;
    R.nx = nx;
    R.ny = ny;
    R.sdd = sdd_thresh;
    R.dx = dx;
    R.dy = dy;
    R.rounds = ridge_rounds(n);
    R.fmin_ptr = nullptr;
    R.fmin_val = use_percentile ? 0.0 : f_min;
    if (use_percentile && percentile != 0.0) {  // ridges.py:48-51
        int rc = percentile_enqueue(f, n, percentile, nullptr, sel, st);
        if (rc) return rc;
        R.fmin_ptr = &sel->st.result;
    }
    NBCS_CUDA_TRY(cudaMemsetAsync(gcnt, 0, sizeof(unsigned int) * (size_t)ng, st));
    ridge_flag_kernel<<<(unsigned)nb, kRidgeThreads, 0, st>>>(
        R, mask, reinterpret_cast<double2*>(rpts_full), cnt, gcnt);
    NBCS_LAUNCH_CHECK();
    ridge_compact_kernel<<<(unsigned)nb, kRidgeThreads, 0, st>>>(
        R, mask, cnt, gcnt, reinterpret_cast<const double2*>(rpts_full),
        reinterpret_cast<double2*>(pts_out), n_out);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

extern "C" int nbcs_ridge_pts(const double* f, const double* evec_max, const double* x, int32_t nx,
                              const double* y, int32_t ny, double sdd_thresh, double percentile,
                              uint8_t* mask_out, double* rpts_full, double* pts_out,
                              int64_t* n_out, void* scratch, size_t scratch_bytes, void* stream)
{
    NBCS_RANGE();
    return ridge_run(f, evec_max, x, nx, y, ny, NAN, NAN, sdd_thresh, true, percentile, 0.0,
                     mask_out, rpts_full, pts_out, n_out, scratch, scratch_bytes, stream);
}

extern "C" int nbcs_ridge_pts_fmin(const double* f, const double* evec_max, const double* x,
                                   int32_t nx, const double* y, int32_t ny, double dx, double dy,
                                   double sdd_thresh, double f_min, uint8_t* mask_out,
                                   double* rpts_full, double* pts_out, int64_t* n_out,
                                   void* scratch, size_t scratch_bytes, void* stream)
{
    NBCS_RANGE();
    if (!(dx > 0.0 || dx < 0.0) || !(dy > 0.0 || dy < 0.0))
        return set_error(NBCS_ERR_INVALID, "ridge_pts_fmin: dx, dy must be nonzero");
    return ridge_run(f, evec_max, x, nx, y, ny, dx, dy, sdd_thresh, false, 0.0, f_min, mask_out,
                     rpts_full, pts_out, n_out, scratch, scratch_bytes, stream);
}

// ---------------------------------------------------------------------------
// Allocation-free ridge extraction.
//
// Some callers cannot allocate device memory: a plugin whose host program
// keeps every cudaMalloc to itself (for example inside its time-step loop), or
// a caller that binds this library through a thin FFI and has no device
// allocator of its own.  nbcs_ridge_pts_noalloc gives them ridge extraction
// without a scratch argument: its scratch is the file-scope array below,
// sized for grids of up to NBCS_RIDGE_NOALLOC_MAX_POINTS points (about 8.4 MB,
// held by every GPU that loads the library until the process exits).
//
// The array's name is only a host-side stand-in, so the device address is
// looked up with cudaGetSymbolAddress, once per device, on the first call made
// with that device current (make that first call before any stream capture).
// The address is cached per device ordinal, i.e. for the runtime's primary
// context; it is not refreshed after cudaDeviceReset.
// Every call shares the array and leaves its contents behind; the kernels
// re-initialise everything they read (the selection state and histogram, the
// per-block and per-group counts and the mask), and calls whose work overlaps
// on the GPU race on it.

namespace nbcs {

constexpr size_t align256c(size_t b) { return (b + 255) & ~(size_t)255; }
// ridge_blocks() is at most kRidgeFillBlocks + 1 below 8 rounds, n / kRidgeTile
// rounded up at 8 rounds
constexpr long kNoallocBlocks =
    (NBCS_RIDGE_NOALLOC_MAX_POINTS + kRidgeTile - 1) / kRidgeTile > kRidgeFillBlocks + 1
        ? (NBCS_RIDGE_NOALLOC_MAX_POINTS + kRidgeTile - 1) / kRidgeTile
        : kRidgeFillBlocks + 1;
constexpr size_t kNoallocScratchBytes =
    align256c(sizeof(SelScratch)) + align256c(sizeof(unsigned int) * kNoallocBlocks) +
    align256c(sizeof(unsigned int) * ((kNoallocBlocks + kRidgeGroup - 1) / kRidgeGroup)) +
    align256c((size_t)NBCS_RIDGE_NOALLOC_MAX_POINTS);

static __device__ __align__(256) unsigned char g_ridge_noalloc_scratch[kNoallocScratchBytes];

static int noalloc_scratch(void** out)
{
    static std::mutex mu;
    static void* addr[64] = {nullptr};
    int dev = 0;
    NBCS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return set_error(NBCS_ERR_INVALID, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        NBCS_CUDA_TRY(cudaGetSymbolAddress(&p, g_ridge_noalloc_scratch));
        addr[dev] = p;
    }
    *out = addr[dev];
    return NBCS_OK;
}

}  // namespace nbcs

extern "C" size_t nbcs_ridge_noalloc_scratch_bytes(void) { return nbcs::kNoallocScratchBytes; }

extern "C" int nbcs_ridge_pts_noalloc(const double* f, const double* evec_max, const double* x,
                                      int32_t nx, const double* y, int32_t ny, double sdd_thresh,
                                      double percentile, uint8_t* mask_out, double* rpts_full,
                                      double* pts_out, int64_t* n_out, void* stream)
{
    NBCS_RANGE();
    if (nx < 0 || ny < 0 || (long)nx * ny > NBCS_RIDGE_NOALLOC_MAX_POINTS)
        return set_error(NBCS_ERR_INVALID,
                         "ridge_pts_noalloc: %d x %d grid exceeds the fixed scratch limit of %ld "
                         "points; use nbcs_ridge_pts with caller scratch",
                         nx, ny, (long)NBCS_RIDGE_NOALLOC_MAX_POINTS);
    void* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    return nbcs_ridge_pts(f, evec_max, x, nx, y, ny, sdd_thresh, percentile, mask_out, rpts_full,
                          pts_out, n_out, scratch, kNoallocScratchBytes, stream);
}
