// 8-connected component labelling of a ridge mask (the scipy.ndimage.label
// call of ftle_ridges, extraction/ridges.py:219-222, structure = 3x3 ones).
//
// Union-find on the pixel grid: every pixel links to the smaller of two roots
// (compare-and-swap on the larger root), so a component's final root is its
// smallest row-major index -- its first pixel in raster order.  Numbering the
// roots in increasing index order (an order-preserving scan) then reproduces
// scipy's labels exactly: 1..n by first pixel, 0 for background.
//
// Kernels: init (parent = self or -1), merge (each foreground pixel unites
// with its W, NW, N, NE neighbours, which covers every 8-adjacency once),
// flatten (parent = root, read-only walk), root flags + per-block counts, block scan, root
// numbers, and labels of the non-root pixels.  Every loop is bounded: find()
// follows parent links that strictly decrease, and unite() gives up (setting
// an error flag) after a fixed number of failed swaps.
#include "nbcs_internal.cuh"

namespace nbcs {

constexpr int kLblThreads = 256;
constexpr int kUniteLimit = 1 << 20;

__device__ __forceinline__ int ccl_find(int* parent, int x)
{
    for (;;) {
        int p = parent[x];
        if (p == x) return x;
        // a link always points down to a smaller index of the same component
        if (!NBCS_CHECKED(p >= 0 && p < x, NBCS_CHECK_LABEL_LINK)) return x;
        int gp = parent[p];
        if (gp != p) parent[x] = gp;  // path halving: gp is an ancestor of x
        x = p;
    }
}

__device__ __forceinline__ void ccl_unite(int* parent, int a, int b, int* err)
{
    int ra = ccl_find(parent, a), rb = ccl_find(parent, b);
    for (int it = 0; ra != rb; ++it) {
        if (it >= kUniteLimit) {
            atomicExch(err, 1);
            return;
        }
        if (ra > rb) {
            int t = ra;
            ra = rb;
            rb = t;
        }
        int old = atomicCAS(&parent[rb], rb, ra);
        if (old == rb) return;
        rb = ccl_find(parent, old);
    }
}

__global__ void ccl_init_kernel(const uint8_t* __restrict__ mask, long n, int* __restrict__ parent)
{
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        parent[k] = mask[k] ? (int)k : -1;
}

__global__ void ccl_merge_kernel(int nx, int ny, int* parent, int* err)
{
    const long n = (long)nx * ny;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        if (parent[k] < 0) continue;
        const int i = (int)(k / ny), j = (int)(k - (long)i * ny);
        if (j > 0 && parent[k - 1] >= 0) ccl_unite(parent, (int)k, (int)(k - 1), err);
        if (i > 0) {
            const long up = k - ny;
            if (j > 0 && parent[up - 1] >= 0) ccl_unite(parent, (int)k, (int)(up - 1), err);
            if (parent[up] >= 0) ccl_unite(parent, (int)k, (int)up, err);
            if (j < ny - 1 && parent[up + 1] >= 0) ccl_unite(parent, (int)k, (int)(up + 1), err);
        }
    }
}

// After merging the roots no longer change, so a plain walk up the links finds
// them.  Flatten must not halve paths: a halving write racing with another
// thread's final `parent[x] = root` could put a non-root ancestor back.
__device__ __forceinline__ int ccl_root(const int* parent, int x)
{
    for (int p = parent[x]; p != x; p = parent[x]) {
        if (!NBCS_CHECKED(p >= 0 && p < x, NBCS_CHECK_LABEL_LINK)) return x;
        x = p;
    }
    return x;
}

__global__ void ccl_flatten_kernel(long n, int* parent)
{
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        if (parent[k] >= 0) parent[k] = ccl_root(parent, (int)k);
}

// one block per kLblThreads pixels: count the roots
__global__ void __launch_bounds__(kLblThreads)
ccl_count_kernel(long n, const int* __restrict__ parent, unsigned int* __restrict__ cnt)
{
    const long k = (long)blockIdx.x * kLblThreads + threadIdx.x;
    const bool root = k < n && parent[k] == (int)k;
    const int c = __syncthreads_count(root);
    if (threadIdx.x == 0) cnt[blockIdx.x] = (unsigned)c;
}

// exclusive scan of the per-block root counts (one block); total -> *nlabels
__global__ void __launch_bounds__(1024)
ccl_scan_kernel(const unsigned int* __restrict__ cnt, long nb, unsigned int* __restrict__ off,
                int* __restrict__ nlabels, const int* __restrict__ err)
{
    __shared__ unsigned int part[1024];
    const long per = (nb + blockDim.x - 1) / blockDim.x;
    const long b0 = (long)threadIdx.x * per;
    unsigned int s = 0;
    for (long q = 0; q < per; ++q)
        if (b0 + q < nb) s += cnt[b0 + q];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        unsigned int v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned int run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (long q = 0; q < per; ++q) {
        if (b0 + q < nb) {
            off[b0 + q] = run;
            run += cnt[b0 + q];
        }
    }
    if (threadIdx.x == blockDim.x - 1) *nlabels = *err ? -1 : (int)part[blockDim.x - 1];
}

// roots get 1 + (number of roots before them in row-major order)
__global__ void __launch_bounds__(kLblThreads)
ccl_number_kernel(long n, const int* __restrict__ parent, const unsigned int* __restrict__ off,
                  int* __restrict__ labels)
{
    __shared__ unsigned int wsum[kLblThreads / 32];
    const long k = (long)blockIdx.x * kLblThreads + threadIdx.x;
    const bool root = k < n && parent[k] == (int)k;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, root);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    unsigned int before = 0;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    if (root) labels[k] = (int)(off[blockIdx.x] + before + __popc(bal & ((1u << lane) - 1u)) + 1u);
}

__global__ void ccl_propagate_kernel(long n, const int* __restrict__ parent, int* __restrict__ labels)
{
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int p = parent[k];
        if (p < 0) labels[k] = 0;
        else if (p != (int)k && NBCS_CHECKED(p < k, NBCS_CHECK_LABEL_LINK)) labels[k] = labels[p];
    }
}

static inline size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace nbcs

using namespace nbcs;

extern "C" size_t nbcs_label8_scratch_bytes(int32_t nx, int32_t ny)
{
    if (nx < 0 || ny < 0) return 0;
    long n = (long)nx * ny, nb = (n + kLblThreads - 1) / kLblThreads;
    return a256(sizeof(int) * (size_t)n) + 2 * a256(sizeof(unsigned int) * (size_t)nb) + a256(sizeof(int));
}

extern "C" int nbcs_label8(const uint8_t* mask, int32_t nx, int32_t ny, int32_t* labels,
                           int32_t* nlabels, void* scratch, size_t scratch_bytes, void* stream)
{
    NBCS_RANGE();
    if (nx < 0 || ny < 0 || (long)nx * ny > 0x7fffffffL)
        return set_error(NBCS_ERR_INVALID, "label8: grid size out of range");
    const long n = (long)nx * ny;
    if (!mask || !labels || !nlabels) return set_error(NBCS_ERR_INVALID, "label8: NULL array");
    const size_t need = nbcs_label8_scratch_bytes(nx, ny);
    if (!scratch || scratch_bytes < need)
        return set_error(NBCS_ERR_SCRATCH, "label8: scratch needs %zu bytes", need);
    cudaStream_t s = as_stream(stream);
    if (n == 0) {
        NBCS_CUDA_TRY(cudaMemsetAsync(nlabels, 0, sizeof(int32_t), s));
        return NBCS_OK;
    }
    const long nb = (n + kLblThreads - 1) / kLblThreads;
    char* p = static_cast<char*>(scratch);
    int* parent = reinterpret_cast<int*>(p);
    p += a256(sizeof(int) * (size_t)n);
    unsigned int* cnt = reinterpret_cast<unsigned int*>(p);
    p += a256(sizeof(unsigned int) * (size_t)nb);
    unsigned int* off = reinterpret_cast<unsigned int*>(p);
    p += a256(sizeof(unsigned int) * (size_t)nb);
    int* err = reinterpret_cast<int*>(p);
    long g = nb;
    if (g > (long)sm_count() * 16) g = (long)sm_count() * 16;
    NBCS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
    ccl_init_kernel<<<(unsigned)g, kLblThreads, 0, s>>>(mask, n, parent);
    NBCS_LAUNCH_CHECK();
    ccl_merge_kernel<<<(unsigned)g, kLblThreads, 0, s>>>(nx, ny, parent, err);
    NBCS_LAUNCH_CHECK();
    ccl_flatten_kernel<<<(unsigned)g, kLblThreads, 0, s>>>(n, parent);
    NBCS_LAUNCH_CHECK();
    ccl_count_kernel<<<(unsigned)nb, kLblThreads, 0, s>>>(n, parent, cnt);
    NBCS_LAUNCH_CHECK();
    ccl_scan_kernel<<<1, 1024, 0, s>>>(cnt, nb, off, nlabels, err);
    NBCS_LAUNCH_CHECK();
    ccl_number_kernel<<<(unsigned)nb, kLblThreads, 0, s>>>(n, parent, off, labels);
    NBCS_LAUNCH_CHECK();
    ccl_propagate_kernel<<<(unsigned)g, kLblThreads, 0, s>>>(n, parent, labels);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}
