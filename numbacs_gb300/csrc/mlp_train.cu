// Training and batch inference of the step-size MLP (mlp.cuh) on the tensor
// cores: BF16 operands, FP32 accumulation, mma.sync m16n8k16.
//
// One training kernel computes the loss gradient of a mini-batch: each block
// takes 128 samples at a time (four warps x 32), runs the forward pass,
// back-propagates to the per-sample layer deltas, and accumulates the weight
// gradients dW2 = dZ2^T A1 and dW1 = dZ1^T X with K = 128 samples per
// tensor-core product (operands staged in shared memory).  Accumulators stay
// in registers across the block's samples and are added to the global FP32
// gradient once per block.  Loss: mean squared error on standardised targets.
#include "mlp.cuh"

namespace nbcs {

constexpr int kTrainWarps = 4, kTrainRows = 32 * kTrainWarps;

struct TrainSmem {
    MlpBlob W;
    __nv_bfloat16 xs[kTrainRows * kMlpInPad];
    __nv_bfloat16 a1[kTrainRows * kMlpHid];
    __nv_bfloat16 dz2[kTrainRows * kMlpHid];
    __nv_bfloat16 dz1[kTrainRows * kMlpHid];
};

__device__ __forceinline__ uint32_t pack_bf16_raw(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    __nv_bfloat162 v;
    v.x = lo;
    v.y = hi;
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ float bf_lo(uint32_t v)
{
    return __bfloat162float(reinterpret_cast<__nv_bfloat162*>(&v)->x);
}
__device__ __forceinline__ float bf_hi(uint32_t v)
{
    return __bfloat162float(reinterpret_cast<__nv_bfloat162*>(&v)->y);
}

// B fragment of a row-major [k][n] matrix (element (k, n) = w[k * ld + n]).
__device__ __forceinline__ void load_b_frag_kn(const __nv_bfloat16* w, int ld, int nt, int ks,
                                               uint32_t* b)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int n = nt * 8 + g, k = ks * 16 + 2 * t;
    b[0] = pack_bf16_raw(w[k * ld + n], w[(k + 1) * ld + n]);
    b[1] = pack_bf16_raw(w[(k + 8) * ld + n], w[(k + 9) * ld + n]);
}

// A fragment of the transpose of a row-major [k][m] matrix (element (m, k) = w[k * ld + m]).
__device__ __forceinline__ void load_a_frag_t(const __nv_bfloat16* w, int ld, int mt, int ks,
                                              uint32_t* a)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int m = mt * 16 + g, k = ks * 16 + 2 * t;
    a[0] = pack_bf16_raw(w[k * ld + m], w[(k + 1) * ld + m]);
    a[1] = pack_bf16_raw(w[k * ld + m + 8], w[(k + 1) * ld + m + 8]);
    a[2] = pack_bf16_raw(w[(k + 8) * ld + m], w[(k + 9) * ld + m]);
    a[3] = pack_bf16_raw(w[(k + 8) * ld + m + 8], w[(k + 9) * ld + m + 8]);
}

__global__ void __launch_bounds__(32 * kTrainWarps)
mlp_grad_kernel(const MlpBlob* __restrict__ blob, const float* __restrict__ feats,
                const float* __restrict__ targets, long n, float scale, float* __restrict__ grad,
                float* __restrict__ loss)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    mlp_stage(blob, &S.W);
    __syncthreads();
    const MlpBlob& W = S.W;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float acc2[8][4], acc1[2][4];  // dW2 rows 16*warp.., dW1 rows 16*warp..
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc2[nt][e] = 0.f;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc1[nt][e] = 0.f;
    float gw3[8][2], gb2[8][2], gb1[8][2], gb3 = 0.f, lsum = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
        gw3[nt][0] = gw3[nt][1] = gb2[nt][0] = gb2[nt][1] = gb1[nt][0] = gb1[nt][1] = 0.f;

    for (long base = (long)blockIdx.x * kTrainRows; base < n; base += (long)gridDim.x * kTrainRows) {
        // ---- inputs of this warp's 32 samples
        const long s = base + warp * 32 + lane;
        float f[kMlpIn], tn = 0.f;
        const bool valid = s < n;
#pragma unroll
        for (int i = 0; i < kMlpIn; ++i) f[i] = valid ? feats[s * kMlpIn + i] : W.k.mu[i];
        if (valid) tn = (targets[s] - W.k.out_mu) / W.k.out_sigma;
        __nv_bfloat16* xs = S.xs + warp * 32 * kMlpInPad;
        mlp_put_features(W, f, xs);
        __syncwarp();
        // ---- forward
        float h2[2][8][4];
        uint32_t a1[2][4][4];
        mlp_hidden(W, xs, h2, a1);
        float o[2][2];
        mlp_out_rows(W, h2, o);
        // the 4 rows this lane's group owns: local rows g, g+8, 16+g, 24+g
        float dout[2][2];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = mt * 16 + g + 8 * h;
                const float tr = __shfl_sync(0xffffffffu, tn, r);
                const bool vr = base + warp * 32 + r < n;
                const float e = vr ? o[mt][h] - tr : 0.f;
                dout[mt][h] = 2.f * e * scale;
                if (t == 0) {
                    lsum = fmaf(e, e, lsum);
                    gb3 += dout[mt][h];
                }
            }
        // ---- output layer gradients, dZ2, A1 to shared memory
        __nv_bfloat16* a1s = S.a1 + warp * 32 * kMlpHid;
        __nv_bfloat16* dz2s = S.dz2 + warp * 32 * kMlpHid;
        float dz2[2][8][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int c = nt * 8 + 2 * t;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float d = dout[mt][e >> 1];
                    const float hv = h2[mt][nt][e];
                    gw3[nt][e & 1] = fmaf(d, hv, gw3[nt][e & 1]);
                    dz2[mt][nt][e] = hv > 0.f ? d * W.k.w3[c + (e & 1)] : 0.f;
                    gb2[nt][e & 1] += dz2[mt][nt][e];
                }
                const int r0 = mt * 16 + g;
                dz2s[r0 * kMlpHid + c] = __float2bfloat16_rn(dz2[mt][nt][0]);
                dz2s[r0 * kMlpHid + c + 1] = __float2bfloat16_rn(dz2[mt][nt][1]);
                dz2s[(r0 + 8) * kMlpHid + c] = __float2bfloat16_rn(dz2[mt][nt][2]);
                dz2s[(r0 + 8) * kMlpHid + c + 1] = __float2bfloat16_rn(dz2[mt][nt][3]);
            }
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const int r0 = mt * 16 + g, c = ks * 16 + 2 * t;
                *reinterpret_cast<uint32_t*>(a1s + r0 * kMlpHid + c) = a1[mt][ks][0];
                *reinterpret_cast<uint32_t*>(a1s + (r0 + 8) * kMlpHid + c) = a1[mt][ks][1];
                *reinterpret_cast<uint32_t*>(a1s + r0 * kMlpHid + c + 8) = a1[mt][ks][2];
                *reinterpret_cast<uint32_t*>(a1s + (r0 + 8) * kMlpHid + c + 8) = a1[mt][ks][3];
            }
        }
        // ---- dA1 = dZ2 W2 (rows = samples), dZ1 = dA1 * [A1 > 0]
        __nv_bfloat16* dz1s = S.dz1 + warp * 32 * kMlpHid;
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            uint32_t adz[4][4];
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                adz[ks][0] = pack_bf16(dz2[mt][2 * ks][0], dz2[mt][2 * ks][1]);
                adz[ks][1] = pack_bf16(dz2[mt][2 * ks][2], dz2[mt][2 * ks][3]);
                adz[ks][2] = pack_bf16(dz2[mt][2 * ks + 1][0], dz2[mt][2 * ks + 1][1]);
                adz[ks][3] = pack_bf16(dz2[mt][2 * ks + 1][2], dz2[mt][2 * ks + 1][3]);
            }
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                float da[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int ks = 0; ks < 4; ++ks) {
                    uint32_t b[2];
                    load_b_frag_kn(W.w2, kMlpHid, nt, ks, b);  // element (k=out2, n=in2) = W2[k][n]
                    mma_bf16_16816(da, adz[ks], b);
                }
                const uint32_t m0 = a1[mt][nt >> 1][(nt & 1) * 2];
                const uint32_t m1 = a1[mt][nt >> 1][(nt & 1) * 2 + 1];
                float dz[4];
                dz[0] = bf_lo(m0) > 0.f ? da[0] : 0.f;
                dz[1] = bf_hi(m0) > 0.f ? da[1] : 0.f;
                dz[2] = bf_lo(m1) > 0.f ? da[2] : 0.f;
                dz[3] = bf_hi(m1) > 0.f ? da[3] : 0.f;
                gb1[nt][0] += dz[0] + dz[2];
                gb1[nt][1] += dz[1] + dz[3];
                const int r0 = mt * 16 + g, c = nt * 8 + 2 * t;
                dz1s[r0 * kMlpHid + c] = __float2bfloat16_rn(dz[0]);
                dz1s[r0 * kMlpHid + c + 1] = __float2bfloat16_rn(dz[1]);
                dz1s[(r0 + 8) * kMlpHid + c] = __float2bfloat16_rn(dz[2]);
                dz1s[(r0 + 8) * kMlpHid + c + 1] = __float2bfloat16_rn(dz[3]);
            }
        }
        __syncthreads();
        // ---- weight gradients over the block's 128 samples: warp w owns output rows 16w..16w+15
#pragma unroll
        for (int ks = 0; ks < kTrainRows / 16; ++ks) {
            uint32_t a[4];
            load_a_frag_t(S.dz2, kMlpHid, warp, ks, a);  // (m = out2, k = sample)
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                uint32_t b[2];
                load_b_frag_kn(S.a1, kMlpHid, nt, ks, b);  // (k = sample, n = in2)
                mma_bf16_16816(acc2[nt], a, b);
            }
            uint32_t a_1[4];
            load_a_frag_t(S.dz1, kMlpHid, warp, ks, a_1);  // (m = out1, k = sample)
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
                uint32_t b[2];
                load_b_frag_kn(S.xs, kMlpInPad, nt, ks, b);  // (k = sample, n = input)
                mma_bf16_16816(acc1[nt], a_1, b);
            }
        }
        __syncthreads();
    }
    // ---- flush: weight matrices from the accumulators
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int r = warp * 16 + g, c = nt * 8 + 2 * t;
        atomicAdd(&grad[kMlpOffW2 + r * kMlpHid + c], acc2[nt][0]);
        atomicAdd(&grad[kMlpOffW2 + r * kMlpHid + c + 1], acc2[nt][1]);
        atomicAdd(&grad[kMlpOffW2 + (r + 8) * kMlpHid + c], acc2[nt][2]);
        atomicAdd(&grad[kMlpOffW2 + (r + 8) * kMlpHid + c + 1], acc2[nt][3]);
    }
    {
        const int r = warp * 16 + g, c = 2 * t;  // n-tile 0 holds the 8 real inputs
        atomicAdd(&grad[kMlpOffW1 + r * kMlpIn + c], acc1[0][0]);
        atomicAdd(&grad[kMlpOffW1 + r * kMlpIn + c + 1], acc1[0][1]);
        atomicAdd(&grad[kMlpOffW1 + (r + 8) * kMlpIn + c], acc1[0][2]);
        atomicAdd(&grad[kMlpOffW1 + (r + 8) * kMlpIn + c + 1], acc1[0][3]);
    }
    // ---- vectors: reduce over the 8 row groups (lanes with the same t), then add
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int o = 4; o < 32; o <<= 1) {
                gw3[nt][h] += __shfl_xor_sync(0xffffffffu, gw3[nt][h], o);
                gb2[nt][h] += __shfl_xor_sync(0xffffffffu, gb2[nt][h], o);
                gb1[nt][h] += __shfl_xor_sync(0xffffffffu, gb1[nt][h], o);
            }
    // loss and db3 were accumulated by lane t == 0 of each group only
    for (int o = 1; o < 32; o <<= 1) {
        lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
        gb3 += __shfl_xor_sync(0xffffffffu, gb3, o);
    }
    if (g == 0) {
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = nt * 8 + 2 * t + h;
                atomicAdd(&grad[kMlpOffW3 + c], gw3[nt][h]);
                atomicAdd(&grad[kMlpOffB2 + c], gb2[nt][h]);
                atomicAdd(&grad[kMlpOffB1 + c], gb1[nt][h]);
            }
    }
    if (lane == 0) {
        atomicAdd(loss, lsum);
        atomicAdd(&grad[kMlpOffB3], gb3);
    }
}

__global__ void __launch_bounds__(32 * kTrainWarps)
mlp_predict_kernel(const MlpBlob* __restrict__ blob, const float* __restrict__ feats, long n,
                   float* __restrict__ out)
{
    __shared__ MlpBlob W;
    __shared__ __align__(16) __nv_bfloat16 xs[kTrainWarps][32 * kMlpInPad];
    __shared__ float outs[kTrainWarps][32];
    mlp_stage(blob, &W);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (long base = (long)blockIdx.x * kTrainRows; base < n; base += (long)gridDim.x * kTrainRows) {
        const long s = base + warp * 32 + lane;
        float f[kMlpIn];
#pragma unroll
        for (int i = 0; i < kMlpIn; ++i) f[i] = s < n ? feats[s * kMlpIn + i] : W.k.mu[i];
        float p = mlp_predict_warp(W, f, xs[warp], outs[warp]);
        if (s < n) out[s] = p;
    }
}

// FP32 master parameters -> device blob (bf16 matrices, fp32 vectors); the
// normalisation constants already in the blob are left alone.
__global__ void mlp_pack_kernel(const float* __restrict__ p, MlpBlob* __restrict__ blob)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpHid * kMlpInPad;
         i += gridDim.x * blockDim.x) {
        int r = i / kMlpInPad, c = i % kMlpInPad;
        blob->w1[i] = __float2bfloat16_rn(c < kMlpIn ? p[kMlpOffW1 + r * kMlpIn + c] : 0.f);
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpHid * kMlpHid;
         i += gridDim.x * blockDim.x)
        blob->w2[i] = __float2bfloat16_rn(p[kMlpOffW2 + i]);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpHid; i += gridDim.x * blockDim.x) {
        blob->k.b1[i] = p[kMlpOffB1 + i];
        blob->k.b2[i] = p[kMlpOffB2 + i];
        blob->k.w3[i] = p[kMlpOffW3 + i];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) blob->k.b3 = p[kMlpOffB3];
}

// Adam with bias correction on the FP32 master vector.
__global__ void mlp_adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                                const float* __restrict__ g, int n, float lr, float b1, float b2,
                                float eps, float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float gi = g[i];
        float mi = fmaf(b1, m[i], (1.f - b1) * gi);
        float vi = fmaf(b2, v[i], (1.f - b2) * gi * gi);
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace nbcs

using namespace nbcs;

extern "C" size_t nbcs_mlp_blob_bytes(void) { return sizeof(MlpBlob); }
extern "C" int nbcs_mlp_param_count(void) { return kMlpParams; }

extern "C" int nbcs_mlp_pack(const float* params, void* blob, void* stream)
{
    NBCS_RANGE();
    if (!params || !blob || (reinterpret_cast<uintptr_t>(blob) & 15))
        return set_error(NBCS_ERR_INVALID, "mlp_pack: NULL or misaligned arguments");
    mlp_pack_kernel<<<8, 256, 0, as_stream(stream)>>>(params, static_cast<MlpBlob*>(blob));
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

extern "C" int nbcs_mlp_predict(const void* blob, const float* feats, int64_t n, float* out,
                                void* stream)
{
    NBCS_RANGE();
    if (n < 0 || (n > 0 && (!blob || !feats || !out)))
        return set_error(NBCS_ERR_INVALID, "mlp_predict: bad arguments");
    if (n == 0) return NBCS_OK;
    long blocks = (n + kTrainRows - 1) / kTrainRows;
    if (blocks > (long)sm_count() * 8) blocks = (long)sm_count() * 8;
    mlp_predict_kernel<<<(unsigned)blocks, 32 * kTrainWarps, 0, as_stream(stream)>>>(
        static_cast<const MlpBlob*>(blob), feats, n, out);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

extern "C" int nbcs_mlp_grad(const void* blob, const float* feats, const float* targets, int64_t n,
                             float* grad, float* loss, void* stream)
{
    NBCS_RANGE();
    if (n <= 0 || !blob || !feats || !targets || !grad || !loss)
        return set_error(NBCS_ERR_INVALID, "mlp_grad: bad arguments");
    cudaStream_t s = as_stream(stream);
    NBCS_CUDA_TRY(cudaMemsetAsync(grad, 0, sizeof(float) * kMlpParams, s));
    NBCS_CUDA_TRY(cudaMemsetAsync(loss, 0, sizeof(float), s));
    const size_t smem = sizeof(TrainSmem);
    NBCS_CUDA_TRY(cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    long blocks = (n + kTrainRows - 1) / kTrainRows;
    if (blocks > (long)sm_count() * 2) blocks = (long)sm_count() * 2;
    const float scale = 1.0f / (float)n;
    mlp_grad_kernel<<<(unsigned)blocks, 32 * kTrainWarps, smem, s>>>(
        static_cast<const MlpBlob*>(blob), feats, targets, n, scale, grad, loss);
    NBCS_LAUNCH_CHECK();
    return NBCS_OK;
}

extern "C" int nbcs_mlp_adam(float* params, float* m, float* v, const float* grad, float lr,
                             float beta1, float beta2, float eps, int32_t step, void* blob,
                             void* stream)
{
    NBCS_RANGE();
    if (!params || !m || !v || !grad || step < 1)
        return set_error(NBCS_ERR_INVALID, "mlp_adam: bad arguments");
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    mlp_adam_kernel<<<8, 256, 0, as_stream(stream)>>>(params, m, v, grad, kMlpParams, lr, beta1,
                                                      beta2, eps, c1, c2);
    NBCS_LAUNCH_CHECK();
    if (blob) return nbcs_mlp_pack(params, blob, stream);
    return NBCS_OK;
}
