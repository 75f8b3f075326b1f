// Learned step-size proposer: an 8 -> 64 -> 64 -> 1 MLP (ReLU) with BF16
// weights and FP32 accumulation on the tensor cores (mma.sync m16n8k16).
//
// A warp evaluates 32 samples at once (two 16-row tiles).  Inside the
// integrator those are the warp's 32 particles; in training they are 32
// logged steps.  Layer 1 and 2 outputs stay in registers: the FP32
// accumulator tile of an m16n8 product is exactly the A-operand fragment of
// the next layer's m16k16 step once packed to BF16.
//
// Device weight blob (nbcs_mlp_* entry points; 16-byte aligned):
//   MlpConsts (feature mean / inverse std, target mean / std, b1, b2, w3, b3)
//   W1 bf16 [64][16]  (out, in; inputs 8..15 are zero padding)
//   W2 bf16 [64][64]  (out, in)
#pragma once

#include <cuda_bf16.h>

#include "nbcs_internal.cuh"

namespace nbcs {

constexpr int kMlpIn = 8, kMlpInPad = 16, kMlpHid = 64;
// FP32 master parameter vector: W1[64][8], b1[64], W2[64][64], b2[64], w3[64], b3
constexpr int kMlpOffW1 = 0, kMlpOffB1 = 512, kMlpOffW2 = 576, kMlpOffB2 = 4672, kMlpOffW3 = 4736,
              kMlpOffB3 = 4800, kMlpParams = 4801;

struct MlpConsts {
    float mu[kMlpIn], inv_sigma[kMlpIn];
    float out_mu, out_sigma, b3, pad0;
    float b1[kMlpHid], b2[kMlpHid], w3[kMlpHid];
};

struct MlpBlob {
    MlpConsts k;
    __nv_bfloat16 w1[kMlpHid * kMlpInPad];
    __nv_bfloat16 w2[kMlpHid * kMlpHid];
};

__device__ __forceinline__ void mma_bf16_16816(float* d, const uint32_t* a, const uint32_t* b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// Copy a blob into shared memory (whole block; call before __syncthreads()).
__device__ __forceinline__ void mlp_stage(const MlpBlob* __restrict__ g, MlpBlob* s)
{
    const int n = (int)(sizeof(MlpBlob) / 16);
    const int4* src = reinterpret_cast<const int4*>(g);
    int4* dst = reinterpret_cast<int4*>(s);
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// B fragment (k16 x n8) of W^T for n-tile nt, k-step ks, from a row-major
// [out][in] weight matrix with `ld` inputs per row.
__device__ __forceinline__ void load_b_frag(const __nv_bfloat16* w, int ld, int nt, int ks,
                                            uint32_t* b)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* row = w + (size_t)(nt * 8 + g) * ld + ks * 16 + 2 * t;
    b[0] = *reinterpret_cast<const uint32_t*>(row);
    b[1] = *reinterpret_cast<const uint32_t*>(row + 8);
}

// Layers 1 and 2 for the warp's 32 samples.  `xs` holds the standardised
// inputs as bf16 [32][16] (row = sample, columns 8..15 zero).  On return,
// h2[mt][nt][4] holds ReLU(layer-2) in accumulator layout; h1 (optional)
// receives layer-1 activations packed as layer-2 A fragments and z1/z2 masks
// are implied by the zeros of the ReLU outputs.
__device__ __forceinline__ void mlp_hidden(const MlpBlob& W, const __nv_bfloat16* xs,
                                           float h2[2][8][4], uint32_t a1[2][4][4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        uint32_t ax[4];
        const __nv_bfloat16* r0 = xs + (mt * 16 + g) * kMlpInPad + 2 * t;
        const __nv_bfloat16* r1 = r0 + 8 * kMlpInPad;
        ax[0] = *reinterpret_cast<const uint32_t*>(r0);
        ax[1] = *reinterpret_cast<const uint32_t*>(r1);
        ax[2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
        ax[3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
        float h1[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float bb0 = W.k.b1[nt * 8 + 2 * t], bb1 = W.k.b1[nt * 8 + 2 * t + 1];
            h1[nt][0] = bb0;
            h1[nt][1] = bb1;
            h1[nt][2] = bb0;
            h1[nt][3] = bb1;
            uint32_t b[2];
            load_b_frag(W.w1, kMlpInPad, nt, 0, b);
            mma_bf16_16816(h1[nt], ax, b);
        }
        // ReLU and repack as the A operand of layer 2 (k-step ks = n-tiles 2ks, 2ks+1)
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            const float* c0 = h1[2 * ks];
            const float* c1 = h1[2 * ks + 1];
            a1[mt][ks][0] = pack_bf16(fmaxf(c0[0], 0.f), fmaxf(c0[1], 0.f));
            a1[mt][ks][1] = pack_bf16(fmaxf(c0[2], 0.f), fmaxf(c0[3], 0.f));
            a1[mt][ks][2] = pack_bf16(fmaxf(c1[0], 0.f), fmaxf(c1[1], 0.f));
            a1[mt][ks][3] = pack_bf16(fmaxf(c1[2], 0.f), fmaxf(c1[3], 0.f));
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float bb0 = W.k.b2[nt * 8 + 2 * t], bb1 = W.k.b2[nt * 8 + 2 * t + 1];
            h2[mt][nt][0] = bb0;
            h2[mt][nt][1] = bb1;
            h2[mt][nt][2] = bb0;
            h2[mt][nt][3] = bb1;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                uint32_t b[2];
                load_b_frag(W.w2, kMlpHid, nt, ks, b);
                mma_bf16_16816(h2[mt][nt], a1[mt][ks], b);
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) h2[mt][nt][e] = fmaxf(h2[mt][nt][e], 0.f);
        }
    }
}

// Output layer: out[row] for the 4 rows this lane's group owns
// (mt*16 + g and mt*16 + g + 8), reduced over the 4 lanes of the group.
__device__ __forceinline__ void mlp_out_rows(const MlpBlob& W, const float h2[2][8][4],
                                             float out[2][2])
{
    const int lane = threadIdx.x & 31, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float w0 = W.k.w3[nt * 8 + 2 * t], w1 = W.k.w3[nt * 8 + 2 * t + 1];
            s0 = fmaf(h2[mt][nt][0], w0, fmaf(h2[mt][nt][1], w1, s0));
            s1 = fmaf(h2[mt][nt][2], w0, fmaf(h2[mt][nt][3], w1, s1));
        }
        s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
        s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
        s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
        s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
        out[mt][0] = s0 + W.k.b3;
        out[mt][1] = s1 + W.k.b3;
    }
}

// Standardise a lane's 8 raw features into row `lane` of xs (bf16, padded).
__device__ __forceinline__ void mlp_put_features(const MlpBlob& W, const float* f,
                                                 __nv_bfloat16* xs)
{
    const int lane = threadIdx.x & 31;
    __nv_bfloat16* row = xs + lane * kMlpInPad;
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i)
        row[i] = __float2bfloat16_rn((f[i] - W.k.mu[i]) * W.k.inv_sigma[i]);
#pragma unroll
    for (int i = kMlpIn; i < kMlpInPad; ++i) row[i] = __float2bfloat16_rn(0.f);
}

// Inference-only forward pass of rows 0 .. 16*MT-1 of xs into outs[row] (net
// output before the target de-standardisation).  Same arithmetic, in the same
// order, as mlp_hidden + mlp_out_rows, but layer 2 runs one n-tile at a time
// straight into the output dot product, so only the layer-1 A fragments stay
// live (~40 registers instead of ~100: this sits inside the integrator loop,
// where registers decide occupancy).
template <int MT>
__device__ __forceinline__ void mlp_rows(const MlpBlob& W, const __nv_bfloat16* xs, float* outs)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
        uint32_t ax[4];
        const __nv_bfloat16* r0 = xs + (mt * 16 + g) * kMlpInPad + 2 * t;
        const __nv_bfloat16* r1 = r0 + 8 * kMlpInPad;
        ax[0] = *reinterpret_cast<const uint32_t*>(r0);
        ax[1] = *reinterpret_cast<const uint32_t*>(r1);
        ax[2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
        ax[3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
        uint32_t a1[4][4];
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            float c[2][4];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int nt = 2 * ks + h;
                const float bb0 = W.k.b1[nt * 8 + 2 * t], bb1 = W.k.b1[nt * 8 + 2 * t + 1];
                c[h][0] = bb0;
                c[h][1] = bb1;
                c[h][2] = bb0;
                c[h][3] = bb1;
                uint32_t b[2];
                load_b_frag(W.w1, kMlpInPad, nt, 0, b);
                mma_bf16_16816(c[h], ax, b);
            }
            a1[ks][0] = pack_bf16(fmaxf(c[0][0], 0.f), fmaxf(c[0][1], 0.f));
            a1[ks][1] = pack_bf16(fmaxf(c[0][2], 0.f), fmaxf(c[0][3], 0.f));
            a1[ks][2] = pack_bf16(fmaxf(c[1][0], 0.f), fmaxf(c[1][1], 0.f));
            a1[ks][3] = pack_bf16(fmaxf(c[1][2], 0.f), fmaxf(c[1][3], 0.f));
        }
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float bb0 = W.k.b2[nt * 8 + 2 * t], bb1 = W.k.b2[nt * 8 + 2 * t + 1];
            float c[4] = {bb0, bb1, bb0, bb1};
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                uint32_t b[2];
                load_b_frag(W.w2, kMlpHid, nt, ks, b);
                mma_bf16_16816(c, a1[ks], b);
            }
            const float w0 = W.k.w3[nt * 8 + 2 * t], w1 = W.k.w3[nt * 8 + 2 * t + 1];
            s0 = fmaf(fmaxf(c[0], 0.f), w0, fmaf(fmaxf(c[1], 0.f), w1, s0));
            s1 = fmaf(fmaxf(c[2], 0.f), w0, fmaf(fmaxf(c[3], 0.f), w1, s1));
        }
        s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
        s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
        s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
        s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
        if (t == 0) {
            outs[mt * 16 + g] = s0 + W.k.b3;
            outs[mt * 16 + g + 8] = s1 + W.k.b3;
        }
    }
}

// Whole-warp inference: every lane passes its features, gets its prediction
// (in target units: out_mu + out_sigma * net).  All 32 lanes must call it.
__device__ __forceinline__ float mlp_predict_warp(const MlpBlob& W, const float* feat,
                                                  __nv_bfloat16* xs, float* outs)
{
    const int lane = threadIdx.x & 31;
    mlp_put_features(W, feat, xs);
    __syncwarp();
    mlp_rows<2>(W, xs, outs);
    __syncwarp();
    float r = fmaf(W.k.out_sigma, outs[lane], W.k.out_mu);
    __syncwarp();
    return r;
}

// Inference for a warp whose lane groups of LP lanes share one sample: the
// group leader's features go to row lane / LP, so 32 / LP rows (one 16-row
// tile for LP >= 2) are evaluated.  All 32 lanes must call it; every lane of
// a group gets the group's prediction.
template <int LP>
__device__ __forceinline__ float mlp_predict_groups(const MlpBlob& W, const float* feat,
                                                    __nv_bfloat16* xs, float* outs)
{
    const int lane = threadIdx.x & 31;
    if ((lane & (LP - 1)) == 0) {
        __nv_bfloat16* row = xs + (lane / LP) * kMlpInPad;
#pragma unroll
        for (int i = 0; i < kMlpIn; ++i)
            row[i] = __float2bfloat16_rn((feat[i] - W.k.mu[i]) * W.k.inv_sigma[i]);
#pragma unroll
        for (int i = kMlpIn; i < kMlpInPad; ++i) row[i] = __float2bfloat16_rn(0.f);
    }
    __syncwarp();
    mlp_rows<(32 / LP + 15) / 16>(W, xs, outs);
    __syncwarp();
    float r = fmaf(W.k.out_sigma, outs[lane / LP], W.k.out_mu);
    __syncwarp();
    return r;
}

}  // namespace nbcs
