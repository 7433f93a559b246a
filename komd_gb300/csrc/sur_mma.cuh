// sur_mma.cuh -- the 32-64-64-1 MLP of the learned three-body term on the
// tensor cores (mma.sync m16n8k16, BF16 operands, FP32 accumulation), shared
// by inference (surrogate.cu) and training (sur_train.cu).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "surrogate.cuh"

namespace komd {

// ---------------------------------------------------------------------------
// MLP on the tensor cores: one warp per 16 sites (m16n8k16, BF16 in, FP32 acc)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// hardware tanh (PTX tanh.approx.f32, max relative error about 2^-11: below
// the BF16 rounding of the activations that follow)
__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void mma16816(float *c, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// B fragment (m16n8k16) of an N x K weight matrix stored in fragment order:
// for n-tile t, k-step s and lane (g = lane/4, tig = lane%4) one uint2 holding
// W[8t+g][16s+2tig .. +1] and W[8t+g][16s+8+2tig .. +1] (S = K/16 k-steps).
// One conflict-free 8-byte shared load per MMA.
__device__ __forceinline__ void load_frag(const __nv_bfloat16 *F, int S, int t, int s, int lane, uint32_t &b0,
                                          uint32_t &b1) {
    const uint2 v = reinterpret_cast<const uint2 *>(F)[(t * S + s) * 32 + lane];
    b0 = v.x;
    b1 = v.y;
}

// BF16 weights and FP32 biases staged in shared memory
struct SurW {
    const __nv_bfloat16 *w1, *w1t, *w2, *w2t;
    const float *b1, *b2, *w3;
};

// one 16-site tile on the tensor cores: thread (g = lane/4, tig = lane%4)
// reads its rows g and g + 8 of the features (xr0, xr1) and writes the same
// rows of dE/dx (dr0, dr1, which may alias xr0, xr1); E0, E1 return the MLP
// outputs (before b3 and scaling) of those rows, complete in the tig == 0 lanes
__device__ __forceinline__ void sur_mlp_tile(const SurW &W, const float *xr0, const float *xr1, bool v0, bool v1,
                                             float *dr0, float *dr1, float &E0, float &E1, int lane) {
    const int tig = lane & 3;
    // layer 1: Z1 = X W1^T  (X 16x32 -> 2 k-steps)
    uint32_t ax[2][4];
#pragma unroll
    for (int s = 0; s < 2; s++) {
        const int k = 16 * s + tig * 2;
        const float2 x00 = v0 ? *reinterpret_cast<const float2 *>(xr0 + k) : make_float2(0.f, 0.f);
        const float2 x10 = v1 ? *reinterpret_cast<const float2 *>(xr1 + k) : make_float2(0.f, 0.f);
        const float2 x01 = v0 ? *reinterpret_cast<const float2 *>(xr0 + k + 8) : make_float2(0.f, 0.f);
        const float2 x11 = v1 ? *reinterpret_cast<const float2 *>(xr1 + k + 8) : make_float2(0.f, 0.f);
        ax[s][0] = pack_bf16(x00.x, x00.y);
        ax[s][1] = pack_bf16(x10.x, x10.y);
        ax[s][2] = pack_bf16(x01.x, x01.y);
        ax[s][3] = pack_bf16(x11.x, x11.y);
    }
    float h1[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const int c = t * 8 + tig * 2;
        float acc[4] = {W.b1[c], W.b1[c + 1], W.b1[c], W.b1[c + 1]};
#pragma unroll
        for (int s = 0; s < 2; s++) {
            uint32_t b0, b1;
            load_frag(W.w1, kSurNF / 16, t, s, lane, b0, b1);
            mma16816(acc, ax[s], b0, b1);
        }
#pragma unroll
        for (int q = 0; q < 4; q++) h1[t][q] = tanh_fast(acc[q]);
    }
    // layer 2: Z2 = H1 W2^T (4 k-steps from the h1 fragments)
    uint32_t ah[4][4];
#pragma unroll
    for (int s = 0; s < 4; s++) {
        ah[s][0] = pack_bf16(h1[2 * s][0], h1[2 * s][1]);
        ah[s][1] = pack_bf16(h1[2 * s][2], h1[2 * s][3]);
        ah[s][2] = pack_bf16(h1[2 * s + 1][0], h1[2 * s + 1][1]);
        ah[s][3] = pack_bf16(h1[2 * s + 1][2], h1[2 * s + 1][3]);
    }
    float h2[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const int c = t * 8 + tig * 2;
        float acc[4] = {W.b2[c], W.b2[c + 1], W.b2[c], W.b2[c + 1]};
#pragma unroll
        for (int s = 0; s < 4; s++) {
            uint32_t b0, b1;
            load_frag(W.w2, kSurH / 16, t, s, lane, b0, b1);
            mma16816(acc, ah[s], b0, b1);
        }
#pragma unroll
        for (int q = 0; q < 4; q++) h2[t][q] = tanh_fast(acc[q]);
    }
    // layer 3 and dE/dz2 = w3 (1 - h2^2)
    float e0 = 0.f, e1 = 0.f;
    uint32_t ad[4][4];
    float dz2[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const int c = t * 8 + tig * 2;
        e0 += W.w3[c] * h2[t][0] + W.w3[c + 1] * h2[t][1];
        e1 += W.w3[c] * h2[t][2] + W.w3[c + 1] * h2[t][3];
        dz2[t][0] = W.w3[c] * (1.f - h2[t][0] * h2[t][0]);
        dz2[t][1] = W.w3[c + 1] * (1.f - h2[t][1] * h2[t][1]);
        dz2[t][2] = W.w3[c] * (1.f - h2[t][2] * h2[t][2]);
        dz2[t][3] = W.w3[c + 1] * (1.f - h2[t][3] * h2[t][3]);
    }
    e0 += __shfl_xor_sync(0xffffffffu, e0, 1);
    e0 += __shfl_xor_sync(0xffffffffu, e0, 2);
    e1 += __shfl_xor_sync(0xffffffffu, e1, 1);
    e1 += __shfl_xor_sync(0xffffffffu, e1, 2);
    E0 = e0;
    E1 = e1;
#pragma unroll
    for (int s = 0; s < 4; s++) {
        ad[s][0] = pack_bf16(dz2[2 * s][0], dz2[2 * s][1]);
        ad[s][1] = pack_bf16(dz2[2 * s][2], dz2[2 * s][3]);
        ad[s][2] = pack_bf16(dz2[2 * s + 1][0], dz2[2 * s + 1][1]);
        ad[s][3] = pack_bf16(dz2[2 * s + 1][2], dz2[2 * s + 1][3]);
    }
    // dH1 = dZ2 W2  (B = W2^T rows), dZ1 = dH1 (1 - h1^2)
    uint32_t az[4][4];
    float dz1[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int s = 0; s < 4; s++) {
            uint32_t b0, b1;
            load_frag(W.w2t, kSurH / 16, t, s, lane, b0, b1);
            mma16816(acc, ad[s], b0, b1);
        }
#pragma unroll
        for (int q = 0; q < 4; q++) dz1[t][q] = acc[q] * (1.f - h1[t][q] * h1[t][q]);
    }
#pragma unroll
    for (int s = 0; s < 4; s++) {
        az[s][0] = pack_bf16(dz1[2 * s][0], dz1[2 * s][1]);
        az[s][1] = pack_bf16(dz1[2 * s][2], dz1[2 * s][3]);
        az[s][2] = pack_bf16(dz1[2 * s + 1][0], dz1[2 * s + 1][1]);
        az[s][3] = pack_bf16(dz1[2 * s + 1][2], dz1[2 * s + 1][3]);
    }
    // dX = dZ1 W1  (B = W1^T rows, n = feature); the rows may alias the input rows
    __syncwarp();
#pragma unroll
    for (int t = 0; t < 4; t++) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int s = 0; s < 4; s++) {
            uint32_t b0, b1;
            load_frag(W.w1t, kSurH / 16, t, s, lane, b0, b1);
            mma16816(acc, az[s], b0, b1);
        }
        const int c = t * 8 + tig * 2;
        if (v0) *reinterpret_cast<float2 *>(dr0 + c) = make_float2(acc[0], acc[1]);
        if (v1) *reinterpret_cast<float2 *>(dr1 + c) = make_float2(acc[2], acc[3]);
    }
}

// the fragment-ordered BF16 weights (16-byte copies), the FP32 biases and the
// output weights into shared memory; the block synchronises before use
__device__ __forceinline__ void sur_stage(const __nv_bfloat16 *w1, const __nv_bfloat16 *w1t, const __nv_bfloat16 *w2,
                                          const __nv_bfloat16 *w2t, const float *b1, const float *b2, const float *w3,
                                          __nv_bfloat16 *sW1, __nv_bfloat16 *sW1T, __nv_bfloat16 *sW2,
                                          __nv_bfloat16 *sW2T, float *sb1, float *sb2, float *sw3) {
    // 16-byte staging of the BF16 weights
    const uint4 *g1 = reinterpret_cast<const uint4 *>(w1), *g1t = reinterpret_cast<const uint4 *>(w1t);
    const uint4 *g2 = reinterpret_cast<const uint4 *>(w2), *g2t = reinterpret_cast<const uint4 *>(w2t);
    uint4 *s1 = reinterpret_cast<uint4 *>(sW1), *s1t = reinterpret_cast<uint4 *>(sW1T);
    uint4 *s2 = reinterpret_cast<uint4 *>(sW2), *s2t = reinterpret_cast<uint4 *>(sW2T);
    for (int t = threadIdx.x; t < kSurH * kSurNF / 8; t += blockDim.x) { s1[t] = g1[t]; s1t[t] = g1t[t]; }
    for (int t = threadIdx.x; t < kSurH * kSurH / 8; t += blockDim.x) { s2[t] = g2[t]; s2t[t] = g2t[t]; }
    for (int t = threadIdx.x; t < kSurH; t += blockDim.x) { sb1[t] = b1[t]; sb2[t] = b2[t]; sw3[t] = w3[t]; }
}

}  // namespace komd
