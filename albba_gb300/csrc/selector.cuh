// Direction selector: level features and the 8 -> 32 -> 32 -> 3 ReLU MLP
// (device inference by one warp, host inference for the host-driven loop).
// The reference picks a kernel with a fixed frontier-size threshold
// (bfs/src/bfs_SELLCSv2.c:283-284, 302, 344, 356); the MLP has no
// counterpart there.
#pragma once

#include "dev.cuh"

namespace alb {

constexpr int kMlpIn = 8, kMlpH = 32, kMlpOut = 3;
constexpr int kMlpW1 = 0, kMlpB1 = kMlpW1 + kMlpH * kMlpIn, kMlpW2 = kMlpB1 + kMlpH,
              kMlpB2 = kMlpW2 + kMlpH * kMlpH, kMlpW3 = kMlpB2 + kMlpH,
              kMlpB3 = kMlpW3 + kMlpOut * kMlpH, kMlpParams = kMlpB3 + kMlpOut;
static_assert(kMlpParams == 1443, "MLP parameter block");

// Eight level features, each scaled to roughly [0, 1]:
//  0 log2 frontier vertices   1 log2 frontier push entries
//  2 log2 unvisited vertices  3 log2 unvisited pull entries
//  4 level index              5 log2 mean degree
//  6 degree skew              7 fraction of bitmap words with unvisited rows
__host__ __device__ inline void level_features(const BfsCtl &c, float *f) {
    f[0] = log2f(1.0f + (float)c.nf) * (1.0f / 32.0f);
    f[1] = log2f(1.0f + (float)c.mf) * (1.0f / 32.0f);
    f[2] = log2f(1.0f + (float)c.nu) * (1.0f / 32.0f);
    f[3] = log2f(1.0f + (float)c.mu) * (1.0f / 32.0f);
    f[4] = fminf((float)c.level, 256.0f) * (1.0f / 64.0f);
    f[5] = log2f(1.0f + c.feat_mean_deg) * (1.0f / 8.0f);
    f[6] = c.feat_skew * (1.0f / 16.0f);
    f[7] = c.nwords > 0 ? (float)c.active_words / (float)c.nwords : 0.0f;
}

// Host forward pass: out[3] = predicted cost per variant.
inline void mlp_forward_host(const float *P, const float *x, float *out) {
    float h1[kMlpH], h2[kMlpH];
    for (int j = 0; j < kMlpH; j++) {
        float a = P[kMlpB1 + j];
        for (int i = 0; i < kMlpIn; i++) a += P[kMlpW1 + j * kMlpIn + i] * x[i];
        h1[j] = a > 0.f ? a : 0.f;
    }
    for (int j = 0; j < kMlpH; j++) {
        float a = P[kMlpB2 + j];
        for (int i = 0; i < kMlpH; i++) a += P[kMlpW2 + j * kMlpH + i] * h1[i];
        h2[j] = a > 0.f ? a : 0.f;
    }
    for (int k = 0; k < kMlpOut; k++) {
        float a = P[kMlpB3 + k];
        for (int i = 0; i < kMlpH; i++) a += P[kMlpW3 + k * kMlpH + i] * h2[i];
        out[k] = a;
    }
}

__host__ __device__ inline int argmin3(const float *o) {
    int b = 0;
    for (int k = 1; k < 3; k++)
        if (o[k] < o[b]) b = k;
    return b;
}

#ifdef __CUDACC__
// Warp-parallel forward pass (lane j owns hidden unit j); every lane returns
// the argmin variant. Must be called by a full warp. Each lane first issues
// all of its parameter loads (its rows of W1 and W2 as 16-byte loads, its
// biases, its column of W3), so the pass costs one memory round trip rather
// than one per layer; P must be 16-byte aligned (the parameter blocks are).
// P may point to global memory or to a shared-memory copy (generic loads).
__device__ inline int mlp_select_warp(const float *P, const float *x) {
    const int j = threadIdx.x & 31;
    const float4 *w1 = reinterpret_cast<const float4 *>(P + kMlpW1 + j * kMlpIn);
    const float4 *w2 = reinterpret_cast<const float4 *>(P + kMlpW2 + j * kMlpH);
    float4 r1[kMlpIn / 4], r2[kMlpH / 4];
#pragma unroll
    for (int i = 0; i < kMlpIn / 4; i++) r1[i] = w1[i];
#pragma unroll
    for (int i = 0; i < kMlpH / 4; i++) r2[i] = w2[i];
    const float b1 = P[kMlpB1 + j], b2 = P[kMlpB2 + j];
    float w3[kMlpOut], b3[kMlpOut];
#pragma unroll
    for (int k = 0; k < kMlpOut; k++) {
        w3[k] = P[kMlpW3 + k * kMlpH + j];
        b3[k] = P[kMlpB3 + k];
    }
    float a = b1;
#pragma unroll
    for (int i = 0; i < kMlpIn / 4; i++)
        a += r1[i].x * x[4 * i] + r1[i].y * x[4 * i + 1] + r1[i].z * x[4 * i + 2] +
             r1[i].w * x[4 * i + 3];
    const float h1 = a > 0.f ? a : 0.f;
    float b = b2;
#pragma unroll
    for (int i = 0; i < kMlpH / 4; i++) {
        b += r2[i].x * __shfl_sync(kFull, h1, 4 * i) + r2[i].y * __shfl_sync(kFull, h1, 4 * i + 1) +
             r2[i].z * __shfl_sync(kFull, h1, 4 * i + 2) + r2[i].w * __shfl_sync(kFull, h1, 4 * i + 3);
    }
    const float h2 = b > 0.f ? b : 0.f;
    float o[kMlpOut];
#pragma unroll
    for (int k = 0; k < kMlpOut; k++) o[k] = warp_sum(w3[k] * h2) + b3[k];
    return argmin3(o);
}
#endif

}  // namespace alb
