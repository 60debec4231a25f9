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
// the argmin variant. Must be called by a full warp.
__device__ inline int mlp_select_warp(const float *P, const float *x) {
    const int j = threadIdx.x & 31;
    float a = P[kMlpB1 + j];
#pragma unroll
    for (int i = 0; i < kMlpIn; i++) a += P[kMlpW1 + j * kMlpIn + i] * x[i];
    const float h1 = a > 0.f ? a : 0.f;
    float b = P[kMlpB2 + j];
#pragma unroll 8
    for (int i = 0; i < kMlpH; i++) b += P[kMlpW2 + j * kMlpH + i] * __shfl_sync(kFull, h1, i);
    const float h2 = b > 0.f ? b : 0.f;
    float o[kMlpOut];
#pragma unroll
    for (int k = 0; k < kMlpOut; k++) o[k] = warp_sum(P[kMlpW3 + k * kMlpH + j] * h2) + P[kMlpB3 + k];
    return argmin3(o);
}
#endif

}  // namespace alb
