// Training of the direction-selector MLP on the GPU: forward, backward and
// Adam, hand-written. No counterpart in the reference.
//
// Model: out = W3 relu(W2 relu(W1 x + b1) + b2) + b3, x in R^8, out in R^3
// (predicted cost of each traversal variant). Loss: mean over samples of
// sum_k mask[k] * (out[k] - y[k])^2. One warp per sample: lane j owns hidden
// unit j of both layers; per-sample gradients are summed in shared memory and
// flushed to global memory once per block.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "graph.h"
#include "selector.cuh"

namespace alb {
namespace {

constexpr int kTrainBlock = 256;

__global__ void k_mlp_forward(const float *P, const float *X, int32_t B, float *out) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t b = gw; b < B; b += nw) {
        const float *x = X + b * kMlpIn;
        float a = P[kMlpB1 + lane];
#pragma unroll
        for (int i = 0; i < kMlpIn; i++) a += P[kMlpW1 + lane * kMlpIn + i] * x[i];
        const float h1 = fmaxf(a, 0.f);
        float c = P[kMlpB2 + lane];
        for (int i = 0; i < kMlpH; i++) c += P[kMlpW2 + lane * kMlpH + i] * __shfl_sync(kFull, h1, i);
        const float h2 = fmaxf(c, 0.f);
#pragma unroll
        for (int k = 0; k < kMlpOut; k++) {
            const float o = warp_sum(P[kMlpW3 + k * kMlpH + lane] * h2) + P[kMlpB3 + k];
            if (lane == 0) out[b * kMlpOut + k] = o;
        }
    }
}

__global__ void k_mlp_grad(const float *P, const float *X, const float *Y, const float *M,
                           int32_t B, float inv_b, float *grad, float *loss) {
    __shared__ float sg[kMlpParams];
    __shared__ float sl;
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) sg[i] = 0.f;
    if (threadIdx.x == 0) sl = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t gw = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t b = gw; b < B; b += nw) {
        const float *x = X + b * kMlpIn;
        // forward
        float a1 = P[kMlpB1 + lane];
#pragma unroll
        for (int i = 0; i < kMlpIn; i++) a1 += P[kMlpW1 + lane * kMlpIn + i] * x[i];
        const float h1 = fmaxf(a1, 0.f);
        float a2 = P[kMlpB2 + lane];
        for (int i = 0; i < kMlpH; i++) a2 += P[kMlpW2 + lane * kMlpH + i] * __shfl_sync(kFull, h1, i);
        const float h2 = fmaxf(a2, 0.f);
        float d3[kMlpOut];
        float l = 0.f;
#pragma unroll
        for (int k = 0; k < kMlpOut; k++) {
            const float o = warp_sum(P[kMlpW3 + k * kMlpH + lane] * h2) + P[kMlpB3 + k];
            const float m = M[b * kMlpOut + k];
            const float diff = o - Y[b * kMlpOut + k];
            l += m * diff * diff;
            d3[k] = 2.f * m * diff * inv_b;
        }
        // backward
        float g2 = 0.f;
#pragma unroll
        for (int k = 0; k < kMlpOut; k++) {
            atomicAdd(&sg[kMlpW3 + k * kMlpH + lane], d3[k] * h2);
            g2 += P[kMlpW3 + k * kMlpH + lane] * d3[k];
        }
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < kMlpOut; k++) atomicAdd(&sg[kMlpB3 + k], d3[k]);
            atomicAdd(&sl, l);
        }
        const float d2 = h2 > 0.f ? g2 : 0.f;  // lane j: dL/d(a2_j)
        atomicAdd(&sg[kMlpB2 + lane], d2);
        for (int i = 0; i < kMlpH; i++)
            atomicAdd(&sg[kMlpW2 + lane * kMlpH + i], d2 * __shfl_sync(kFull, h1, i));
        // dL/d(h1_i) = sum_j W2[j][i] d2_j, lane i
        float g1 = 0.f;
        for (int jj = 0; jj < kMlpH; jj++) g1 += P[kMlpW2 + jj * kMlpH + lane] * __shfl_sync(kFull, d2, jj);
        const float d1 = h1 > 0.f ? g1 : 0.f;
        atomicAdd(&sg[kMlpB1 + lane], d1);
#pragma unroll
        for (int i = 0; i < kMlpIn; i++) atomicAdd(&sg[kMlpW1 + lane * kMlpIn + i], d1 * x[i]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x)
        if (sg[i] != 0.f) atomicAdd(&grad[i], sg[i]);
    if (threadIdx.x == 0 && sl != 0.f) atomicAdd(loss, sl * inv_b);
}

// Adam (Kingma & Ba 2015): m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2;
// p -= lr * (m / (1 - b1^t)) / (sqrt(v / (1 - b2^t)) + eps).
__global__ void k_adam(float *P, const float *G, float *Mm, float *Vv, float c1, float c2,
                       float lr, float b1, float b2, float eps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    const float g = G[i];
    const float m = b1 * Mm[i] + (1.f - b1) * g;
    const float v = b2 * Vv[i] + (1.f - b2) * g * g;
    Mm[i] = m;
    Vv[i] = v;
    P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { dfree(p); }
};

template <class T>
alb_status to_dev(DevBuf &b, const T *h, size_t n, const char *what) {
    ALB_TRY(dmalloc(&b.p, sizeof(T) * (n ? n : 1), what));
    if (h && n) ALB_CK(cudaMemcpy(b.p, h, sizeof(T) * n, cudaMemcpyHostToDevice));
    return ALB_OK;
}

unsigned grid_for_samples(int32_t B) {
    const int wpb = kTrainBlock / 32;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((B + wpb - 1) / wpb, 1024));
}

}  // namespace
}  // namespace alb

using namespace alb;

extern "C" {

alb_status alb_mlp_forward(const float *params, const float *x, int32_t batch, float *out) {
    if (!params || !x || !out || batch < 1) return fail(ALB_ERR_INVALID, "alb_mlp_forward: bad arguments");
    DevBuf dp, dx, dout;
    ALB_TRY(to_dev(dp, params, kMlpParams, "mlp params"));
    ALB_TRY(to_dev(dx, x, (size_t)batch * kMlpIn, "mlp inputs"));
    ALB_TRY(to_dev<float>(dout, nullptr, (size_t)batch * kMlpOut, "mlp outputs"));
    k_mlp_forward<<<grid_for_samples(batch), kTrainBlock>>>((float *)dp.p, (float *)dx.p, batch,
                                                            (float *)dout.p);
    ALB_CK(cudaGetLastError());
    ALB_CK(cudaMemcpy(out, dout.p, sizeof(float) * batch * kMlpOut, cudaMemcpyDeviceToHost));
    return ALB_OK;
}

alb_status alb_mlp_loss_grad(const float *params, const float *x, const float *y,
                             const float *mask, int32_t batch, float *grad, float *loss) {
    if (!params || !x || !y || !mask || !grad || batch < 1)
        return fail(ALB_ERR_INVALID, "alb_mlp_loss_grad: bad arguments");
    DevBuf dp, dx, dy, dm, dg, dl;
    ALB_TRY(to_dev(dp, params, kMlpParams, "mlp params"));
    ALB_TRY(to_dev(dx, x, (size_t)batch * kMlpIn, "mlp inputs"));
    ALB_TRY(to_dev(dy, y, (size_t)batch * kMlpOut, "mlp targets"));
    ALB_TRY(to_dev(dm, mask, (size_t)batch * kMlpOut, "mlp masks"));
    ALB_TRY(to_dev<float>(dg, nullptr, kMlpParams, "mlp grad"));
    ALB_TRY(to_dev<float>(dl, nullptr, 1, "mlp loss"));
    ALB_CK(cudaMemset(dg.p, 0, sizeof(float) * kMlpParams));
    ALB_CK(cudaMemset(dl.p, 0, sizeof(float)));
    k_mlp_grad<<<grid_for_samples(batch), kTrainBlock>>>((float *)dp.p, (float *)dx.p, (float *)dy.p,
                                                         (float *)dm.p, batch, 1.0f / batch,
                                                         (float *)dg.p, (float *)dl.p);
    ALB_CK(cudaGetLastError());
    ALB_CK(cudaMemcpy(grad, dg.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    float l = 0;
    ALB_CK(cudaMemcpy(&l, dl.p, sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) *loss = l;
    return ALB_OK;
}

alb_status alb_adam_step(float *params, const float *grad, float *m, float *v, int32_t t,
                         float lr, float beta1, float beta2, float eps) {
    if (!params || !grad || !m || !v || t < 1) return fail(ALB_ERR_INVALID, "alb_adam_step: bad arguments");
    DevBuf dp, dg, dm, dv;
    ALB_TRY(to_dev(dp, params, kMlpParams, "adam params"));
    ALB_TRY(to_dev(dg, grad, kMlpParams, "adam grad"));
    ALB_TRY(to_dev(dm, m, kMlpParams, "adam m"));
    ALB_TRY(to_dev(dv, v, kMlpParams, "adam v"));
    const float c1 = 1.f - std::pow(beta1, (float)t), c2 = 1.f - std::pow(beta2, (float)t);
    k_adam<<<(kMlpParams + 255) / 256, 256>>>((float *)dp.p, (float *)dg.p, (float *)dm.p,
                                              (float *)dv.p, c1, c2, lr, beta1, beta2, eps);
    ALB_CK(cudaGetLastError());
    ALB_CK(cudaMemcpy(params, dp.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    ALB_CK(cudaMemcpy(m, dm.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    ALB_CK(cudaMemcpy(v, dv.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    return ALB_OK;
}

alb_status alb_selector_train(const float *x, const float *y, const float *mask, int32_t batch,
                              int32_t steps, float lr, uint64_t seed, int32_t init,
                              float *params, float *loss_out) {
    if (!x || !y || !mask || !params || batch < 1 || steps < 0)
        return fail(ALB_ERR_INVALID, "alb_selector_train: bad arguments");
    std::vector<float> p0(params, params + kMlpParams);
    if (init) {
        // He initialisation, biases zero
        std::mt19937_64 rng(seed);
        auto fill = [&](int off, int rows, int cols) {
            std::normal_distribution<float> nd(0.f, std::sqrt(2.0f / cols));
            for (int i = 0; i < rows * cols; i++) p0[off + i] = nd(rng);
        };
        std::fill(p0.begin(), p0.end(), 0.f);
        fill(kMlpW1, kMlpH, kMlpIn);
        fill(kMlpW2, kMlpH, kMlpH);
        fill(kMlpW3, kMlpOut, kMlpH);
    }
    DevBuf dp, dx, dy, dm, dg, dl, dmm, dvv;
    ALB_TRY(to_dev(dp, p0.data(), kMlpParams, "train params"));
    ALB_TRY(to_dev(dx, x, (size_t)batch * kMlpIn, "train inputs"));
    ALB_TRY(to_dev(dy, y, (size_t)batch * kMlpOut, "train targets"));
    ALB_TRY(to_dev(dm, mask, (size_t)batch * kMlpOut, "train masks"));
    ALB_TRY(to_dev<float>(dg, nullptr, kMlpParams, "train grad"));
    ALB_TRY(to_dev<float>(dl, nullptr, 1, "train loss"));
    ALB_TRY(to_dev<float>(dmm, nullptr, kMlpParams, "adam m"));
    ALB_TRY(to_dev<float>(dvv, nullptr, kMlpParams, "adam v"));
    ALB_CK(cudaMemset(dmm.p, 0, sizeof(float) * kMlpParams));
    ALB_CK(cudaMemset(dvv.p, 0, sizeof(float) * kMlpParams));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int32_t t = 1; t <= steps; t++) {
        ALB_CK(cudaMemsetAsync(dg.p, 0, sizeof(float) * kMlpParams));
        ALB_CK(cudaMemsetAsync(dl.p, 0, sizeof(float)));
        k_mlp_grad<<<grid_for_samples(batch), kTrainBlock>>>(
            (float *)dp.p, (float *)dx.p, (float *)dy.p, (float *)dm.p, batch, 1.0f / batch,
            (float *)dg.p, (float *)dl.p);
        const float c1 = 1.f - std::pow(b1, (float)t), c2 = 1.f - std::pow(b2, (float)t);
        k_adam<<<(kMlpParams + 255) / 256, 256>>>((float *)dp.p, (float *)dg.p, (float *)dmm.p,
                                                  (float *)dvv.p, c1, c2, lr, b1, b2, eps);
    }
    ALB_CK(cudaGetLastError());
    ALB_CK(cudaDeviceSynchronize());
    ALB_CK(cudaMemcpy(params, dp.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    if (loss_out) {
        // loss of the final parameters
        ALB_CK(cudaMemset(dg.p, 0, sizeof(float) * kMlpParams));
        ALB_CK(cudaMemset(dl.p, 0, sizeof(float)));
        k_mlp_grad<<<grid_for_samples(batch), kTrainBlock>>>(
            (float *)dp.p, (float *)dx.p, (float *)dy.p, (float *)dm.p, batch, 1.0f / batch,
            (float *)dg.p, (float *)dl.p);
        ALB_CK(cudaGetLastError());
        ALB_CK(cudaMemcpy(loss_out, dl.p, sizeof(float), cudaMemcpyDeviceToHost));
    }
    return ALB_OK;
}

}  // extern "C"
