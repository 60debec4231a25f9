// Device exclusive scan into int64 (reduce-then-scan, three launches).
// out[i] = sum of in[0..i), out[count] = total; out may not alias in.
#pragma once

#include "graph.h"

namespace alb {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int64_t kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *total) {
    __shared__ int64_t ws[kScanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t inc = warp_inclusive_scan(v);
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        int64_t x = lane < kScanThreads / 32 ? ws[lane] : 0;
        int64_t xi = warp_inclusive_scan(x);
        if (lane < kScanThreads / 32) ws[lane] = xi - x;
        if (lane == kScanThreads / 32 - 1) *total = xi;
    }
    __syncthreads();
    int64_t r = ws[w] + inc - v;
    __syncthreads();
    return r;
}

template <class Tin>
__global__ void k_scan_tile_sums(const Tin *in, int64_t count, int64_t *bsum) {
    const int64_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++)
        if (base + i < count) s += (int64_t)in[base + i];
    __shared__ int64_t tot;
    block_exclusive_scan<int64_t>(s, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

static __global__ void k_scan_tile_offsets(int64_t *bsum, int64_t ntiles, int64_t *grand_total) {
    __shared__ int64_t tot;
    int64_t carry = 0;
    for (int64_t b = 0; b < ntiles; b += kScanThreads) {
        int64_t i = b + threadIdx.x;
        int64_t v = i < ntiles ? bsum[i] : 0;
        int64_t ex = block_exclusive_scan<int64_t>(v, &tot);
        if (i < ntiles) bsum[i] = carry + ex;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) *grand_total = carry;
}

template <class Tin>
__global__ void k_scan_tiles(const Tin *in, int64_t count, const int64_t *boff, int64_t *out) {
    const int64_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        v[i] = (base + i < count) ? (int64_t)in[base + i] : 0;
        s += v[i];
    }
    __shared__ int64_t tot;
    int64_t run = boff[blockIdx.x] + block_exclusive_scan<int64_t>(s, &tot);
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < count) out[base + i] = run;
        run += v[i];
    }
}

template <class Tin>
alb_status exclusive_scan(const Tin *in, int64_t *out, int64_t count, cudaStream_t st) {
    const int64_t ntiles = (count + kScanTile - 1) / kScanTile;
    if (ntiles == 0) {
        ALB_CK(cudaMemsetAsync(out, 0, sizeof(int64_t), st));
        ALB_CK(cudaStreamSynchronize(st));
        return ALB_OK;
    }
    int64_t *bsum = nullptr;
    ALB_TRY(dmalloc((void **)&bsum, sizeof(int64_t) * ntiles, "scan tile sums"));
    k_scan_tile_sums<Tin><<<(unsigned)ntiles, kScanThreads, 0, st>>>(in, count, bsum);
    k_scan_tile_offsets<<<1, kScanThreads, 0, st>>>(bsum, ntiles, out + count);
    k_scan_tiles<Tin><<<(unsigned)ntiles, kScanThreads, 0, st>>>(in, count, bsum, out);
    cudaError_t e = cudaGetLastError();
    // the temporary must outlive the kernels that use it
    cudaError_t e2 = cudaStreamSynchronize(st);
    dfree(bsum);
    if (e != cudaSuccess || e2 != cudaSuccess)
        return fail(ALB_ERR_CUDA, "exclusive_scan: %s",
                    cudaGetErrorString(e != cudaSuccess ? e : e2));
    return ALB_OK;
}

}  // namespace alb
