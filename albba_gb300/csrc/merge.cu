// Sparse-frontier expansion with a sorted, duplicate-free result: the
// reference's push-merge kernel csc_spmspv_merge (bfs/src/bfs_par_kernels.c:
// 350-416, with merge_kernel :287-348 and the task merge merge_arr,
// bfs/src/bfs_SELLCSv2.c:530-575). There, each task copies the unvisited rows
// of its first frontier column and merges every further column into that
// list (two-pointer merge of ascending lists, equal entries kept once,
// entries of the new column kept only when unvisited), and the tasks' lists
// are merged again: the next frontier as the ascending list of the distinct
// unvisited out-neighbours of the frontier.
//
// GB300 form: the same set is the set bits of a bitmap, and an ordered
// compaction of a bitmap is ascending and duplicate-free by construction, so
// no merge or sort is needed: one warp per frontier vertex marks its
// unvisited out-neighbours with atomicOr (reading the word first, so a target
// hit by many pushes costs one atomic), the per-word bit counts are scanned,
// and one pass over the bitmap writes every word's set bits at its scanned
// offset: the list comes out in id order.
#include <cstring>

#include "graph.h"
#include "scan.cuh"

namespace alb {
namespace {

__global__ void k_merge_mark(const int32_t *x, int64_t nx, const int64_t *rp, const int32_t *col,
                             int64_t n, const uint32_t *visited, uint32_t *mark, int *err) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < nx; i += nw) {
        const int32_t u = x[i];
        if (u < 0 || u >= n) {  // a frontier id outside the graph
            if (lane == 0) atomicExch(err, 1);
            continue;
        }
        for (int64_t e = rp[u] + lane; e < rp[u + 1]; e += 32) {
            const int32_t v = col[e];
            const uint32_t bit = 1u << (v & 31);
            if (__ldg(visited + (v >> 5)) & bit) continue;
            if (!(__ldcg(mark + (v >> 5)) & bit)) atomicOr(mark + (v >> 5), bit);
        }
    }
}

__global__ void k_merge_count(const uint32_t *mark, int64_t nwords, int32_t *cnt) {
    const int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (w < nwords) cnt[w] = __popc(mark[w]);
}

__global__ void k_merge_write(const uint32_t *mark, int64_t nwords, const int64_t *off,
                              int32_t *y) {
    const int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    uint32_t m = mark[w];
    int64_t pos = off[w];
    while (m) {
        const int b = __ffs(m) - 1;
        m &= m - 1;
        y[pos++] = (int32_t)(w * 32 + b);
    }
}

unsigned blocks(int64_t work, int block) {
    const int64_t g = (work + block - 1) / block;
    return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace
}  // namespace alb

using namespace alb;

extern "C" alb_status alb_spmspv_merge(alb_graph *g, const int32_t *x, int64_t nx,
                                       const uint32_t *visited, int32_t *y, int64_t *ny) {
    if (!g || (nx > 0 && !x) || !visited || !ny)
        return fail(ALB_ERR_INVALID, "alb_spmspv_merge: bad arguments");
    if (nx < 0 || nx > g->n) return fail(ALB_ERR_INVALID, "alb_spmspv_merge: frontier size %lld",
                                          (long long)nx);
    ALB_CK(cudaSetDevice(g->device));
    const int64_t n = g->n, nwords = (n + 31) / 32;
    cudaStream_t st = g->stream;
    int32_t *dx = nullptr, *cnt = nullptr, *dy = nullptr;
    uint32_t *dvis = nullptr, *mark = nullptr;
    int64_t *off = nullptr;
    int *derr = nullptr;
    auto cleanup = [&]() {
        dfree(dx);
        dfree(cnt);
        dfree(dy);
        dfree(dvis);
        dfree(mark);
        dfree(off);
        dfree(derr);
    };
    alb_status rc = [&]() -> alb_status {
        ALB_TRY(dmalloc((void **)&dx, sizeof(int32_t) * (size_t)(nx > 0 ? nx : 1), "merge frontier"));
        ALB_TRY(dmalloc((void **)&dvis, sizeof(uint32_t) * (size_t)nwords, "merge visited"));
        ALB_TRY(dmalloc((void **)&mark, sizeof(uint32_t) * (size_t)nwords, "merge bitmap"));
        ALB_TRY(dmalloc((void **)&cnt, sizeof(int32_t) * (size_t)nwords, "merge counts"));
        ALB_TRY(dmalloc((void **)&off, sizeof(int64_t) * (size_t)(nwords + 1), "merge offsets"));
        ALB_TRY(dmalloc((void **)&derr, sizeof(int), "merge error"));
        if (nx > 0)
            ALB_CK(cudaMemcpyAsync(dx, x, sizeof(int32_t) * (size_t)nx, cudaMemcpyHostToDevice, st));
        ALB_CK(cudaMemcpyAsync(dvis, visited, sizeof(uint32_t) * (size_t)nwords,
                               cudaMemcpyHostToDevice, st));
        ALB_CK(cudaMemsetAsync(mark, 0, sizeof(uint32_t) * (size_t)nwords, st));
        ALB_CK(cudaMemsetAsync(derr, 0, sizeof(int), st));
        if (nx > 0)
            k_merge_mark<<<blocks(nx * 32, 256), 256, 0, st>>>(dx, nx, g->rp_out, g->col_out, n,
                                                               dvis, mark, derr);
        k_merge_count<<<blocks(nwords, 256), 256, 0, st>>>(mark, nwords, cnt);
        ALB_CK(cudaGetLastError());
        ALB_TRY(exclusive_scan(cnt, off, nwords, st));
        int64_t total = 0;
        int herr = 0;
        ALB_CK(cudaMemcpyAsync(&total, off + nwords, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        ALB_CK(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
        ALB_CK(cudaStreamSynchronize(st));
        if (herr) return fail(ALB_ERR_INVALID, "alb_spmspv_merge: frontier id outside [0, n)");
        *ny = total;
        if (y && total > 0) {
            ALB_TRY(dmalloc((void **)&dy, sizeof(int32_t) * (size_t)total, "merge result"));
            k_merge_write<<<blocks(nwords, 256), 256, 0, st>>>(mark, nwords, off, dy);
            ALB_CK(cudaGetLastError());
            ALB_CK(cudaMemcpyAsync(y, dy, sizeof(int32_t) * (size_t)total, cudaMemcpyDeviceToHost,
                                   st));
            ALB_CK(cudaStreamSynchronize(st));
        }
        return ALB_OK;
    }();
    cleanup();
    return rc;
}
