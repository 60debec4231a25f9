// Device-side CSR ingest: validation, row sort, transpose, symmetry test and
// the undirected merge of the reference's driver.
//
// Reference counterparts: the transpose before a directed BFS
// (bfs/src/main.c:117-126 with convert_csr_to_csc, bfs/src/sparse_matrix.c:
// 230-290: counting sort by column, so every column lists its rows in
// ascending order) and the undirected graph built for a non-symmetric input
// (bfs/src/main.c:130-163): row i of the result is MergeArr(column i of A,
// row i of A) (bfs/src/utils.c:351-379). The reference runs both serially on
// the host; here the CSR is copied to the device as given and everything
// O(nnz) runs there:
//
//  * csr_check: row offsets start at 0, never decrease and end at nnz; every
//    column lies in [0, n); whether every row is ascending. One pass over the
//    offsets (thread per row) and one over the columns (thread per entry; an
//    entry smaller than its predecessor is a violation unless it starts a
//    row, found by binary search over the offsets).
//  * sort_rows: every row sorted ascending in place. Rows are classed by
//    length: up to 32 entries one warp (bitonic network over shuffles), up to
//    4096 one CTA (bitonic network in shared memory), longer ones one CTA
//    each with a stable LSD radix sort over global memory (4-bit digits,
//    per-tile (digit, thread) counts so equal digits keep their order).
//  * transpose: column counts (atomics), exclusive scan, scatter by atomic
//    cursor (one warp per row), then sort_rows on the result: each column's
//    rows come out ascending, as the reference's counting transpose leaves
//    them (duplicates included).
//  * csr_equal: A == A^T, entry for entry, after both are sorted.
//  * merge_undirected: MergeArr per row (one thread per row, count pass,
//    scan, write pass), bit for bit the reference's result including its
//    treatment of rows that are not sorted.
#include <cstring>

#include "graph.h"
#include "ingest.h"
#include "scan.cuh"

namespace alb {
namespace {

constexpr int kSortSmall = 32;
constexpr int kSortMedium = 4096;
constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 16;
constexpr int kRadixTile = kRadixThreads * kRadixItems;

enum CheckBits : int {
    kBadOffsets = 1,
    kBadColumn = 2,
    kUnsorted = 4,
};

unsigned grid_for(int64_t work, int block, int64_t cap = 152 * 32) {
    int64_t g = (work + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

// Counters of the CSR check, one device word each.
struct CheckWords {
    int flags;
    int pad;
    unsigned long long descents;      // entries e > 0 with col[e - 1] > col[e]
    unsigned long long start_desc;    // ... of them at the first entry of a row
};

// Offsets: rp[0] == 0, rp[n] == nnz, never decreasing. With check_order,
// also counts the descents at row starts: every non-empty row r with
// rp[r] > 0 compares its first entry with the entry before it (the bounds
// are tested locally, so the loads stay inside col even when some other
// offset is bad).
__global__ void k_check_offsets(int64_t n, const int64_t *rp, const int32_t *col, int64_t nnz,
                                int check_order, CheckWords *cw) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    int bad = 0;
    unsigned cnt = 0;
    if (tid == 0 && (rp[0] != 0 || rp[n] != nnz)) bad = 1;
    for (int64_t r = tid; r < n; r += nth) {
        const int64_t a = rp[r], b = rp[r + 1];
        if (b < a) bad = 1;
        if (check_order && a > 0 && a < b && b <= nnz && col[a - 1] > col[a]) cnt++;
    }
    if (__any_sync(kFull, bad) && (threadIdx.x & 31) == 0) atomicOr(&cw->flags, kBadOffsets);
    cnt = __reduce_add_sync(kFull, cnt);
    if (cnt && (threadIdx.x & 31) == 0) atomicAdd(&cw->start_desc, (unsigned long long)cnt);
}

// Columns: inside [0, n); with check_order, the number of descents (entry
// smaller than the one before it). Rows are sorted exactly when every
// descent sits at a row start, i.e. when this count equals k_check_offsets'.
// Four entries per thread and step (one 16-byte load; the entry before them
// is the previous thread's, read through L1).
__global__ void k_check_columns(int64_t n, const int32_t *col, int64_t nnz, int check_order,
                                CheckWords *cw) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const int64_t ng = nnz >> 2;
    const int4 *c4 = reinterpret_cast<const int4 *>(col);
    int bits = 0;
    unsigned cnt = 0;
    for (int64_t i = tid; i <= ng; i += nth) {
        int32_t c[4];
        int m = 4;
        if (i < ng) {
            const int4 v = c4[i];
            c[0] = v.x, c[1] = v.y, c[2] = v.z, c[3] = v.w;
        } else {  // the last nnz % 4 entries
            m = (int)(nnz & 3);
            for (int k = 0; k < m; k++) c[k] = col[4 * i + k];
        }
        int32_t prev = i > 0 && m > 0 ? __ldg(col + 4 * i - 1) : INT32_MIN;
        for (int k = 0; k < m; k++) {
            if (c[k] < 0 || c[k] >= n) bits |= kBadColumn;
            if (prev > c[k]) cnt++;
            prev = c[k];
        }
    }
    bits = __reduce_or_sync(kFull, bits);
    if (bits && (threadIdx.x & 31) == 0) atomicOr(&cw->flags, bits);
    if (check_order) {
        cnt = __reduce_add_sync(kFull, cnt);
        if (cnt && (threadIdx.x & 31) == 0) atomicAdd(&cw->descents, (unsigned long long)cnt);
    }
}

// ------------------------------------------------------------- row sort

__global__ void k_classify_rows(int64_t n, const int64_t *rp, int32_t *small, int32_t *medium,
                                int32_t *large, unsigned long long *counts) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = tid; r < n; r += nth) {
        const int64_t len = rp[r + 1] - rp[r];
        if (len <= 1) continue;
        if (len <= kSortSmall) small[atomicAdd(&counts[0], 1ull)] = (int32_t)r;
        else if (len <= kSortMedium) medium[atomicAdd(&counts[1], 1ull)] = (int32_t)r;
        else large[atomicAdd(&counts[2], 1ull)] = (int32_t)r;
    }
}

// One warp per row of 2..32 entries: a bitonic sorting network over the
// lanes, padded with INT32_MAX.
__global__ void k_sort_small(int64_t count, const int32_t *rows, const int64_t *rp, int32_t *col) {
    const int lane = threadIdx.x & 31;
    const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w; i < count; i += nw) {
        const int32_t r = rows[i];
        const int64_t st = rp[r];
        const int len = (int)(rp[r + 1] - st);
        int32_t v = lane < len ? col[st + lane] : INT32_MAX;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                const int32_t o = __shfl_xor_sync(kFull, v, j);
                const bool up = (lane & k) == 0;
                const bool lower = (lane & j) == 0;
                v = (lower == up) ? min(v, o) : max(v, o);
            }
        }
        if (lane < len) col[st + lane] = v;
    }
}

// One CTA per row of 33..4096 entries: bitonic network in shared memory over
// the next power of two, padded with INT32_MAX.
__global__ void __launch_bounds__(256) k_sort_medium(const int32_t *rows, const int64_t *rp,
                                                     int32_t *col) {
    __shared__ int32_t s[kSortMedium];
    const int32_t r = rows[blockIdx.x];
    const int64_t st = rp[r];
    const int len = (int)(rp[r + 1] - st);
    int P = 64;
    while (P < len) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < len ? col[st + i] : INT32_MAX;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool up = (i & k) == 0;
                    const int32_t a = s[i], b = s[ixj];
                    if ((a > b) == up) {
                        s[i] = b;
                        s[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < len; i += blockDim.x) col[st + i] = s[i];
}

// One CTA per row of more than 4096 entries: stable LSD radix sort with
// 4-bit digits between the row's range of col and the same range of tmp.
// Per pass: digit histogram of the whole row, then tiles of 4096 entries in
// order; thread t holds 16 consecutive entries of a tile, the (digit, thread)
// counts are scanned digit-major, so an entry's destination is its digit's
// running base + the entries of that digit held by lower threads of the tile
// + those before it in its own thread: equal digits keep their order.
__global__ void __launch_bounds__(kRadixThreads) k_sort_large(const int32_t *rows,
                                                               const int64_t *rp, int32_t *col,
                                                               int32_t *tmp, int bits) {
    __shared__ int32_t cnt[16 * kRadixThreads];
    __shared__ int64_t base[16];
    __shared__ int32_t hist[16];
    __shared__ int32_t dstart[17];
    const int t = threadIdx.x;
    const int32_t r = rows[blockIdx.x];
    const int64_t st = rp[r];
    const int64_t len = rp[r + 1] - st;
    int32_t *src = col + st, *dst = tmp + st;
    const int passes = (bits + 3) / 4;
    for (int pass = 0; pass < passes; pass++) {
        const int sh = 4 * pass;
        if (t < 16) hist[t] = 0;
        __syncthreads();
        for (int64_t i = t; i < len; i += kRadixThreads) atomicAdd(&hist[(src[i] >> sh) & 15], 1);
        __syncthreads();
        if (t == 0) {
            int64_t s = 0;
            for (int d = 0; d < 16; d++) {
                base[d] = s;
                s += hist[d];
            }
        }
        __syncthreads();
        for (int64_t t0 = 0; t0 < len; t0 += kRadixTile) {
            int32_t v[kRadixItems];
            int lc[16];
#pragma unroll
            for (int d = 0; d < 16; d++) lc[d] = 0;
#pragma unroll
            for (int k = 0; k < kRadixItems; k++) {
                const int64_t idx = t0 + (int64_t)t * kRadixItems + k;
                v[k] = idx < len ? src[idx] : -1;
                if (v[k] >= 0) lc[(v[k] >> sh) & 15]++;
            }
#pragma unroll
            for (int d = 0; d < 16; d++) cnt[d * kRadixThreads + t] = lc[d];
            __syncthreads();
            // exclusive scan of the 4096 counts, digit-major: thread t owns
            // entries [16t, 16t + 16)
            int32_t e[16];
            int64_t sum = 0;
#pragma unroll
            for (int k = 0; k < 16; k++) {
                e[k] = cnt[t * 16 + k];
                sum += e[k];
            }
            __shared__ int64_t tot;
            int64_t run = block_exclusive_scan<int64_t>(sum, &tot);
            // entry 256 d is the first count of digit d: owned by thread 16 d
            if ((t & 15) == 0) dstart[t >> 4] = (int32_t)run;
            if (t == 0) dstart[16] = (int32_t)tot;
#pragma unroll
            for (int k = 0; k < 16; k++) {
                const int32_t x = e[k];
                cnt[t * 16 + k] = (int32_t)run;
                run += x;
            }
            __syncthreads();
            int pos[16];
#pragma unroll
            for (int d = 0; d < 16; d++) pos[d] = cnt[d * kRadixThreads + t] - dstart[d];
#pragma unroll
            for (int k = 0; k < kRadixItems; k++) {
                if (v[k] < 0) continue;
                const int d = (v[k] >> sh) & 15;
                dst[base[d] + pos[d]] = v[k];
                pos[d]++;
            }
            __syncthreads();
            if (t < 16) base[t] += dstart[t + 1] - dstart[t];
            __syncthreads();
        }
        int32_t *x = src;
        src = dst;
        dst = x;
        __syncthreads();
    }
    if (passes & 1)  // the sorted row is in tmp
        for (int64_t i = t; i < len; i += kRadixThreads) col[st + i] = src[i];
}

// --------------------------------------------------------------- transpose

__global__ void k_count_columns(const int32_t *col, int64_t nnz, int32_t *cnt) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = tid; e < nnz; e += nth) atomicAdd(&cnt[col[e]], 1);
}

// One warp per row: entry (r, c) goes to a free slot of column c.
__global__ void k_scatter_transpose(int64_t n, const int64_t *rp, const int32_t *col,
                                    const int64_t *trp, int32_t *cur, int32_t *tcol) {
    const int lane = threadIdx.x & 31;
    const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = w; r < n; r += nw)
        for (int64_t e = rp[r] + lane; e < rp[r + 1]; e += 32) {
            const int32_t c = col[e];
            tcol[trp[c] + atomicAdd(&cur[c], 1)] = (int32_t)r;
        }
}

__global__ void k_equal(int64_t count, const int32_t *a, const int32_t *b, int *flag) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    int diff = 0;
    for (int64_t i = tid; i < count; i += nth) diff |= (a[i] != b[i]);
    if (__any_sync(kFull, diff) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

__global__ void k_equal64(int64_t count, const int64_t *a, const int64_t *b, int *flag) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    int diff = 0;
    for (int64_t i = tid; i < count; i += nth) diff |= (a[i] != b[i]);
    if (__any_sync(kFull, diff) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// ------------------------------------------------------- undirected merge

// MergeArr (bfs/src/utils.c:351-379) of a = column i of A (ascending) and
// b = row i of A (as given): count pass (out == nullptr) or write pass.
__device__ int64_t merge_row(const int32_t *a, int64_t al, const int32_t *b, int64_t bl,
                             int32_t *out) {
    int64_t x = 0, y = 0, k = 0;
    while (x < al && y < bl) {
        const int32_t u = a[x], w = b[y];
        int32_t o;
        if (u < w) {
            o = u;
            x++;
        } else if (u == w) {
            o = w;
            x++;
            y++;
        } else {
            o = w;
            y++;
        }
        if (out) out[k] = o;
        k++;
    }
    if (out) {
        for (; x < al; x++) out[k++] = a[x];
        for (; y < bl; y++) out[k++] = b[y];
    } else {
        k += (al - x) + (bl - y);
    }
    return k;
}

__global__ void k_merge_count(int64_t n, const int64_t *rp, const int32_t *col,
                              const int64_t *trp, const int32_t *tcol, int64_t *len) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < n; i += nth)
        len[i] = merge_row(tcol + trp[i], trp[i + 1] - trp[i], col + rp[i], rp[i + 1] - rp[i],
                           nullptr);
}

__global__ void k_merge_write(int64_t n, const int64_t *rp, const int32_t *col,
                              const int64_t *trp, const int32_t *tcol, const int64_t *urp,
                              int32_t *ucol) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < n; i += nth)
        merge_row(tcol + trp[i], trp[i + 1] - trp[i], col + rp[i], rp[i + 1] - rp[i],
                  ucol + urp[i]);
}

int key_bits(int64_t n) {
    int b = 1;
    while (b < 31 && (int64_t(1) << b) < n) b++;
    return b;
}

}  // namespace

alb_status csr_check(int64_t n, const int64_t *d_rp, const int32_t *d_col, int64_t nnz,
                     cudaStream_t st, bool *sorted) {
    CheckWords *d_cw = nullptr;
    ALB_TRY(dmalloc((void **)&d_cw, sizeof(CheckWords), "ingest flags"));
    CheckWords h{};
    const int order = sorted ? 1 : 0;
    cudaError_t e = cudaMemsetAsync(d_cw, 0, sizeof(CheckWords), st);
    if (e == cudaSuccess) {
        k_check_offsets<<<grid_for(n, 256), 256, 0, st>>>(n, d_rp, d_col, nnz, order, d_cw);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && nnz > 0) {
        k_check_columns<<<grid_for((nnz + 3) / 4, 256), 256, 0, st>>>(n, d_col, nnz, order, d_cw);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_cw, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dfree(d_cw);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ALB_ERR_CUDA, "CSR check: %s", cudaGetErrorString(e));
    }
    if (h.flags & kBadOffsets)
        return fail(ALB_ERR_INVALID, "row offsets must start at 0, never decrease and end at nnz");
    if (h.flags & kBadColumn) return fail(ALB_ERR_INVALID, "column index outside [0, n)");
    if (sorted) *sorted = h.descents == h.start_desc;
    return ALB_OK;
}

alb_status sort_rows(int64_t n, const int64_t *d_rp, int32_t *d_col, int64_t nnz,
                     cudaStream_t st) {
    if (nnz == 0) return ALB_OK;
    int32_t *lists = nullptr;
    unsigned long long *d_cnt = nullptr;
    ALB_TRY(dmalloc((void **)&lists, sizeof(int32_t) * (size_t)n * 3, "row sort lists"));
    alb_status s = dmalloc((void **)&d_cnt, sizeof(unsigned long long) * 3, "row sort counts");
    if (s != ALB_OK) {
        dfree(lists);
        return s;
    }
    int32_t *small = lists, *medium = lists + n, *large = lists + 2 * n;
    unsigned long long h[3] = {0, 0, 0};
    int32_t *tmp = nullptr;
    cudaError_t e = cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long) * 3, st);
    if (e == cudaSuccess) {
        k_classify_rows<<<grid_for(n, 256), 256, 0, st>>>(n, d_rp, small, medium, large, d_cnt);
        e = cudaMemcpyAsync(h, d_cnt, sizeof(h), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && h[0])
        k_sort_small<<<grid_for((int64_t)h[0] * 32, 256), 256, 0, st>>>((int64_t)h[0], small, d_rp,
                                                                          d_col);
    if (e == cudaSuccess && h[1]) k_sort_medium<<<(unsigned)h[1], 256, 0, st>>>(medium, d_rp, d_col);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess && h[2]) {
        s = dmalloc((void **)&tmp, sizeof(int32_t) * (size_t)nnz, "row sort buffer");
        if (s == ALB_OK)
            k_sort_large<<<(unsigned)h[2], kRadixThreads, 0, st>>>(large, d_rp, d_col, tmp,
                                                                  key_bits(n));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dfree(tmp);
    dfree(d_cnt);
    dfree(lists);
    if (s != ALB_OK) return s;
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ALB_ERR_CUDA, "row sort: %s", cudaGetErrorString(e));
    }
    return ALB_OK;
}

alb_status transpose(int64_t n, const int64_t *d_rp, const int32_t *d_col, int64_t nnz,
                     int64_t **d_trp, int32_t **d_tcol, cudaStream_t st) {
    *d_trp = nullptr;
    *d_tcol = nullptr;
    int32_t *cnt = nullptr;
    ALB_TRY(dmalloc((void **)&cnt, sizeof(int32_t) * (size_t)n, "transpose counts"));
    alb_status s = dmalloc((void **)d_trp, sizeof(int64_t) * (size_t)(n + 1), "transpose offsets");
    if (s == ALB_OK) s = dmalloc((void **)d_tcol, sizeof(int32_t) * (size_t)nnz, "transpose columns");
    cudaError_t e = cudaSuccess;
    if (s == ALB_OK) {
        e = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t)n, st);
        if (e == cudaSuccess && nnz > 0)
            k_count_columns<<<grid_for(nnz, 256), 256, 0, st>>>(d_col, nnz, cnt);
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (s == ALB_OK && e == cudaSuccess) s = exclusive_scan(cnt, *d_trp, n, st);
    if (s == ALB_OK && e == cudaSuccess) {
        e = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t)n, st);
        if (e == cudaSuccess && nnz > 0)
            k_scatter_transpose<<<grid_for(n * 32, 256), 256, 0, st>>>(n, d_rp, d_col, *d_trp, cnt,
                                                                       *d_tcol);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    dfree(cnt);
    if (s == ALB_OK && e != cudaSuccess) {
        cudaGetLastError();
        s = fail(ALB_ERR_CUDA, "transpose: %s", cudaGetErrorString(e));
    }
    if (s == ALB_OK) s = sort_rows(n, *d_trp, *d_tcol, nnz, st);
    if (s != ALB_OK) {
        dfree(*d_trp);
        dfree(*d_tcol);
        *d_trp = nullptr;
        *d_tcol = nullptr;
    }
    return s;
}

alb_status csr_equal(int64_t n, const int64_t *rp_a, const int32_t *col_a, const int64_t *rp_b,
                     const int32_t *col_b, int64_t nnz, cudaStream_t st, bool *equal) {
    int *d_flag = nullptr;
    ALB_TRY(dmalloc((void **)&d_flag, sizeof(int), "equality flag"));
    int h = 0;
    cudaError_t e = cudaMemsetAsync(d_flag, 0, sizeof(int), st);
    if (e == cudaSuccess) {
        k_equal64<<<grid_for(n + 1, 256), 256, 0, st>>>(n + 1, rp_a, rp_b, d_flag);
        if (nnz > 0) k_equal<<<grid_for(nnz, 256), 256, 0, st>>>(nnz, col_a, col_b, d_flag);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dfree(d_flag);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ALB_ERR_CUDA, "CSR compare: %s", cudaGetErrorString(e));
    }
    *equal = h == 0;
    return ALB_OK;
}

alb_status merge_undirected(int64_t n, const int64_t *d_rp, const int32_t *d_col, int64_t nnz,
                            int64_t **d_urp, int32_t **d_ucol, int64_t *unnz, cudaStream_t st) {
    *d_urp = nullptr;
    *d_ucol = nullptr;
    int64_t *trp = nullptr, *len = nullptr;
    int32_t *tcol = nullptr;
    ALB_TRY(transpose(n, d_rp, d_col, nnz, &trp, &tcol, st));
    alb_status s = dmalloc((void **)&len, sizeof(int64_t) * (size_t)n, "merge lengths");
    if (s == ALB_OK) s = dmalloc((void **)d_urp, sizeof(int64_t) * (size_t)(n + 1), "merged offsets");
    cudaError_t e = cudaSuccess;
    if (s == ALB_OK) {
        k_merge_count<<<grid_for(n, 256), 256, 0, st>>>(n, d_rp, d_col, trp, tcol, len);
        e = cudaGetLastError();
    }
    if (s == ALB_OK && e == cudaSuccess) s = exclusive_scan(len, *d_urp, n, st);
    int64_t total = 0;
    if (s == ALB_OK && e == cudaSuccess) {
        e = cudaMemcpyAsync(&total, *d_urp + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (s == ALB_OK && e == cudaSuccess)
        s = dmalloc((void **)d_ucol, sizeof(int32_t) * (size_t)(total > 0 ? total : 1),
                    "merged columns");
    if (s == ALB_OK && e == cudaSuccess) {
        k_merge_write<<<grid_for(n, 256), 256, 0, st>>>(n, d_rp, d_col, trp, tcol, *d_urp, *d_ucol);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    dfree(len);
    dfree(trp);
    dfree(tcol);
    if (s == ALB_OK && e != cudaSuccess) {
        cudaGetLastError();
        s = fail(ALB_ERR_CUDA, "undirected merge: %s", cudaGetErrorString(e));
    }
    if (s != ALB_OK) {
        dfree(*d_urp);
        dfree(*d_ucol);
        *d_urp = nullptr;
        *d_ucol = nullptr;
        return s;
    }
    *unnz = total;
    return ALB_OK;
}

}  // namespace alb
