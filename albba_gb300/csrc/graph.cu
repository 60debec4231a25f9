// Graph upload and the device SELL-C-sigma builder.
//
// Reference counterparts: the CSR container and its int32 limits
// (bfs/src/sparse_matrix.h:18-29), the transpose done before the BFS
// (bfs/src/main.c:117-126, bfs/src/sparse_matrix.c:230-290), and the SELL
// pre-processing (bfs/src/bfs_SELLCSv2.c:34-59): row lengths
// (bfs/src/utils.c:111-124), stable descending sort inside sigma windows
// (bfs/src/sorting_utils.c:173-253), slice widths and the padded fill
// (bfs/src/sparse_matrix.c:435-521).
//
// GB300 layout, all in sorted-position space (position p holds original row
// perm[p]; neighbour ids are stored as positions):
//   slice s = rows [s*C, s*C+C); width[s] = longest row; w4 = width rounded
//   up to 4; col[slice_off[s] + (k/4)*4*C + r*4 + k%4] = k-th neighbour of
//   row s*C+r, padded with the row's own position. A warp reading group
//   k/4 of a C=32 slice issues one fully coalesced 512-byte int4 load.
//   Self-loops are dropped, so the padding value doubles as an end marker.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <vector>

#include "albba_gen.h"
#include "graph.h"
#include "ingest.h"
#include "scan.cuh"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace alb {

// Device buffers come from the device's default memory pool, which keeps
// freed memory (release threshold: unlimited) instead of returning it to the
// driver: the gigabytes of a graph's CSR, SELL and traversal state are
// reused by the next graph built in the process without new driver
// allocations, and a destroy does not wait on driver frees. A device without
// memory pools gets plain cudaMalloc / cudaFree.
namespace {
bool use_pool() {
    static std::mutex mu;
    static int state[256] = {};  // 0 unknown, 1 pool, 2 plain
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) {
        cudaGetLastError();
        return false;
    }
    std::lock_guard<std::mutex> lk(mu);
    if (state[dev] == 0) {
        int ok = 0;
        cudaMemPool_t pool;
        if (cudaDeviceGetAttribute(&ok, cudaDevAttrMemoryPoolsSupported, dev) == cudaSuccess && ok &&
            cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
            state[dev] = 1;
        } else {
            state[dev] = 2;
        }
        cudaGetLastError();
    }
    return state[dev] == 1;
}
}  // namespace

alb_status dmalloc(void **p, size_t bytes, const char *what) {
    *p = nullptr;
    if (injected_alloc_failure())
        return fail(ALB_ERR_OOM, "device allocation of %zu bytes for %s failed (injected)", bytes,
                    what);
    cudaError_t e;
    if (use_pool()) {
        // allocated in the legacy stream's order, then waited for, so that the
        // buffer can be used from any stream at once
        e = cudaMallocAsync(p, bytes ? bytes : 16, 0);
        if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    } else {
        e = cudaMalloc(p, bytes ? bytes : 16);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        if (e == cudaErrorMemoryAllocation)
            return fail(ALB_ERR_OOM, "device allocation of %zu bytes for %s failed", bytes, what);
        return fail(ALB_ERR_CUDA, "device allocation for %s: %s", what, cudaGetErrorString(e));
    }
    return ALB_OK;
}

void dfree(void *p) {
    if (!p) return;
    if (!use_pool()) {
        cudaFree(p);
        return;
    }
    // work on any stream may still use the buffer (cudaFree waited for the
    // device too); it then goes back to the pool
    cudaDeviceSynchronize();
    cudaFreeAsync(p, 0);
    cudaStreamSynchronize(0);
}

static double now_ms() {
    return std::chrono::duration<double, std::milli>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

PhaseLog::PhaseLog(const char *c) : call(c) {
    static const bool enabled = [] {
        const char *e = std::getenv("ALB_TRACE_PHASES");
        return e && *e && *e != '0';
    }();
    on = enabled;
    if (on) t = now_ms();
}

void PhaseLog::mark(const char *phase, cudaStream_t st) {
    if (!on) return;
    cudaStreamSynchronize(st);
    const double t1 = now_ms();
    std::fprintf(stderr, "alb phase %s/%s %.3f ms\n", call, phase, t1 - t);
    t = t1;
}

int resident_blocks(const void *func, int block) {
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, int> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find({func, block});
    if (it != cache.end()) return it->second;
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, func, block, 0) != cudaSuccess) {
        cudaGetLastError();
        per = 0;
    }
    cache[{func, block}] = per;
    return per;
}

namespace {

// ------------------------------------------------------------ ingest

alb_status upload(int64_t n, const int64_t *rp, const int32_t *col, int64_t **d_rp,
                  int32_t **d_col, cudaStream_t st) {
    ALB_TRY(dmalloc((void **)d_rp, sizeof(int64_t) * (size_t)(n + 1), "row offsets"));
    ALB_TRY(dmalloc((void **)d_col, sizeof(int32_t) * (size_t)rp[n], "columns"));
    ALB_CK(cudaMemcpyAsync(*d_rp, rp, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyHostToDevice, st));
    ALB_CK(cudaMemcpyAsync(*d_col, col, sizeof(int32_t) * (size_t)rp[n], cudaMemcpyHostToDevice, st));
    return ALB_OK;
}

void free_sell(Sell &s) {
    dfree(s.perm);
    dfree(s.inv);
    dfree(s.ideg);
    dfree(s.odeg);
    dfree(s.width);
    dfree(s.slice_off);
    dfree(s.col);
    dfree(s.prow);
    dfree(s.pcol);
    dfree(s.vinit);
    dfree(s.lrow);
    dfree(s.lptr);
    dfree(s.lcol);
    s = Sell();
}

alb_status graph_shell(int64_t n, alb_graph **out) {
    int dev = 0;
    ALB_CK(cudaGetDevice(&dev));
    alb_graph *g = new alb_graph();
    g->device = dev;
    g->n = n;
    cudaError_t e = cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking);
    g->stream = g->own_stream;
    if (e == cudaSuccess) e = cudaEventCreate(&g->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&g->ev1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        alb_graph_destroy(g);
        return fail(ALB_ERR_CUDA, "stream/event setup: %s", cudaGetErrorString(e));
    }
    *out = g;
    return ALB_OK;
}

// Takes a CSR already on the device (d_rp, d_col: dmalloc'ed, owned by g from
// here on) to the traversal's shape: checked, rows ascending, and both
// orientations (the transpose made on the device unless the caller declared
// the matrix symmetric; a transpose equal to the matrix is dropped).
alb_status finish_device_csr(alb_graph *g, int64_t *d_rp, int32_t *d_col, int64_t nnz,
                             uint32_t flags) {
    g->rp_in = g->rp_out = d_rp;
    g->col_in = g->col_out = d_col;
    g->nnz_in = g->nnz_out = nnz;
    bool sorted = true;
    // ALB_CSR_SORTED: the caller vouches for the order, only ranges are checked
    ALB_TRY(csr_check(g->n, d_rp, d_col, nnz, g->stream,
                      (flags & ALB_CSR_SORTED) ? nullptr : &sorted));
    if (!sorted) ALB_TRY(sort_rows(g->n, d_rp, d_col, nnz, g->stream));
    if (flags & ALB_CSR_SYMMETRIC) {
        g->symmetric = true;
        return ALB_OK;
    }
    int64_t *trp = nullptr;
    int32_t *tcol = nullptr;
    ALB_TRY(transpose(g->n, d_rp, d_col, nnz, &trp, &tcol, g->stream));
    bool same = false;
    alb_status s = csr_equal(g->n, d_rp, d_col, trp, tcol, nnz, g->stream, &same);
    if (s != ALB_OK || same) {
        dfree(trp);
        dfree(tcol);
        g->symmetric = same;
        return s;
    }
    if (flags & ALB_CSR_IN) {
        g->rp_out = trp;
        g->col_out = tcol;
    } else {
        g->rp_in = trp;
        g->col_in = tcol;
    }
    return ALB_OK;
}

alb_status create_impl(int64_t n, const int64_t *rowptr, const int32_t *col, uint32_t flags,
                       alb_graph **out) {
    if (rowptr[0] != 0 || rowptr[n] < 0)
        return fail(ALB_ERR_INVALID, "row offsets must start at 0 and end at nnz >= 0");
    PhaseLog ph("graph_create");
    alb_graph *g = nullptr;
    ALB_TRY(graph_shell(n, &g));
    ph.mark("setup", g->stream);
    int64_t *d_rp = nullptr;
    int32_t *d_col = nullptr;
    alb_status st = upload(n, rowptr, col, &d_rp, &d_col, g->stream);
    ph.mark("upload", g->stream);
    if (st == ALB_OK) {
        st = finish_device_csr(g, d_rp, d_col, rowptr[n], flags);
        ph.mark("check_sort_transpose", g->stream);
    } else {
        dfree(d_rp);
        dfree(d_col);
    }
    if (st == ALB_OK) {
        cudaError_t se = cudaStreamSynchronize(g->stream);
        if (se != cudaSuccess) st = fail(ALB_ERR_CUDA, "upload: %s", cudaGetErrorString(se));
    }
    if (st != ALB_OK) {
        alb_graph_destroy(g);
        return st;
    }
    *out = g;
    return ALB_OK;
}

// --------------------------------------------------------- device kernels

// Row lengths without self-loops, for both sides; optionally (sl_off != 0)
// each row's self-loop run: its offset in the row and its length. Grid-stride
// rows; the longest length is combined in the block and posted with one
// atomic only when it beats the current maximum.
__global__ void k_row_lengths(int64_t n, const int64_t *rp, const int32_t *col, int32_t *len,
                              int32_t *max_len, int32_t *sl_off = nullptr,
                              int32_t *sl_num = nullptr) {
    __shared__ int32_t s_max[32];
    int32_t l = 0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
         v += (int64_t)gridDim.x * blockDim.x) {
        // rows are sorted: the self-loops are one run, found by two binary
        // searches (a hub row costs log(deg), not deg); a row whose first
        // entry is above v or last below it has none
        const int64_t b = rp[v], e = rp[v + 1];
        int64_t lo = b, hi = e;
        if (b < e && (col[b] > (int32_t)v || col[e - 1] < (int32_t)v)) {
            lo = hi = col[b] > (int32_t)v ? b : e;
        } else {
            while (lo < hi) {  // first entry >= v
                const int64_t mid = (lo + hi) >> 1;
                if (col[mid] < (int32_t)v) lo = mid + 1;
                else hi = mid;
            }
        }
        int64_t lo2 = lo, hi2 = lo < e && col[lo] == (int32_t)v ? e : lo;
        while (lo2 < hi2) {  // first entry > v
            const int64_t mid = (lo2 + hi2) >> 1;
            if (col[mid] <= (int32_t)v) lo2 = mid + 1;
            else hi2 = mid;
        }
        const int32_t lv = (int32_t)((e - b) - (lo2 - lo));
        len[v] = lv;
        l = max(l, lv);
        if (sl_off) {
            sl_off[v] = (int32_t)(lo - b);
            sl_num[v] = (int32_t)(lo2 - lo);
        }
    }
    l = __reduce_max_sync(kFull, l);
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) l = max(l, s_max[k]);
        if (l > 0 && l > __ldcg(max_len)) atomicMax(max_len, l);
    }
}

// Stable descending sort of row lengths inside one sigma window per CTA:
// LSD radix sort with 4-bit digits (the digit size of
// bfs/src/sorting_utils.c:26-28), each pass a counting sort over
// (digit, thread) buckets so equal digits keep their order.
// Shared memory: key[sigma] int32, idx[2][sigma] uint16, cnt[16*TPB] int32.
__global__ void k_window_sort(int64_t n, int32_t sigma, int32_t items, const int32_t *len,
                              int32_t *perm) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tpb = blockDim.x, t = threadIdx.x;
    int32_t *key = (int32_t *)smem;
    int32_t *cnt = key + sigma;
    uint16_t *ia = (uint16_t *)(cnt + 16 * tpb);
    uint16_t *ib = ia + sigma;
    __shared__ int32_t s_max, s_wsum[32];
    const int64_t wbase = (int64_t)blockIdx.x * sigma;
    const int32_t wlen = (int32_t)min((int64_t)sigma, n - wbase);
    if (t == 0) s_max = 0;
    __syncthreads();
    int32_t lmax = 0;
    for (int32_t i = t; i < wlen; i += tpb) {
        int32_t k = len[wbase + i];
        key[i] = k;
        ia[i] = (uint16_t)i;
        lmax = max(lmax, k);
    }
    atomicMax(&s_max, lmax);
    __syncthreads();
    int32_t passes = 0;
    for (uint32_t m = (uint32_t)s_max; m; m >>= 4) passes++;
    const int32_t lo = t * items, hi = min(lo + items, wlen);
    for (int32_t pass = 0; pass < passes; pass++) {
        const int shift = 4 * pass;
        int32_t c[16];
#pragma unroll
        for (int b = 0; b < 16; b++) c[b] = 0;
        for (int32_t i = lo; i < hi; i++) {
            int d = 15 - ((key[ia[i]] >> shift) & 15);  // descending
#pragma unroll
            for (int b = 0; b < 16; b++) c[b] += (b == d);
        }
#pragma unroll
        for (int b = 0; b < 16; b++) cnt[b * tpb + t] = c[b];
        __syncthreads();
        // exclusive scan of cnt[0 .. 16*tpb): thread t owns entries [16t, 16t+16)
        int32_t run = 0;
#pragma unroll
        for (int j = 0; j < 16; j++) {
            int32_t v = cnt[16 * t + j];
            cnt[16 * t + j] = run;
            run += v;
        }
        int32_t inc = warp_inclusive_scan(run);
        if ((t & 31) == 31) s_wsum[t >> 5] = inc;
        __syncthreads();
        if (t < 32) {
            int32_t v = (t < (tpb >> 5)) ? s_wsum[t] : 0;
            int32_t vi = warp_inclusive_scan(v);
            if (t < (tpb >> 5)) s_wsum[t] = vi - v;
        }
        __syncthreads();
        const int32_t add = s_wsum[t >> 5] + inc - run;
#pragma unroll
        for (int j = 0; j < 16; j++) cnt[16 * t + j] += add;
        __syncthreads();
#pragma unroll
        for (int b = 0; b < 16; b++) c[b] = cnt[b * tpb + t];
        for (int32_t i = lo; i < hi; i++) {
            uint16_t id = ia[i];
            int d = 15 - ((key[id] >> shift) & 15);
            int32_t at = 0;
#pragma unroll
            for (int b = 0; b < 16; b++)
                if (b == d) at = c[b]++;
            ib[at] = id;
        }
        __syncthreads();
        uint16_t *tmp = ia;
        ia = ib;
        ib = tmp;
    }
    for (int32_t i = t; i < wlen; i += tpb) perm[wbase + i] = (int32_t)(wbase + ia[i]);
}

__global__ void k_identity(int64_t n, int32_t *perm) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p < n) perm[p] = (int32_t)p;
}

alb_status window_order_impl(int64_t n, int32_t sigma, const int32_t *d_len, int32_t *d_perm,
                             cudaStream_t st) {
    if (sigma <= 1) {
        k_identity<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, d_perm);
    } else {
        int tpb = std::min(1024, std::max(32, ((sigma / 16 + 31) / 32) * 32));
        int items = (sigma + tpb - 1) / tpb;
        size_t sm = sizeof(int32_t) * sigma + sizeof(int32_t) * 16 * tpb +
                    2 * sizeof(uint16_t) * sigma;
        ALB_CK(cudaFuncSetAttribute(k_window_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sm));
        unsigned nwin = (unsigned)((n + sigma - 1) / sigma);
        k_window_sort<<<nwin, tpb, sm, st>>>(n, sigma, items, d_len, d_perm);
    }
    ALB_CK(cudaGetLastError());
    return ALB_OK;
}

// inv, and per-position degrees; for the flat fill, each position's raw
// pull-row start and self-loop run.
__global__ void k_positions(int64_t n, const int32_t *perm, const int32_t *ilen,
                            const int32_t *olen, int32_t *inv, int32_t *ideg, int32_t *odeg,
                            const int64_t *rp, const int32_t *sl_off, const int32_t *sl_num,
                            int64_t *rstart, int2 *sl) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    int32_t v = perm[p];
    inv[v] = (int32_t)p;
    ideg[p] = ilen[v];
    odeg[p] = olen[v];
    rstart[p] = rp[v];
    sl[p] = make_int2(sl_off[v], sl_num[v]);
}

__device__ __forceinline__ bool is_long(int32_t d, int32_t long_row) {
    return long_row > 0 && d > long_row;
}

// width[s] and the padded slice size C * w4 (int64) for the scan.
__global__ void k_widths(int64_t n, int64_t nslices, int32_t C, int32_t long_row,
                         const int32_t *ideg, int32_t *width, int64_t *ssize) {
    int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nslices) return;
    int32_t w = 0;
    for (int32_t r = 0; r < C; r++) {
        int64_t p = s * C + r;
        if (p < n && !is_long(ideg[p], long_row)) w = max(w, ideg[p]);
    }
    width[s] = w;
    ssize[s] = (int64_t)C * ((w + 3) & ~3);
}

// Largest slice s in [lo, hi] whose first int4 slot is <= q (empty slices
// share their successor's offset and are passed over).
__device__ __forceinline__ int64_t slice_of(const int64_t *slice_off, int64_t q, int64_t lo,
                                            int64_t hi) {
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if ((slice_off[mid] >> 2) <= q) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The slice holding the first int4 slot of every 32-slot chunk (one thread
// per chunk, all lanes searching at once), so that k_fill_flat's warps start
// from a narrow slice range instead of searching the whole offset table on
// one lane.
__global__ void k_chunk_slice(int64_t nslices, int64_t nchunks, const int64_t *slice_off,
                              int32_t *cslice) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c < nchunks) cslice[c] = (int32_t)slice_of(slice_off, c * 32, 0, nslices - 1);
}

// Flat fill of the 4-interleaved SELL: one thread per int4 slot (four entries
// of one row), 32 consecutive slots per warp, so every thread does the same
// small amount of work (four column loads, four inv gathers, one coalesced
// 16-byte store) however long its row is, and a warp's store is 512
// contiguous bytes. A slot's slice is found by binary search inside the
// range from its chunk's first slice to the next chunk's. kPush (symmetric graphs, where
// a position's push row is its SELL row): the same entries are written to the
// push CSR too, so the CSR is read and gathered once for both. Long rows stay
// padding here (their lists are filled by k_fill_chunks).
template <bool kPush>
__global__ void __launch_bounds__(256) k_fill_flat(
    int64_t n, int64_t nslices, int64_t nslots, int32_t C, int32_t log2C, int32_t long_row,
    const int64_t *slice_off, const int32_t *cslice, const int32_t *ideg, const int64_t *rstart,
    const int2 *sl, const int32_t *col, const int32_t *inv, int32_t *scol, const int64_t *prow,
    int32_t *pcol) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = (nslots + 31) >> 5;
    const uint64_t pstream = l2_evict_first();
    int4 *scol4 = reinterpret_cast<int4 *>(scol);
    for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < nchunks;
         w += nw) {
        const int64_t q = w * 32 + lane;
        // slots of this chunk lie in [slice of its first slot, slice of the
        // next chunk's first slot]
        const int64_t s_lo = __ldg(cslice + w);
        const int64_t s_hi = w + 1 < nchunks ? __ldg(cslice + w + 1) : nslices - 1;
        if (q >= nslots) continue;
        const int64_t sc = slice_of(slice_off, q, s_lo, s_hi);
        const int64_t k4 = q - (slice_off[sc] >> 2);
        const int32_t g = (int32_t)(k4 >> log2C);
        const int64_t p = sc * C + (k4 & (C - 1));
        const int32_t pad = p < n ? (int32_t)p : 0;
        int32_t v[4] = {pad, pad, pad, pad};
        const int32_t d = p < n ? __ldg(ideg + p) : 0;
        const int32_t k0 = 4 * g;
        if (p < n && !is_long(d, long_row) && k0 < d) {
            const int64_t b = __ldg(rstart + p);
            const int2 run = __ldg(sl + p);
            int32_t c[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int32_t kk = k0 + k;
                const int32_t raw = kk < run.x ? kk : kk + run.y;
                c[k] = kk < d ? ld_hint(col + b + raw, pstream) : -1;
            }
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (c[k] >= 0) v[k] = __ldg(inv + c[k]);
            if (kPush) {
                const int64_t at = __ldg(prow + p) + k0;
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (k0 + k < d) __stcs(pcol + at + k, v[k]);
            }
        }
        __stcs(scol4 + q, make_int4(v[0], v[1], v[2], v[3]));
    }
}

// Push-side CSR in position space for graphs whose push side differs from
// the pull side, one thread per row: four column loads, then four inv
// gathers, per step (columns read evict-first, outputs streamed). Rows with
// more than kFillChunk raw entries are left to k_fill_chunks.
__global__ void k_fill_push(int64_t n, const int32_t *perm, const int32_t *inv,
                            const int64_t *prow, const int64_t *rp, const int32_t *col,
                            int32_t *pcol) {
    const int64_t str = (int64_t)gridDim.x * blockDim.x;
    const uint64_t pstream = l2_evict_first();
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += str) {
        const int32_t v = perm[p];
        int64_t at = prow[p];
        const int64_t b = rp[v], e = rp[v + 1];
        if (e - b > kFillChunk) continue;
        for (int64_t i = b; i < e; i += 4) {
            int32_t c[4], q[4];
#pragma unroll
            for (int k = 0; k < 4; k++) c[k] = i + k < e ? ld_hint(col + i + k, pstream) : v;
#pragma unroll
            for (int k = 0; k < 4; k++) q[k] = c[k] != v ? __ldg(inv + c[k]) : 0;
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (c[k] != v) __stcs(pcol + at++, q[k]);
        }
    }
}

// Long-row list: flags, then scatter of positions and lengths after a scan.
__global__ void k_long_flags(int64_t n, int32_t long_row, const int32_t *ideg, int32_t *flag) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p < n) flag[p] = is_long(ideg[p], long_row) ? 1 : 0;
}

__global__ void k_long_scatter(int64_t n, const int32_t *flag, const int64_t *idx,
                               const int32_t *ideg, int32_t *lrow, int32_t *llen) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p < n && flag[p]) {
        lrow[idx[p]] = (int32_t)p;
        llen[idx[p]] = ideg[p];
    }
}

// ------------------------------------------------ rows filled in chunks
// Long rows (hubs, up to millions of entries) are copied in kFillChunk-entry
// chunks spread over all warps instead of by one warp each. Rows are sorted,
// so a row's self-loops form one run [lo, hi); the output index of input
// entry j of row v is then (j - b) - (clamp(j, lo, hi) - lo), computable per
// entry without a scan.
__global__ void k_flag_raw(int64_t n, const int32_t *perm, const int64_t *rp, int64_t thr,
                           int32_t *flag) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p < n) {
        const int32_t v = perm[p];
        flag[p] = (rp[v + 1] - rp[v]) > thr ? 1 : 0;
    }
}

__global__ void k_scatter_flagged(int64_t n, const int32_t *flag, const int64_t *idx,
                                  int32_t *rows) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p < n && flag[p]) rows[idx[p]] = (int32_t)p;
}

// Per listed row: chunk count over its raw entries and its self-loop run.
__global__ void k_chunk_src(int64_t nr, const int32_t *rows, const int32_t *perm,
                            const int64_t *rp, const int32_t *col, int64_t chunk, int32_t *cnt,
                            int64_t *slo, int64_t *shi) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nr) return;
    const int32_t v = perm[rows[i]];
    const int64_t b = rp[v], e = rp[v + 1];
    cnt[i] = (int32_t)((e - b + chunk - 1) / chunk);
    int64_t lo = b, hi = e;  // first entry >= v
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (col[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    int64_t lo2 = lo, hi2 = e;  // first entry > v
    while (lo2 < hi2) {
        const int64_t mid = (lo2 + hi2) >> 1;
        if (col[mid] <= v) lo2 = mid + 1;
        else hi2 = mid;
    }
    slo[i] = lo;
    shi[i] = lo2;
}

// crow[cb[i] + c] = i for every chunk c of row i.
__global__ void k_chunk_rows(int64_t nr, const int64_t *cb, int32_t *crow) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nr) return;
    for (int64_t k = cb[i]; k < cb[i + 1]; k++) crow[k] = (int32_t)i;
}

// One warp per chunk: out[obase + kept index] = inv[col[j]] for the chunk's
// raw entries j, self-loops dropped. obase is indexed by position (by_pos)
// or by list index.
__global__ void k_fill_chunks(int64_t nchunks, const int32_t *crow, const int32_t *rows,
                              const int64_t *cb, const int64_t *slo, const int64_t *shi,
                              const int32_t *perm, const int32_t *inv, const int64_t *rp,
                              const int32_t *col, const int64_t *obase, int by_pos,
                              int32_t *out, const int64_t *obase2, int32_t *out2) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    const uint64_t pstream = l2_evict_first();
    for (int64_t k = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); k < nchunks;
         k += nw) {
        const int32_t i = crow[k];
        const int32_t p = rows[i];
        const int32_t v = perm[p];
        const int64_t b = rp[v], e = rp[v + 1];
        const int64_t s0 = b + (k - cb[i]) * kFillChunk;
        const int64_t s1 = min(e, s0 + kFillChunk);
        const int64_t lo = slo[i], hi = shi[i];
        const int64_t o = by_pos ? obase[p] : obase[i];
        const int64_t o2 = out2 ? obase2[p] : 0;
        // four entries per lane per step: their column loads, then their
        // four inv gathers, are issued before any is used
        for (int64_t j0 = s0 + lane; j0 < s1; j0 += 128) {
            int32_t c[4], q[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int64_t j = j0 + 32 * u;
                c[u] = j < s1 ? ld_hint(col + j, pstream) : v;
            }
#pragma unroll
            for (int u = 0; u < 4; u++) q[u] = c[u] != v ? __ldg(inv + c[u]) : 0;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int64_t j = j0 + 32 * u;
                if (c[u] == v) continue;  // a self-loop, or past the chunk
                const int64_t at = (j - b) - (min(max(j, lo), hi) - lo);
                __stcs(out + o + at, q[u]);
                if (out2) __stcs(out2 + o2 + at, q[u]);
            }
        }
    }
}

// Initial visited mask: padded tail rows and rows without sources can never
// be discovered by a pull, so they start visited (their level stays -1).
__global__ void k_vinit(int64_t n, int64_t nwords, const int32_t *ideg, uint32_t *vinit,
                        unsigned long long *counters) {
    // warp per word, grid-stride (coalesced degree loads, one ballot per
    // word); the three counts are combined in the block, then one atomic each
    __shared__ unsigned long long s_c[3][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long act = 0, zero = 0, sum = 0;
    for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < nwords; w += nw) {
        const int64_t p = w * 32 + lane;
        const int32_t d = p < n ? ideg[p] : 0;
        const uint32_t m = __ballot_sync(kFull, p >= n || d == 0);
        if (lane == 0) vinit[w] = m;
        act += lane == 0 && m != kFull;                 // active words
        zero += p < n && d == 0;                        // rows without sources
        sum += (unsigned long long)d;                   // pull-side entries
    }
    act = warp_sum(act);
    zero = warp_sum(zero);
    sum = warp_sum(sum);
    if (lane == 0) {
        s_c[0][wib] = act;
        s_c[1][wib] = zero;
        s_c[2][wib] = sum;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        unsigned long long t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += s_c[threadIdx.x][k];
        if (t) atomicAdd(&counters[threadIdx.x], t);
    }
}

inline unsigned grid_for(int64_t count, int tpb) { return (unsigned)((count + tpb - 1) / tpb); }

// Reads one int64 device value on stream st.
alb_status read_i64(const int64_t *d, int64_t *h, cudaStream_t st) {
    ALB_CK(cudaMemcpyAsync(h, d, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    ALB_CK(cudaStreamSynchronize(st));
    return ALB_OK;
}

// Chunk list of nr rows: cb (nr + 1 first-chunk indices) from per-row counts,
// crow (row of each chunk). cb and crow are allocated here.
alb_status chunk_list(const int32_t *cnt, int64_t nr, int64_t **cb, int32_t **crow,
                      int64_t *nchunks, cudaStream_t st) {
    ALB_TRY(dmalloc((void **)cb, sizeof(int64_t) * (nr + 1), "chunk bases"));
    ALB_TRY(exclusive_scan(cnt, *cb, nr, st));
    ALB_TRY(read_i64(*cb + nr, nchunks, st));
    ALB_TRY(dmalloc((void **)crow, sizeof(int32_t) * std::max<int64_t>(*nchunks, 1),
                    "chunk rows"));
    if (nr) k_chunk_rows<<<grid_for(nr, 256), 256, 0, st>>>(nr, *cb, *crow);
    ALB_CK(cudaGetLastError());
    return ALB_OK;
}

// Copies the rows listed in rows[0..nr) (positions) into out in position
// space, kFillChunk raw entries per warp task (see k_fill_chunks).
alb_status fill_rows_chunked(const int32_t *rows, int64_t nr, const int32_t *perm,
                             const int32_t *inv, const int64_t *rp, const int32_t *col,
                             const int64_t *obase, bool by_pos, int32_t *out, unsigned grid,
                             cudaStream_t st, const int64_t *obase2 = nullptr,
                             int32_t *out2 = nullptr) {
    if (nr == 0) return ALB_OK;
    int32_t *cnt = nullptr, *crow = nullptr;
    int64_t *slo = nullptr, *shi = nullptr, *cb = nullptr;
    auto cleanup = [&]() {
        dfree(cnt);
        dfree(crow);
        dfree(slo);
        dfree(shi);
        dfree(cb);
    };
    alb_status rc = [&]() -> alb_status {
        ALB_TRY(dmalloc((void **)&cnt, sizeof(int32_t) * nr, "chunk counts"));
        ALB_TRY(dmalloc((void **)&slo, sizeof(int64_t) * nr, "self-loop runs"));
        ALB_TRY(dmalloc((void **)&shi, sizeof(int64_t) * nr, "self-loop runs"));
        k_chunk_src<<<grid_for(nr, 256), 256, 0, st>>>(nr, rows, perm, rp, col, kFillChunk, cnt,
                                                        slo, shi);
        ALB_CK(cudaGetLastError());
        int64_t nchunks = 0;
        ALB_TRY(chunk_list(cnt, nr, &cb, &crow, &nchunks, st));
        if (nchunks)
            k_fill_chunks<<<grid, 256, 0, st>>>(nchunks, crow, rows, cb, slo, shi, perm, inv, rp,
                                                col, obase, by_pos ? 1 : 0, out, obase2, out2);
        ALB_CK(cudaGetLastError());
        // the temporaries are freed below: finish with them first
        ALB_CK(cudaStreamSynchronize(st));
        return ALB_OK;
    }();
    cleanup();
    return rc;
}

alb_status sell_build_impl(alb_graph *g, int32_t C, int32_t sigma, int32_t long_row) {
    const int64_t n = g->n;
    cudaStream_t st = g->stream;
    free_sell(g->sell);
    loop_cache_free(g);
    bfs_scratch_free(g);  // bitmap sizes depend on C
    ms_scratch_free(g);
    Sell &s = g->sell;
    s.C = C;
    s.log2C = C == 8 ? 3 : C == 16 ? 4 : C == 32 ? 5 : 6;
    s.sigma = sigma;
    s.long_row = long_row;
    s.nslices = (n + C - 1) / C;
    const int64_t npad = s.nslices * C;
    s.nwords = (npad + 31) / 32;
    int32_t *ilen = nullptr, *olen = nullptr, *dmax = nullptr, *sl_off = nullptr, *sl_num = nullptr;
    int64_t *ssize = nullptr, *rstart = nullptr;
    int2 *slrun = nullptr;
    unsigned long long *dcnt = nullptr;
    auto tmp_free = [&]() {
        dfree(ilen);
        dfree(olen);
        dfree(dmax);
        dfree(ssize);
        dfree(dcnt);
        dfree(sl_off);
        dfree(sl_num);
        dfree(rstart);
        dfree(slrun);
    };
    PhaseLog ph("sell_build");
    alb_status rc = [&]() -> alb_status {
        ALB_TRY(dmalloc((void **)&ilen, sizeof(int32_t) * n, "row lengths"));
        ALB_TRY(dmalloc((void **)&olen, sizeof(int32_t) * n, "row lengths"));
        ALB_TRY(dmalloc((void **)&dmax, sizeof(int32_t) * 2, "max length"));
        ALB_TRY(dmalloc((void **)&dcnt, sizeof(unsigned long long) * 3, "counters"));
        ALB_TRY(dmalloc((void **)&s.perm, sizeof(int32_t) * n, "perm"));
        ALB_TRY(dmalloc((void **)&s.inv, sizeof(int32_t) * n, "inv"));
        ALB_TRY(dmalloc((void **)&s.ideg, sizeof(int32_t) * n, "ideg"));
        ALB_TRY(dmalloc((void **)&s.odeg, sizeof(int32_t) * n, "odeg"));
        ALB_TRY(dmalloc((void **)&s.width, sizeof(int32_t) * s.nslices, "width"));
        ALB_TRY(dmalloc((void **)&s.slice_off, sizeof(int64_t) * (s.nslices + 1), "slice_off"));
        ALB_TRY(dmalloc((void **)&ssize, sizeof(int64_t) * (s.nslices + 1), "slice sizes"));
        ALB_TRY(dmalloc((void **)&s.prow, sizeof(int64_t) * (n + 1), "push offsets"));
        ALB_TRY(dmalloc((void **)&s.vinit, sizeof(uint32_t) * s.nwords, "vinit"));
        ALB_TRY(dmalloc((void **)&sl_off, sizeof(int32_t) * n, "self-loop runs"));
        ALB_TRY(dmalloc((void **)&sl_num, sizeof(int32_t) * n, "self-loop runs"));
        ALB_TRY(dmalloc((void **)&rstart, sizeof(int64_t) * n, "row starts"));
        ALB_TRY(dmalloc((void **)&slrun, sizeof(int2) * n, "self-loop runs"));
        ALB_CK(cudaMemsetAsync(dmax, 0, sizeof(int32_t) * 2, st));
        ALB_CK(cudaMemsetAsync(dcnt, 0, sizeof(unsigned long long) * 3, st));
        const int T = 256;
        // grid-stride kernels that end in a block-combined atomic
        const unsigned red_grid =
            (unsigned)std::min<int64_t>(grid_for(n, T), (int64_t)g->num_sms * 16);
        k_row_lengths<<<red_grid, T, 0, st>>>(n, g->rp_in, g->col_in, ilen, dmax, sl_off,
                                                     sl_num);
        if (g->symmetric)
            ALB_CK(cudaMemcpyAsync(olen, ilen, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st));
        else
            k_row_lengths<<<red_grid, T, 0, st>>>(n, g->rp_out, g->col_out, olen, dmax + 1);
        ALB_CK(cudaGetLastError());
        ph.mark("alloc_lengths", st);
        ALB_TRY(window_order(n, sigma, ilen, s.perm, st));
        ph.mark("sort", st);
        k_positions<<<grid_for(n, T), T, 0, st>>>(n, s.perm, ilen, olen, s.inv, s.ideg, s.odeg,
                                                   g->rp_in, sl_off, sl_num, rstart, slrun);
        k_widths<<<grid_for(s.nslices, T), T, 0, st>>>(n, s.nslices, C, long_row, s.ideg, s.width,
                                                        ssize);
        ALB_CK(cudaGetLastError());
        ALB_TRY(exclusive_scan(ssize, s.slice_off, s.nslices, st));
        ALB_TRY(exclusive_scan(s.odeg, s.prow, n, st));
        int64_t hsz[2] = {0, 0};
        ALB_CK(cudaMemcpyAsync(&hsz[0], s.slice_off + s.nslices, sizeof(int64_t),
                               cudaMemcpyDeviceToHost, st));
        ALB_CK(cudaMemcpyAsync(&hsz[1], s.prow + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        int32_t hmax[2] = {0, 0};
        ALB_CK(cudaMemcpyAsync(hmax, dmax, sizeof(hmax), cudaMemcpyDeviceToHost, st));
        ALB_CK(cudaStreamSynchronize(st));
        s.ncol = hsz[0];
        s.m_out = hsz[1];
        s.max_deg = std::max(hmax[0], hmax[1]);
        ALB_TRY(dmalloc((void **)&s.col, sizeof(int32_t) * (size_t)std::max<int64_t>(s.ncol, 4),
                        "SELL columns"));
        ALB_TRY(dmalloc((void **)&s.pcol, sizeof(int32_t) * (size_t)std::max<int64_t>(s.m_out, 1),
                        "push columns"));
        ph.mark("positions_widths_scans", st);
        const unsigned fill_grid = (unsigned)(g->num_sms * 8);
        // a symmetric graph's push row of a position is its pull row: one
        // pass writes both (long rows' push rows come with their lists)
        const bool fused = g->symmetric;
        const int64_t nslots = s.ncol / 4;
        if (nslots > 0) {
            const int64_t nchunks = (nslots + 31) / 32;
            int32_t *cslice = nullptr;
            struct Tmp {
                int32_t *&a;
                ~Tmp() { dfree(a); }
            } tmp{cslice};
            ALB_TRY(dmalloc((void **)&cslice, sizeof(int32_t) * nchunks, "chunk slices"));
            k_chunk_slice<<<grid_for(nchunks, T), T, 0, st>>>(s.nslices, nchunks, s.slice_off,
                                                               cslice);
            const unsigned flat_grid =
                (unsigned)std::min<int64_t>((nslots + T - 1) / T, (int64_t)g->num_sms * 64);
            if (fused)
                k_fill_flat<true><<<flat_grid, T, 0, st>>>(n, s.nslices, nslots, C, s.log2C,
                                                           long_row, s.slice_off, cslice, s.ideg,
                                                           rstart, slrun, g->col_in, s.inv, s.col,
                                                           s.prow, s.pcol);
            else
                k_fill_flat<false><<<flat_grid, T, 0, st>>>(n, s.nslices, nslots, C, s.log2C,
                                                            long_row, s.slice_off, cslice, s.ideg,
                                                            rstart, slrun, g->col_in, s.inv,
                                                            s.col, s.prow, s.pcol);
            ALB_CK(cudaGetLastError());
        }
        if (!fused)
            k_fill_push<<<fill_grid, T, 0, st>>>(n, s.perm, s.inv, s.prow, g->rp_out, g->col_out,
                                                 s.pcol);
        ALB_CK(cudaGetLastError());
        // push rows too long for one warp: listed, then copied in chunks
        if (!fused) {
            int32_t *flag = nullptr, *rows = nullptr;
            int64_t *idx = nullptr;
            struct Tmp {
                int32_t *&a, *&b;
                int64_t *&c;
                ~Tmp() {
                    dfree(a);
                    dfree(b);
                    dfree(c);
                }
            } tmp{flag, rows, idx};
            ALB_TRY(dmalloc((void **)&flag, sizeof(int32_t) * n, "long push-row flags"));
            ALB_TRY(dmalloc((void **)&idx, sizeof(int64_t) * (n + 1), "long push-row index"));
            k_flag_raw<<<grid_for(n, T), T, 0, st>>>(n, s.perm, g->rp_out, kFillChunk, flag);
            ALB_CK(cudaGetLastError());
            ALB_TRY(exclusive_scan(flag, idx, n, st));
            int64_t nr = 0;
            ALB_TRY(read_i64(idx + n, &nr, st));
            if (nr) {
                ALB_TRY(dmalloc((void **)&rows, sizeof(int32_t) * nr, "long push rows"));
                k_scatter_flagged<<<grid_for(n, T), T, 0, st>>>(n, flag, idx, rows);
                ALB_CK(cudaGetLastError());
                ALB_TRY(fill_rows_chunked(rows, nr, s.perm, s.inv, g->rp_out, g->col_out, s.prow,
                                          true, s.pcol, fill_grid, st));
            }
        }
        ph.mark("fill", st);
        // long rows: flags -> scan -> scatter -> offsets -> fill
        {
            int32_t *flag = nullptr, *llen = nullptr;
            int64_t *idx = nullptr;
            struct Tmp {
                int32_t *&a, *&b;
                int64_t *&c;
                ~Tmp() {
                    dfree(a);
                    dfree(b);
                    dfree(c);
                }
            } tmp{flag, llen, idx};
            ALB_TRY(dmalloc((void **)&flag, sizeof(int32_t) * n, "long-row flags"));
            ALB_TRY(dmalloc((void **)&idx, sizeof(int64_t) * (n + 1), "long-row index"));
            k_long_flags<<<grid_for(n, T), T, 0, st>>>(n, long_row, s.ideg, flag);
            ALB_CK(cudaGetLastError());
            ALB_TRY(exclusive_scan(flag, idx, n, st));
            ALB_CK(cudaMemcpyAsync(&s.nlong, idx + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
            ALB_CK(cudaStreamSynchronize(st));
            ALB_TRY(dmalloc((void **)&s.lrow, sizeof(int32_t) * std::max<int64_t>(s.nlong, 1),
                            "long rows"));
            ALB_TRY(dmalloc((void **)&llen, sizeof(int32_t) * std::max<int64_t>(s.nlong, 1),
                            "long-row lengths"));
            ALB_TRY(dmalloc((void **)&s.lptr, sizeof(int64_t) * (s.nlong + 1), "long-row offsets"));
            k_long_scatter<<<grid_for(n, T), T, 0, st>>>(n, flag, idx, s.ideg, s.lrow, llen);
            ALB_CK(cudaGetLastError());
            ALB_TRY(exclusive_scan(llen, s.lptr, s.nlong, st));
            int64_t nent = 0;
            ALB_CK(cudaMemcpyAsync(&nent, s.lptr + s.nlong, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
            ALB_CK(cudaStreamSynchronize(st));
            ALB_TRY(dmalloc((void **)&s.lcol, sizeof(int32_t) * std::max<int64_t>(nent, 1),
                            "long-row sources"));
            // (fused: the same entries are the long rows' push rows)
            ALB_TRY(fill_rows_chunked(s.lrow, s.nlong, s.perm, s.inv, g->rp_in, g->col_in, s.lptr,
                                      false, s.lcol, fill_grid, st, fused ? s.prow : nullptr,
                                      fused ? s.pcol : nullptr));
        }
        ph.mark("long_rows", st);
        k_vinit<<<(unsigned)std::min<int64_t>(grid_for(s.nwords * 32, T), (int64_t)g->num_sms * 16),
                  T, 0, st>>>(n, s.nwords, s.ideg, s.vinit, dcnt);
        ALB_CK(cudaGetLastError());
        unsigned long long hc[3];
        ALB_CK(cudaMemcpyAsync(hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
        ALB_CK(cudaStreamSynchronize(st));
        s.active0 = (int64_t)hc[0];
        s.zero_in = (int64_t)hc[1];
        s.m_in = (int64_t)hc[2];
        return ALB_OK;
    }();
    tmp_free();
    ph.mark("vinit_free", st);
    if (rc != ALB_OK) {
        free_sell(g->sell);
        return rc;
    }
    s.built = true;
    return ALB_OK;
}

}  // namespace
}  // namespace alb

namespace alb {
alb_status window_order(int64_t n, int32_t sigma, const int32_t *d_len, int32_t *d_perm,
                        cudaStream_t st) {
    return window_order_impl(n, sigma, d_len, d_perm, st);
}
}  // namespace alb

using namespace alb;

extern "C" {

alb_status alb_graph_create(int64_t n, const int64_t *rowptr, const int32_t *col, uint32_t flags,
                            alb_graph **out) {
    if (!out) return fail(ALB_ERR_INVALID, "alb_graph_create: out is NULL");
    *out = nullptr;
    if (n <= 0 || n > INT32_MAX || !rowptr || (!col && rowptr[n] > 0))
        return fail(ALB_ERR_INVALID, "alb_graph_create: bad arguments (n=%lld)", (long long)n);
    try {
        return create_impl(n, rowptr, col, flags, out);
    } catch (const std::bad_alloc &) {
        return fail(ALB_ERR_OOM, "alb_graph_create: host allocation failed");
    }
}

alb_status alb_graph_create32(int32_t n, const int32_t *rowptr, const int32_t *col,
                              uint32_t flags, alb_graph **out) {
    if (!out) return fail(ALB_ERR_INVALID, "alb_graph_create32: out is NULL");
    *out = nullptr;
    if (n <= 0 || !rowptr) return fail(ALB_ERR_INVALID, "alb_graph_create32: bad arguments");
    try {
        std::vector<int64_t> rp((size_t)n + 1);
        for (int64_t i = 0; i <= n; i++) rp[i] = rowptr[i];
        if (!col && rp[n] > 0) return fail(ALB_ERR_INVALID, "alb_graph_create32: col is NULL");
        return create_impl(n, rp.data(), col, flags, out);
    } catch (const std::bad_alloc &) {
        return fail(ALB_ERR_OOM, "alb_graph_create32: host allocation failed");
    }
}

alb_status alb_graph_create_undirected(int64_t n, const int64_t *rowptr, const int32_t *col,
                                       alb_graph **out) {
    if (!out) return fail(ALB_ERR_INVALID, "alb_graph_create_undirected: out is NULL");
    *out = nullptr;
    if (n <= 0 || n > INT32_MAX || !rowptr || (!col && rowptr[n] > 0))
        return fail(ALB_ERR_INVALID, "alb_graph_create_undirected: bad arguments");
    if (rowptr[0] != 0 || rowptr[n] < 0)
        return fail(ALB_ERR_INVALID, "row offsets must start at 0 and end at nnz >= 0");
    alb_graph *g = nullptr;
    ALB_TRY(graph_shell(n, &g));
    int64_t *d_rp = nullptr, *d_urp = nullptr;
    int32_t *d_col = nullptr, *d_ucol = nullptr;
    const int64_t nnz = rowptr[n];
    int64_t unnz = 0;
    alb_status st = upload(n, rowptr, col, &d_rp, &d_col, g->stream);
    bool sorted = true;
    if (st == ALB_OK) st = csr_check(n, d_rp, d_col, nnz, g->stream, &sorted);
    if (st == ALB_OK) st = merge_undirected(n, d_rp, d_col, nnz, &d_urp, &d_ucol, &unnz, g->stream);
    dfree(d_rp);
    dfree(d_col);
    if (st == ALB_OK) st = finish_device_csr(g, d_urp, d_ucol, unnz, ALB_CSR_SYMMETRIC);
    else {
        dfree(d_urp);
        dfree(d_ucol);
    }
    if (st != ALB_OK) {
        alb_graph_destroy(g);
        return st;
    }
    *out = g;
    return ALB_OK;
}

alb_status alb_graph_load(const char *path, alb_graph **out) {
    if (!path || !out) return fail(ALB_ERR_INVALID, "alb_graph_load: bad arguments");
    *out = nullptr;
    const size_t len = std::strlen(path);
    auto ends = [&](const char *ext) { return len >= 4 && std::strcmp(path + len - 4, ext) == 0; };
    alb_host_csr h;
    std::memset(&h, 0, sizeof(h));
    int32_t sym = 1;
    alb_status st;
    if (ends(".cbd")) st = alb_cbd_read(path, &h);
    else if (ends(".mtx")) st = alb_mtx_read(path, &h, &sym);
    else return fail(ALB_ERR_UNSUPPORTED, "alb_graph_load: %s is neither .mtx nor .cbd", path);
    if (st != ALB_OK) return st;
    if (h.n <= 0) {
        alb_host_csr_free(&h);
        return fail(ALB_ERR_IO, "alb_graph_load: %s holds no vertices", path);
    }
    // a .cbd file is taken as the reference takes it (its CSR as is, rows
    // and their transpose on the device); a non-symmetric .mtx becomes the
    // reference driver's undirected graph
    if (ends(".mtx") && !sym) st = alb_graph_create_undirected(h.n, h.rowptr, h.col, out);
    else st = alb_graph_create(h.n, h.rowptr, h.col, ends(".mtx") ? ALB_CSR_SYMMETRIC : ALB_CSR_IN, out);
    alb_host_csr_free(&h);
    return st;
}

alb_status alb_graph_export_csr(const alb_graph *g, int32_t side, int64_t *rowptr, int32_t *col) {
    if (!g || (side != 0 && side != 1))
        return fail(ALB_ERR_INVALID, "alb_graph_export_csr: bad arguments");
    ALB_CK(cudaSetDevice(g->device));
    const int64_t *rp = side == 0 ? g->rp_in : g->rp_out;
    const int32_t *cl = side == 0 ? g->col_in : g->col_out;
    const int64_t nnz = side == 0 ? g->nnz_in : g->nnz_out;
    if (rowptr)
        ALB_CK(cudaMemcpyAsync(rowptr, rp, sizeof(int64_t) * (size_t)(g->n + 1),
                               cudaMemcpyDeviceToHost, g->stream));
    if (col && nnz > 0)
        ALB_CK(cudaMemcpyAsync(col, cl, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToHost,
                               g->stream));
    ALB_CK(cudaStreamSynchronize(g->stream));
    return ALB_OK;
}

alb_status alb_graph_is_symmetric(const alb_graph *g, int32_t *symmetric) {
    if (!g || !symmetric) return fail(ALB_ERR_INVALID, "alb_graph_is_symmetric: bad arguments");
    *symmetric = g->symmetric ? 1 : 0;
    return ALB_OK;
}

void alb_graph_destroy(alb_graph *g) {
    if (!g) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    loop_cache_free(g);
    bfs_scratch_free(g);
    ms_scratch_free(g);
    free_sell(g->sell);
    if (g->col_out != g->col_in) dfree(g->col_out);
    if (g->rp_out != g->rp_in) dfree(g->rp_out);
    dfree(g->col_in);
    dfree(g->rp_in);
    if (g->ev0) cudaEventDestroy(g->ev0);
    if (g->ev1) cudaEventDestroy(g->ev1);
    if (g->own_stream) cudaStreamDestroy(g->own_stream);
    cudaGetLastError();
    if (prev >= 0) cudaSetDevice(prev);
    delete g;
}

alb_status alb_graph_info(const alb_graph *g, int64_t *n, int64_t *nnz) {
    if (!g) return fail(ALB_ERR_INVALID, "alb_graph_info: graph is NULL");
    if (n) *n = g->n;
    if (nnz) *nnz = g->nnz_in;
    return ALB_OK;
}

alb_status alb_graph_set_stream(alb_graph *g, void *cuda_stream) {
    if (!g) return fail(ALB_ERR_INVALID, "alb_graph_set_stream: graph is NULL");
    ALB_CK(cudaSetDevice(g->device));
    ALB_CK(cudaStreamSynchronize(g->stream));
    g->stream = cuda_stream ? (cudaStream_t)cuda_stream : g->own_stream;
    return ALB_OK;
}

void alb_sell_opts_default(alb_sell_opts *o) {
    if (!o) return;
    o->C = 32;
    o->sigma = 1024;
    // RMAT s22-s26, both BFS forms: 1024 beats 256 by 5-10 %; at 2048 the
    // widest slices (one lane per row, 512 column groups) make a level's tail
    o->long_row = 1024;
}

alb_status alb_sell_build(alb_graph *g, const alb_sell_opts *o, double *ms) {
    if (!g) return fail(ALB_ERR_INVALID, "alb_sell_build: graph is NULL");
    alb_sell_opts d;
    alb_sell_opts_default(&d);
    if (!o) o = &d;
    if (!(o->C == 8 || o->C == 16 || o->C == 32 || o->C == 64))
        return fail(ALB_ERR_UNSUPPORTED, "alb_sell_build: C must be 8, 16, 32 or 64 (got %d)", o->C);
    if (o->sigma < 1 || o->sigma > 16384)
        return fail(ALB_ERR_UNSUPPORTED, "alb_sell_build: sigma must be in [1, 16384] (got %d)",
                    o->sigma);
    ALB_CK(cudaSetDevice(g->device));
    ALB_CK(cudaEventRecord(g->ev0, g->stream));
    alb_status rc;
    try {
        rc = sell_build_impl(g, o->C, o->sigma, o->long_row);
    } catch (const std::bad_alloc &) {
        rc = fail(ALB_ERR_OOM, "alb_sell_build: host allocation failed");
    }
    if (rc != ALB_OK) return rc;
    ALB_CK(cudaEventRecord(g->ev1, g->stream));
    ALB_CK(cudaEventSynchronize(g->ev1));
    if (ms) {
        float f = 0;
        ALB_CK(cudaEventElapsedTime(&f, g->ev0, g->ev1));
        *ms = f;
    }
    return ALB_OK;
}

alb_status alb_sell_export(const alb_graph *g, int64_t *nslices, int32_t *perm, int32_t *width,
                           int64_t *slice_off, int32_t *col) {
    if (!g) return fail(ALB_ERR_INVALID, "alb_sell_export: graph is NULL");
    if (!g->sell.built) return fail(ALB_ERR_STATE, "alb_sell_export: SELL not built");
    const Sell &s = g->sell;
    ALB_CK(cudaSetDevice(g->device));
    if (nslices) *nslices = s.nslices;
    if (perm) ALB_CK(cudaMemcpy(perm, s.perm, sizeof(int32_t) * g->n, cudaMemcpyDeviceToHost));
    if (width)
        ALB_CK(cudaMemcpy(width, s.width, sizeof(int32_t) * s.nslices, cudaMemcpyDeviceToHost));
    if (slice_off)
        ALB_CK(cudaMemcpy(slice_off, s.slice_off, sizeof(int64_t) * (s.nslices + 1),
                          cudaMemcpyDeviceToHost));
    if (col) ALB_CK(cudaMemcpy(col, s.col, sizeof(int32_t) * s.ncol, cudaMemcpyDeviceToHost));
    return ALB_OK;
}

alb_status alb_sell_long_export(const alb_graph *g, int64_t *nlong, int32_t *lrow, int64_t *lptr,
                                int32_t *lcol) {
    if (!g) return fail(ALB_ERR_INVALID, "alb_sell_long_export: graph is NULL");
    if (!g->sell.built) return fail(ALB_ERR_STATE, "alb_sell_long_export: SELL not built");
    const Sell &s = g->sell;
    ALB_CK(cudaSetDevice(g->device));
    if (nlong) *nlong = s.nlong;
    if (lrow && s.nlong)
        ALB_CK(cudaMemcpy(lrow, s.lrow, sizeof(int32_t) * s.nlong, cudaMemcpyDeviceToHost));
    if (lptr) ALB_CK(cudaMemcpy(lptr, s.lptr, sizeof(int64_t) * (s.nlong + 1), cudaMemcpyDeviceToHost));
    if (lcol) {
        int64_t nent = 0;
        ALB_CK(cudaMemcpy(&nent, s.lptr + s.nlong, sizeof(int64_t), cudaMemcpyDeviceToHost));
        if (nent) ALB_CK(cudaMemcpy(lcol, s.lcol, sizeof(int32_t) * nent, cudaMemcpyDeviceToHost));
    }
    return ALB_OK;
}

}  // extern "C"
