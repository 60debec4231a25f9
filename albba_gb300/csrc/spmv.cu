// fp64 SELL-C-sigma SpMV, y = A x.
//
// Reference: kernel_SELLCS_DFC (bfs/src/bfs_par_kernels.c:8-53) over the
// matrix built by convert_csr_to_sellcs_dfc (bfs/src/sparse_matrix.c:
// 523-623): rows sorted by length inside sigma windows, C = 256 lanes per
// slice, one column op per entry index, and per lane a fused multiply-add
// (_vel_vfmadd_vvvvl) of value * x[column] into an accumulator that starts at
// 0; y[row] is that accumulator. Entry k of a row is handled by column op k,
// so every row sums its entries in CSR order with one rounding per entry --
// the result is fixed by the CSR alone, whatever C, sigma or the lanes are.
//
// GB300 layout: the same sigma-window order (the library's device sort), C =
// 32 rows per slice so that one warp owns a slice and lane r its row r, and
// the 4-interleaved layout of the BFS's SELL: group g of slice s holds entries
// 4g..4g+3 of every row, lane r's four column ids at col[off + 128 g + 4 r]
// (one int4 per lane, 512 contiguous bytes per warp) and its four values at
// the same index of val (two double2 per lane, 1 KB per warp). Entries are
// kept exactly as given (diagonal and repeated entries included); padding is
// never read: a lane stops at its row's length, so the fma chain is the
// reference's, bit for bit.
//
// Rows longer than kSpLong entries (the hubs of a power-law graph) keep an
// empty SELL row: in a slice a hub's lane waits on one group of x gathers at
// a time and holds its warp -- and the whole launch -- for tens of
// milliseconds. They are copied in CSR order to a separate list (longest
// first, each row padded to 8 entries so that a lane reads its row in
// aligned 32-byte column and 64-byte value blocks) and summed lane per row
// by k_spmv_long, which keeps two blocks of x gathers in flight ahead of the
// fma chain. The chain itself stays sequential -- its order is what makes y
// bit-identical -- and a dependent fp64 fma costs about 90 cycles on GB300
// (the fp64 pipe takes as long for one active lane as for 32), so the launch
// can end no sooner than the longest row's length x that latency; lane per
// row keeps every other row's chains, 32 per warp instruction, off the fp64
// pipe's critical path. The long rows run on a side stream beside the slices.
#include <algorithm>
#include <cstring>
#include <vector>

#include "graph.h"
#include "ingest.h"
#include "scan.cuh"

struct alb_sellmat {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;  // the long rows run beside the slices
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, fork = nullptr, join = nullptr;
    int64_t n = 0, nnz = 0, nslices = 0, stored = 0;
    int32_t sigma = 0;
    int32_t *perm = nullptr;       // position -> row
    int32_t *deg = nullptr;        // row length by position
    int64_t *slice_off = nullptr;  // first entry of each slice (multiple of 128)
    int32_t *col = nullptr;        // 4-interleaved column ids
    double *val = nullptr;         // values, same layout
    double *dx = nullptr, *dy = nullptr;  // staging for host vectors
    int64_t nlong = 0;             // rows longer than kSpLong, summed by a warp each
    int32_t *lrow = nullptr;       // their row ids, longest first
    int64_t *lptr = nullptr;       // first entry of each in lcol / lval (multiple of 8)
    int32_t *llen = nullptr;       // their lengths
    int32_t *lcol = nullptr;       // their entries in CSR order, each row padded to 8
    double *lval = nullptr;
    int32_t max_long = 0;          // the longest row's length
};

namespace alb {
namespace {

constexpr int kSpC = 32;
constexpr int32_t kSpLong = 512;  // longer rows are summed by a warp each

unsigned blocks_for(int64_t work, int block) {
    int64_t g = (work + block - 1) / block;
    return (unsigned)(g < 1 ? 1 : g);
}

__global__ void k_lengths(int64_t n, const int64_t *rp, int32_t *len) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r < n) len[r] = (int32_t)(rp[r + 1] - rp[r]);
}

__global__ void k_sp_positions(int64_t n, const int32_t *perm, const int32_t *len, int32_t *deg) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p < n) deg[p] = len[perm[p]];
}

// Slice sizes: 32 rows x the longest row rounded up to 4.
__global__ void k_sp_sizes(int64_t n, int64_t nslices, const int32_t *deg, int64_t *ssize) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= nslices) return;
    int32_t w = 0;
    for (int r = 0; r < kSpC; r++) {
        const int64_t p = s * kSpC + r;
        if (p < n && deg[p] <= kSpLong) w = max(w, deg[p]);
    }
    ssize[s] = (int64_t)kSpC * ((w + 3) & ~3);
}

// One thread per position: copies its row's entries (CSR order) into the
// interleaved slots; the slice's remaining groups of the row are padded with
// column 0 and value 0 (never read).
__global__ void k_sp_fill(int64_t n, int64_t npad, const int32_t *perm, const int32_t *deg,
                          const int64_t *slice_off, const int64_t *rp, const int32_t *col,
                          const double *val, int32_t *scol, double *sval) {
    const int64_t str = (int64_t)gridDim.x * blockDim.x;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npad; p += str) {
        const int64_t s = p / kSpC;
        const int64_t base = slice_off[s] + 4 * (p % kSpC);
        const int32_t ng = (int32_t)((slice_off[s + 1] - slice_off[s]) / (4 * kSpC));
        const int32_t d = p < n && deg[p] <= kSpLong ? deg[p] : 0;
        const int64_t b = p < n ? rp[perm[p]] : 0;
        for (int32_t g = 0; g < ng; g++) {
            int32_t c4[4];
            double v4[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int32_t e = 4 * g + k;
                c4[k] = e < d ? col[b + e] : 0;
                v4[k] = e < d ? val[b + e] : 0.0;
            }
            const int64_t at = base + (int64_t)g * 4 * kSpC;
            *reinterpret_cast<int4 *>(scol + at) = make_int4(c4[0], c4[1], c4[2], c4[3]);
            reinterpret_cast<double2 *>(sval + at)[0] = make_double2(v4[0], v4[1]);
            reinterpret_cast<double2 *>(sval + at)[1] = make_double2(v4[2], v4[3]);
        }
    }
}

// Warp per slice, lane per row. The next group's columns and values are
// requested before this group's x gathers are used, so each lane keeps the
// stream and the gathers in flight together.
// 512 threads a block (32 K registers): such a block does not fit on an SM
// beside a solo long-row CTA (k_spmv_long<true>), which keeps the slices off
// the longest chains' SMs.
constexpr int kSpBlock = 512;

__global__ void __launch_bounds__(kSpBlock) k_spmv(int64_t n, int64_t nslices, const int32_t *perm,
                                              const int32_t *deg, const int64_t *slice_off,
                                              const int32_t *col, const double *val,
                                              const double *x, double *y) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t pol = l2_evict_first();
    for (int64_t s = w0; s < nslices; s += nw) {
        const int64_t p = s * kSpC + lane;
        const int32_t dr = p < n ? __ldg(deg + p) : 0;
        const bool mine = p < n && dr <= kSpLong;  // long rows: k_spmv_long
        const int32_t d = mine ? dr : 0;
        const int32_t ng = (d + 3) >> 2;
        const int64_t base = __ldg(slice_off + s) + 4 * lane;
        const int4 *cp = reinterpret_cast<const int4 *>(col + base);
        const double2 *vp = reinterpret_cast<const double2 *>(val + base);
        double acc = 0.0;
        int4 c = make_int4(0, 0, 0, 0);
        double2 va = make_double2(0.0, 0.0), vb = va;
        if (ng > 0) {
            c = ld_stream(cp, pol);
            va = __ldcs(vp);
            vb = __ldcs(vp + 1);
        }
        for (int32_t g = 0; g < ng; g++) {
            int4 cn = c;
            double2 van = va, vbn = vb;
            if (g + 1 < ng) {
                cn = ld_stream(cp + (int64_t)(g + 1) * kSpC, pol);
                van = __ldcs(vp + (int64_t)(g + 1) * 2 * kSpC);
                vbn = __ldcs(vp + (int64_t)(g + 1) * 2 * kSpC + 1);
            }
            const int32_t left = d - 4 * g;
            const double x0 = __ldg(x + c.x);
            const double x1 = left > 1 ? __ldg(x + c.y) : 0.0;
            const double x2 = left > 2 ? __ldg(x + c.z) : 0.0;
            const double x3 = left > 3 ? __ldg(x + c.w) : 0.0;
            acc = fma(va.x, x0, acc);
            if (left > 1) acc = fma(va.y, x1, acc);
            if (left > 2) acc = fma(vb.x, x2, acc);
            if (left > 3) acc = fma(vb.y, x3, acc);
            c = cn;
            va = van;
            vb = vbn;
        }
        if (mine) y[__ldg(perm + p)] = acc;
    }
}

// Lane per long row (rows longest first). kSolo: the launch's longest rows,
// one per CTA of 1024 threads of which one lane works: the CTA holds most of
// its SM's registers until the row ends, so no slices block shares the SM
// and its fp64 pipe with the chain that sets the SpMV's length (measured: a
// slices kernel beside the longest chain slowed it from 8.0 to about 10 ms at
// RMAT s22), and the chain waits on no other lane's gathers (a warp's
// cp.async wait ends when its slowest lane's copies land). The other long
// rows go 32 of similar length per warp.
// Entries in blocks of kLb. Each lane streams its row through two
// shared-memory rings filled by cp.async: column ids kLd blocks ahead of the
// x gathers that need them, values and x (each gather 8 bytes) kLd blocks
// ahead of the fmas. The group committed at step t carries block t's values
// and gathers and block t + kLd's columns, so one wait gives both. With the
// fma chain at about 90 cycles per entry, each load has kLd x kLb entries'
// worth of chain time to land. Ring layout: lane-fastest, so that the 32
// lanes' accesses fall in different banks.
constexpr int kSpLongBlock = 32;  // one warp per CTA
constexpr int kLb = 8;
constexpr int kLd = 8;

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

constexpr int kSoloThreads = 1024;
constexpr int64_t kSoloRows = 8;  // rows on CTAs of their own

template <bool kSolo>
__global__ void __launch_bounds__(kSolo ? kSoloThreads : kSpLongBlock)
    k_spmv_long(int64_t nlong, int64_t first, const int32_t *lrow, const int64_t *lptr,
                const int32_t *llen, const int32_t *lcol, const double *lval, const double *x,
                double *y) {
    __shared__ double2 s_v[1][kLd][kLb / 2][32];
    __shared__ double s_x[1][kLd][kLb][32];
    __shared__ int4 s_c[1][kLd][kLb / 4][32];
    // kSolo: warp 0 of CTA b takes row first + b on lane 0 (the other warps
    // leave at once); otherwise warp w takes rows first + 32 w + lane
    if (kSolo && threadIdx.x >= 32) return;
    const int lane = threadIdx.x & 31, wib = 0;
    const int64_t i = kSolo ? (lane == 0 ? first + blockIdx.x : nlong)
                            : first + (int64_t)blockIdx.x * 32 + lane;
    const int64_t b = i < nlong ? lptr[i] : 0;
    const int64_t e = i < nlong ? b + llen[i] : 0;
    const int64_t nblk = (e - b + kLb - 1) / kLb;
    // values and x of block t (columns c); columns of block t + kLd
    auto issue = [&](int64_t t, const int32_t (&c)[kLb]) {
        const int slot = (int)(t % kLd);
        if (t < nblk) {
            const int64_t s0 = b + t * kLb;
            const double2 *src = reinterpret_cast<const double2 *>(lval + s0);
#pragma unroll
            for (int h = 0; h < kLb / 2; h++) cp_async16(&s_v[wib][slot][h][lane], src + h);
#pragma unroll
            for (int k = 0; k < kLb; k++)
                if (s0 + k < e) cp_async8(&s_x[wib][slot][k][lane], x + c[k]);
        }
        if (t + kLd < nblk) {
            const int4 *src = reinterpret_cast<const int4 *>(lcol + b + (t + kLd) * kLb);
#pragma unroll
            for (int h = 0; h < kLb / 4; h++) cp_async16(&s_c[wib][slot][h][lane], src + h);
        }
        cp_async_commit();
    };
    int32_t c[kLb];
    for (int t = 0; t < kLd; t++) {
#pragma unroll
        for (int k = 0; k < kLb; k++) c[k] = 0;
        if (t < nblk) {
            const int4 *q = reinterpret_cast<const int4 *>(lcol + b + (int64_t)t * kLb);
            const int4 u = __ldcs(q), w = __ldcs(q + 1);
            c[0] = u.x, c[1] = u.y, c[2] = u.z, c[3] = u.w;
            c[4] = w.x, c[5] = w.y, c[6] = w.z, c[7] = w.w;
        }
        issue(t, c);
    }
    double acc = 0.0;
    for (int64_t t = 0; t < nblk; t++) {
        cp_async_wait<kLd - 1>();  // this lane's group t has landed
        const int slot = (int)(t % kLd);
        const int64_t rem = e - (b + t * kLb);
#pragma unroll
        for (int h = 0; h < kLb / 2; h++) {
            const double2 v = s_v[wib][slot][h][lane];
            if (2 * h < rem) acc = fma(v.x, s_x[wib][slot][2 * h][lane], acc);
            if (2 * h + 1 < rem) acc = fma(v.y, s_x[wib][slot][2 * h + 1][lane], acc);
        }
        // block t + kLd's columns (landed with group t), read out before the
        // slot is refilled; the refill comes after the fmas in program order,
        // so their shared loads have landed when the copies issue
        const int4 u = s_c[wib][slot][0][lane], w = s_c[wib][slot][1][lane];
        c[0] = u.x, c[1] = u.y, c[2] = u.z, c[3] = u.w;
        c[4] = w.x, c[5] = w.y, c[6] = w.z, c[7] = w.w;
        asm volatile("" ::"d"(acc), "r"(c[0]), "r"(c[7]) : "memory");
        issue(t + kLd, c);
    }
    cp_async_wait<0>();
    if (i < nlong) y[lrow[i]] = acc;
}

__global__ void k_sp_long_flags(int64_t n, const int32_t *len, int32_t *flag) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r < n) flag[r] = len[r] > kSpLong ? 1 : 0;
}

__global__ void k_sp_long_scatter(int64_t n, const int32_t *flag, const int64_t *idx,
                                  int32_t *lrow) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r < n && flag[r]) lrow[idx[r]] = (int32_t)r;
}

// One warp per long row: its entries copied in CSR order.
__global__ void k_sp_long_fill(int64_t nlong, const int32_t *lrow, const int64_t *lptr,
                               const int32_t *llen, const int64_t *rp, const int32_t *col,
                               const double *val, int32_t *lcol, double *lval) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < nlong; i += nw) {
        const int64_t src = rp[lrow[i]], dst = lptr[i], len = llen[i];
        for (int64_t k = lane; k < len; k += 32) {
            lcol[dst + k] = col[src + k];
            lval[dst + k] = val[src + k];
        }
    }
}

alb_status build(alb_sellmat *m, const int64_t *rowptr, const int32_t *col, const double *val) {
    const int64_t n = m->n, nnz = m->nnz;
    cudaStream_t st = m->stream;
    int64_t *d_rp = nullptr, *ssize = nullptr;
    int32_t *d_col = nullptr, *len = nullptr;
    double *d_val = nullptr;
    auto tmp_free = [&]() {
        dfree(d_rp);
        dfree(d_col);
        dfree(d_val);
        dfree(len);
        dfree(ssize);
    };
    alb_status rc = [&]() -> alb_status {
        ALB_TRY(dmalloc((void **)&d_rp, sizeof(int64_t) * (size_t)(n + 1), "SpMV row offsets"));
        ALB_TRY(dmalloc((void **)&d_col, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1), "SpMV columns"));
        ALB_TRY(dmalloc((void **)&d_val, sizeof(double) * (size_t)(nnz > 0 ? nnz : 1), "SpMV values"));
        ALB_CK(cudaMemcpyAsync(d_rp, rowptr, sizeof(int64_t) * (size_t)(n + 1),
                               cudaMemcpyHostToDevice, st));
        if (nnz > 0) {
            ALB_CK(cudaMemcpyAsync(d_col, col, sizeof(int32_t) * (size_t)nnz, cudaMemcpyHostToDevice, st));
            ALB_CK(cudaMemcpyAsync(d_val, val, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, st));
        }
        bool sorted = true;
        ALB_TRY(csr_check(n, d_rp, d_col, nnz, st, &sorted));
        m->nslices = (n + kSpC - 1) / kSpC;
        const int64_t npad = m->nslices * kSpC;
        ALB_TRY(dmalloc((void **)&len, sizeof(int32_t) * (size_t)n, "SpMV lengths"));
        ALB_TRY(dmalloc((void **)&m->perm, sizeof(int32_t) * (size_t)n, "SpMV order"));
        ALB_TRY(dmalloc((void **)&m->deg, sizeof(int32_t) * (size_t)n, "SpMV degrees"));
        ALB_TRY(dmalloc((void **)&ssize, sizeof(int64_t) * (size_t)(m->nslices + 1), "SpMV sizes"));
        ALB_TRY(dmalloc((void **)&m->slice_off, sizeof(int64_t) * (size_t)(m->nslices + 1),
                        "SpMV slice offsets"));
        k_lengths<<<blocks_for(n, 256), 256, 0, st>>>(n, d_rp, len);
        ALB_CK(cudaGetLastError());
        ALB_TRY(window_order(n, m->sigma, len, m->perm, st));
        k_sp_positions<<<blocks_for(n, 256), 256, 0, st>>>(n, m->perm, len, m->deg);
        k_sp_sizes<<<blocks_for(m->nslices, 256), 256, 0, st>>>(n, m->nslices, m->deg, ssize);
        ALB_CK(cudaGetLastError());
        ALB_TRY(exclusive_scan(ssize, m->slice_off, m->nslices, st));
        ALB_CK(cudaMemcpyAsync(&m->stored, m->slice_off + m->nslices, sizeof(int64_t),
                               cudaMemcpyDeviceToHost, st));
        ALB_CK(cudaStreamSynchronize(st));
        ALB_TRY(dmalloc((void **)&m->col, sizeof(int32_t) * (size_t)(m->stored > 0 ? m->stored : 4),
                        "SpMV SELL columns"));
        ALB_TRY(dmalloc((void **)&m->val, sizeof(double) * (size_t)(m->stored > 0 ? m->stored : 4),
                        "SpMV SELL values"));
        k_sp_fill<<<blocks_for(npad, 256), 256, 0, st>>>(n, npad, m->perm, m->deg, m->slice_off,
                                                          d_rp, d_col, d_val, m->col, m->val);
        ALB_CK(cudaGetLastError());
        // long rows: list (longest first, ordered on the host: a few
        // thousand ids), offsets, entries
        int64_t *idx = nullptr;
        ALB_TRY(dmalloc((void **)&idx, sizeof(int64_t) * (size_t)(n + 1), "SpMV long index"));
        struct Free {
            int64_t *p;
            ~Free() { dfree(p); }
        } free_idx{idx};
        int32_t *flags = nullptr;
        ALB_TRY(dmalloc((void **)&flags, sizeof(int32_t) * (size_t)n, "SpMV long flags"));
        struct Free32 {
            int32_t *p;
            ~Free32() { dfree(p); }
        } free_flags{flags};
        k_sp_long_flags<<<blocks_for(n, 256), 256, 0, st>>>(n, len, flags);
        ALB_CK(cudaGetLastError());
        ALB_TRY(exclusive_scan(flags, idx, n, st));
        ALB_CK(cudaMemcpyAsync(&m->nlong, idx + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        ALB_CK(cudaStreamSynchronize(st));
        if (m->nlong > 0) {
            const int64_t nl = m->nlong;
            ALB_TRY(dmalloc((void **)&m->lrow, sizeof(int32_t) * (size_t)nl, "SpMV long rows"));
            ALB_TRY(dmalloc((void **)&m->lptr, sizeof(int64_t) * (size_t)(nl + 1), "SpMV long offsets"));
            k_sp_long_scatter<<<blocks_for(n, 256), 256, 0, st>>>(n, flags, idx, m->lrow);
            ALB_CK(cudaGetLastError());
            std::vector<int32_t> hrow((size_t)nl);
            ALB_CK(cudaMemcpyAsync(hrow.data(), m->lrow, sizeof(int32_t) * (size_t)nl,
                                   cudaMemcpyDeviceToHost, st));
            ALB_CK(cudaStreamSynchronize(st));
            std::vector<int64_t> hlen((size_t)nl);
            for (int64_t i = 0; i < nl; i++) hlen[(size_t)i] = rowptr[hrow[(size_t)i] + 1] - rowptr[hrow[(size_t)i]];
            std::vector<int64_t> order((size_t)nl);
            for (int64_t i = 0; i < nl; i++) order[(size_t)i] = i;
            std::stable_sort(order.begin(), order.end(),
                             [&](int64_t x, int64_t y) { return hlen[(size_t)x] > hlen[(size_t)y]; });
            std::vector<int32_t> srow((size_t)nl), slen((size_t)nl);
            std::vector<int64_t> sptr((size_t)nl + 1, 0);
            for (int64_t i = 0; i < nl; i++) {
                const int64_t len = hlen[(size_t)order[(size_t)i]];
                srow[(size_t)i] = hrow[(size_t)order[(size_t)i]];
                slen[(size_t)i] = (int32_t)len;
                sptr[(size_t)i + 1] = sptr[(size_t)i] + ((len + kLb - 1) / kLb) * kLb;
            }
            m->max_long = slen[0];
            ALB_TRY(dmalloc((void **)&m->llen, sizeof(int32_t) * (size_t)nl, "SpMV long lengths"));
            ALB_CK(cudaMemcpyAsync(m->lrow, srow.data(), sizeof(int32_t) * (size_t)nl,
                                   cudaMemcpyHostToDevice, st));
            ALB_CK(cudaMemcpyAsync(m->llen, slen.data(), sizeof(int32_t) * (size_t)nl,
                                   cudaMemcpyHostToDevice, st));
            ALB_CK(cudaMemcpyAsync(m->lptr, sptr.data(), sizeof(int64_t) * (size_t)(nl + 1),
                                   cudaMemcpyHostToDevice, st));
            // padded entries are never summed; zeroed so that the layout is
            // fixed by the CSR alone
            const int64_t nent = sptr[(size_t)nl];
            ALB_TRY(dmalloc((void **)&m->lcol, sizeof(int32_t) * (size_t)nent, "SpMV long columns"));
            ALB_TRY(dmalloc((void **)&m->lval, sizeof(double) * (size_t)nent, "SpMV long values"));
            ALB_CK(cudaMemsetAsync(m->lcol, 0, sizeof(int32_t) * (size_t)nent, st));
            ALB_CK(cudaMemsetAsync(m->lval, 0, sizeof(double) * (size_t)nent, st));
            k_sp_long_fill<<<blocks_for(nl * 32, 256), 256, 0, st>>>(
                nl, m->lrow, m->lptr, m->llen, d_rp, d_col, d_val, m->lcol, m->lval);
            ALB_CK(cudaGetLastError());
            // the host vectors must outlive the copies
            ALB_CK(cudaStreamSynchronize(st));
        }
        ALB_CK(cudaStreamSynchronize(st));
        return ALB_OK;
    }();
    tmp_free();
    return rc;
}

void destroy(alb_sellmat *m) {
    if (!m) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    dfree(m->perm);
    dfree(m->deg);
    dfree(m->slice_off);
    dfree(m->col);
    dfree(m->val);
    dfree(m->dx);
    dfree(m->dy);
    dfree(m->lrow);
    dfree(m->lptr);
    dfree(m->lcol);
    dfree(m->lval);
    dfree(m->llen);
    if (m->side) cudaStreamSynchronize(m->side);
    if (m->ev0) cudaEventDestroy(m->ev0);
    if (m->ev1) cudaEventDestroy(m->ev1);
    if (m->fork) cudaEventDestroy(m->fork);
    if (m->join) cudaEventDestroy(m->join);
    if (m->stream) cudaStreamDestroy(m->stream);
    if (m->side) cudaStreamDestroy(m->side);
    cudaGetLastError();
    if (prev >= 0) cudaSetDevice(prev);
    delete m;
}

alb_status launch(alb_sellmat *m, const double *d_x, double *d_y, float *us) {
    int per = 0, sms = 0;
    ALB_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_spmv, kSpBlock, 0));
    ALB_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device));
    const int64_t want = (m->nslices + 15) / 16;  // 16 warps a block, one slice each
    const int64_t cap = (int64_t)(per > 0 ? per : 2) * sms;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min(want, cap));
    if (us) ALB_CK(cudaEventRecord(m->ev0, m->stream));
    // the long rows' chains (one dependent fma per entry, the longest row
    // the critical path) start first, and the slices run beside them
    if (m->nlong > 0) {
        ALB_CK(cudaEventRecord(m->fork, m->stream));
        ALB_CK(cudaStreamWaitEvent(m->side, m->fork, 0));
        // the few longest rows on CTAs of their own (side stream); the other
        // long rows, then the slices, on the main stream beside them
        const int64_t nsolo = std::min<int64_t>(m->nlong, kSoloRows);
        k_spmv_long<true><<<(unsigned)nsolo, kSoloThreads, 0, m->side>>>(
            m->nlong, 0, m->lrow, m->lptr, m->llen, m->lcol, m->lval, d_x, d_y);
        ALB_CK(cudaGetLastError());
        ALB_CK(cudaEventRecord(m->join, m->side));
        if (m->nlong > nsolo)
            k_spmv_long<false><<<blocks_for(m->nlong - nsolo, 32), kSpLongBlock, 0, m->stream>>>(
                m->nlong, nsolo, m->lrow, m->lptr, m->llen, m->lcol, m->lval, d_x, d_y);
    }
    k_spmv<<<grid, kSpBlock, 0, m->stream>>>(m->n, m->nslices, m->perm, m->deg, m->slice_off, m->col,
                                         m->val, d_x, d_y);
    ALB_CK(cudaGetLastError());
    if (m->nlong > 0) ALB_CK(cudaStreamWaitEvent(m->stream, m->join, 0));
    if (us) {
        ALB_CK(cudaEventRecord(m->ev1, m->stream));
        ALB_CK(cudaEventSynchronize(m->ev1));
        float ms = 0;
        ALB_CK(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
        *us = ms * 1000.0f;
    }
    return ALB_OK;
}

}  // namespace
}  // namespace alb

using namespace alb;

extern "C" {

alb_status alb_sellmat_create(int64_t n, const int64_t *rowptr, const int32_t *col,
                              const double *values, int32_t sigma, alb_sellmat **out) {
    if (!out) return fail(ALB_ERR_INVALID, "alb_sellmat_create: out is NULL");
    *out = nullptr;
    if (n <= 0 || n > INT32_MAX || !rowptr || rowptr[0] != 0 || rowptr[n] < 0 ||
        (rowptr[n] > 0 && (!col || !values)))
        return fail(ALB_ERR_INVALID, "alb_sellmat_create: bad arguments");
    if (sigma < 1 || sigma > 16384)
        return fail(ALB_ERR_UNSUPPORTED, "alb_sellmat_create: sigma %d outside 1..16384", sigma);
    alb_sellmat *m = new alb_sellmat();
    m->n = n;
    m->nnz = rowptr[n];
    m->sigma = sigma;
    cudaError_t e = cudaGetDevice(&m->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&m->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&m->ev1);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaGetLastError();
        destroy(m);
        return fail(ALB_ERR_CUDA, "alb_sellmat_create: %s", cudaGetErrorString(e));
    }
    alb_status rc = build(m, rowptr, col, values);
    if (rc != ALB_OK) {
        destroy(m);
        return rc;
    }
    *out = m;
    return ALB_OK;
}

void alb_sellmat_destroy(alb_sellmat *m) { destroy(m); }

alb_status alb_sellmat_info(const alb_sellmat *m, int64_t *n, int64_t *nnz, int64_t *stored) {
    if (!m) return fail(ALB_ERR_INVALID, "alb_sellmat_info: matrix is NULL");
    if (n) *n = m->n;
    if (nnz) *nnz = m->nnz;
    if (stored) *stored = m->stored;
    return ALB_OK;
}

alb_status alb_sellmat_spmv(alb_sellmat *m, const double *d_x, double *d_y, float *kernel_us) {
    if (!m || !d_x || !d_y) return fail(ALB_ERR_INVALID, "alb_sellmat_spmv: bad arguments");
    ALB_CK(cudaSetDevice(m->device));
    ALB_TRY(launch(m, d_x, d_y, kernel_us));
    ALB_CK(cudaStreamSynchronize(m->stream));
    return ALB_OK;
}

alb_status alb_sellmat_spmv_host(alb_sellmat *m, const double *x, double *y) {
    if (!m || !x || !y) return fail(ALB_ERR_INVALID, "alb_sellmat_spmv_host: bad arguments");
    ALB_CK(cudaSetDevice(m->device));
    if (!m->dx) ALB_TRY(dmalloc((void **)&m->dx, sizeof(double) * (size_t)m->n, "SpMV x"));
    if (!m->dy) ALB_TRY(dmalloc((void **)&m->dy, sizeof(double) * (size_t)m->n, "SpMV y"));
    ALB_CK(cudaMemcpyAsync(m->dx, x, sizeof(double) * (size_t)m->n, cudaMemcpyHostToDevice,
                           m->stream));
    ALB_TRY(launch(m, m->dx, m->dy, nullptr));
    ALB_CK(cudaMemcpyAsync(y, m->dy, sizeof(double) * (size_t)m->n, cudaMemcpyDeviceToHost,
                           m->stream));
    ALB_CK(cudaStreamSynchronize(m->stream));
    return ALB_OK;
}

}  // extern "C"
