// Single-root direction-optimising BFS over SELL-C-sigma (position space).
//
// Reference: the level loop of run_custom_bfs_test (bfs/src/bfs_SELLCSv2.c:
// 296-762) with its pull kernel (bfs/src/bfs_par_kernels.c:128-198), its
// sparse-frontier kernel (:566-656) and the frontier representation changes
// (:696-797). GB300 design:
//
//  * bottom-up pull (k_bu): one warp per 32-row bitmap word. The visited word
//    is the slice bypass test (a full word is skipped), each unvisited lane
//    walks its row with 16-byte int4 loads, tests frontier bits, and stops at
//    the first hit (the smallest original id, rows being ascending) or at the
//    padding (its own position). __ballot_sync drops the warp out as soon as
//    no lane is active, and one ballot writes the next-frontier word: no
//    atomics on the pull side.
//  * top-down push (k_td): warp-cooperative over the frontier queue; the 32
//    rows a warp holds are flattened by a warp prefix sum so every lane
//    processes one edge per step regardless of degree skew. Unvisited targets
//    get atomicMin(parent) (so the parent is the smallest original id) and an
//    atomicOr claim on the next-frontier word; claimers append to the next
//    queue with one atomicAdd per warp.
//  * bitmap -> queue compaction (k_prep): ballot/popc warp prefix sums.
//  * the level loop runs host-driven, as a CUDA graph whose while node is
//    driven by a device-side decision, or as one persistent cooperative
//    kernel with a bounded grid barrier.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "graph.h"
#include "selector.cuh"

namespace alb {

constexpr int kMaxBlock = 1024;
constexpr uint64_t kBarrierTimeoutNs = 4ull * 1000 * 1000 * 1000;
constexpr unsigned long long kBarFailed = 1ull << 62;  // grid barrier gave up (bit 62 of bar)

// Loads of bitmaps/queues: .nc is safe in standalone kernels (the data was
// written by an earlier launch); the persistent kernel needs ordinary loads.
template <bool kPersist, class T>
__device__ __forceinline__ T ld_state(const T *p) {
    if constexpr (kPersist)
        return *(const volatile T *)p;
    else
        return __ldg(p);
}
template <bool kPersist>
__device__ __forceinline__ uint32_t ld_bits(const uint32_t *p) {
    if constexpr (kPersist)
        return __ldcg(p);
    else
        return __ldg(p);
}

struct Range {
    int bid, nblk;
};

// ------------------------------------------------------------ level phases

// Decision (one warp). forced >= 0 overrides the policy (host-driven loop).
// P: the network's parameters (a.mlp, or a shared-memory copy of them).
__device__ int decide_warp(const BfsArgs &a, const BfsCtl &c, int forced,
                           const float *P = nullptr) {
    int dir;
    if (forced >= 0) {
        dir = forced;
    } else if (c.policy == ALB_POLICY_LEARNED && a.mlp && a.mlp[kMlpParams] != 0.0f) {
        float f[kMlpIn];
        level_features(c, f);
        dir = mlp_select_warp(P ? P : a.mlp, f);
    } else {
        dir = rule_dir(c);
    }
    return dir;
}

__device__ void record_trace(const BfsArgs &a, const BfsCtl &c, int dir) {
    if (a.trace && c.level < c.trace_cap) {
        alb_level_rec r;
        r.dir = dir;
        r.level = c.level;
        r.nf = c.nf;
        r.mf = c.mf;
        r.nu = c.nu;
        r.mu = c.mu;
        r.active_slices = c.active_words;
        r.t_ns = (int64_t)globaltimer_ns();
        r.bytes = 0;
        r.step_us = -1.0f;
        r.pad_ = 0;
        r.words_bypassed = r.rows_scanned = r.groups_read = r.groups_bypassed = 0;
        r.edges_bypassed = 0;
        a.trace[c.level] = r;
    }
}

// F -> queue compaction and/or clearing of the next bitmap.
template <bool kPersist>
__device__ void prep_phase(const BfsArgs &a, int L, bool compact, bool zero_next, Range r) {
    const uint32_t *F = (L & 1) ? a.bm1 : a.bm0;
    uint32_t *N = (L & 1) ? a.bm0 : a.bm1;
    int32_t *Q = (L & 1) ? a.q1 : a.q0;
    unsigned long long *slot = &a.ctl->qn[L % 3];
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t gw = (int64_t)r.bid * wpb + (threadIdx.x >> 5);
    const int64_t stride = (int64_t)r.nblk * wpb * 32;
    for (int64_t wb = gw * 32; wb < a.nwords; wb += stride) {
        const int64_t w = wb + lane;
        uint32_t word = 0;
        if (w < a.nwords) {
            if (compact) word = ld_bits<kPersist>(F + w);
            if (zero_next) N[w] = 0;
        }
        if (!compact) continue;
        const int cnt = __popc(word);
        const int inc = warp_inclusive_scan(cnt);
        const int tot = __shfl_sync(kFull, inc, 31);
        unsigned long long base = 0;
        if (lane == 31 && tot) base = atomicAdd(slot, (unsigned long long)tot);
        base = __shfl_sync(kFull, base, 31);
        int64_t pos = (int64_t)base + inc - cnt;
        while (word) {
            int b = __ffs(word) - 1;
            word &= word - 1;
            if (ALB_CHECK_POS(pos, a.n, &a.ctl->err)) Q[pos] = (int32_t)(w * 32 + b);
            pos++;
        }
    }
}

// Adds a warp's count of bypass statistic `which` to level L's slot (all 32
// lanes call it).
__device__ __forceinline__ void add_stat(const BfsArgs &a, int L, int which, unsigned long long v) {
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&a.ctl->acc_stat[(L + 1) % 3][which], v);
}

// Pushed edges u -> v (u's original id ou): the smallest source wins the
// parent, and v's bit goes into the next-frontier bitmap N. The next queue,
// levels and counters are made from N by td_finish_phase (no counter shared
// by every claim) -- or, in append mode (a small frontier, where scanning all
// of N would cost more than the level), the claimer of v (the push whose
// atomicOr set v's bit) records v for the next queue.
// Four edges per lane (v[k] < 0: none): the visited words of all four are
// requested together, then the parent and bitmap words of the unvisited
// targets together, then the atomics, so one lane keeps four loads in
// flight where one edge at a time kept one.
__device__ __forceinline__ void push_edges4(const BfsArgs &a, uint32_t *N, const int32_t (&v)[4],
                                            const uint32_t (&ou)[4], bool persist,
                                            unsigned &bypassed, bool append, unsigned &claimed) {
    bool live[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        live[k] = false;
        if (v[k] >= 0) {
            const uint32_t w = persist ? __ldcg(a.vis + (v[k] >> 5)) : __ldg(a.vis + (v[k] >> 5));
            live[k] = !((w >> (v[k] & 31)) & 1u);
            bypassed += !live[k];
        }
    }
    // read before writing: a hub target receives thousands of pushes in one
    // level, and atomics on one address serialise in L2, so the atomics are
    // issued only when they can still change something
    uint32_t cur_parent[4], cur_n[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        cur_parent[k] = 0;
        cur_n[k] = ~0u;
        if (live[k]) {
            cur_parent[k] = __ldcg(a.parent_pos + v[k]);
            cur_n[k] = __ldcg(N + (v[k] >> 5));
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (!live[k]) continue;
        const uint32_t bit = 1u << (v[k] & 31);
        if (ou[k] < cur_parent[k]) atomicMin(a.parent_pos + v[k], ou[k]);
        if (!(cur_n[k] & bit)) {
            const uint32_t old = atomicOr(N + (v[k] >> 5), bit);
            if (append && !(old & bit)) claimed |= 1u << k;
        }
    }
}

// Lazy push (persistent loop, small frontiers): a target counts as visited
// when its level was set before this level (level_pos <= L), and the push
// that claims an unvisited target is the one whose atomicCAS moves its level
// from -1 to L + 1. Parents still meet by atomicMin over every source one
// level up. Neither the visited nor the frontier bitmaps are touched: a level
// that needs them rebuilds them from the levels first (materialize_phase),
// so a run of such levels costs one grid barrier each. The CAS is issued at
// once, together with the parent read (one round trip): a CAS that finds a
// level set changes nothing, and its old value tells a target claimed this
// level (L + 1: still a parent candidate) from one visited before.
__device__ __forceinline__ void push_edges4_lazy(const BfsArgs &a, int L, const int32_t (&v)[4],
                                                 const uint32_t (&ou)[4], unsigned &bypassed,
                                                 unsigned &claimed) {
    int32_t old[4];
    uint32_t cur_parent[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        old[k] = v[k] >= 0 ? atomicCAS(a.level_pos + v[k], -1, L + 1) : 0;
        cur_parent[k] = v[k] >= 0 ? __ldcg(a.parent_pos + v[k]) : 0u;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const bool live = v[k] >= 0 && (old[k] == -1 || old[k] == L + 1);
        bypassed += v[k] >= 0 && !live;
        if (!live) continue;
        if (ou[k] < cur_parent[k]) atomicMin(a.parent_pos + v[k], ou[k]);
        if (old[k] == -1) claimed |= 1u << k;
    }
}

// Appends the warp's claimed targets (bit k of claimed: v[k], one lane's
// four edges of push_edges4) to the next queue, one atomicAdd per warp. Call
// from all lanes of a warp.
__device__ __forceinline__ void flush_claims(const BfsArgs &a, int32_t *NQ,
                                             unsigned long long *nq_slot, const int32_t (&v)[4],
                                             unsigned &claimed) {
    const int lane = threadIdx.x & 31;
    const int cnt = __popc(claimed);
    const int inc = warp_inclusive_scan(cnt);
    const int tot = __shfl_sync(kFull, inc, 31);
    if (tot) {
        unsigned long long base = 0;
        if (lane == 31) base = atomicAdd(nq_slot, (unsigned long long)tot);
        base = __shfl_sync(kFull, base, 31);
        int64_t pos = (int64_t)base + inc - cnt;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (!((claimed >> k) & 1u)) continue;
            if (ALB_CHECK_POS(pos, a.n, &a.ctl->err)) NQ[pos] = v[k];
            pos++;
        }
    }
    claimed = 0;
}

// Counters of a lazy level, kept by the claimers (no finish pass counts them).
struct LazyCounts {
    unsigned n = 0;
    unsigned long long mo = 0, mi = 0;
    int32_t od[4], id[4];
    // the claimed targets' degrees, requested before the queue append so
    // that both round trips overlap; add() uses them after it
    __device__ __forceinline__ void load(const BfsArgs &a, const int32_t (&v)[4], unsigned claimed) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const bool c = (claimed >> k) & 1u;
            od[k] = c ? __ldg(a.odeg + v[k]) : 0;
            id[k] = c ? __ldg(a.ideg + v[k]) : 0;
        }
    }
    __device__ __forceinline__ void add(unsigned claimed) {
        n += __popc(claimed);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            mo += (unsigned long long)od[k];
            mi += (unsigned long long)id[k];
        }
    }
    __device__ __forceinline__ void flush(const BfsArgs &a, int L) {
        const unsigned cn = warp_sum(n);
        const unsigned long long cmo = warp_sum(mo), cmi = warp_sum(mi);
        if ((threadIdx.x & 31) == 0 && cn) {
            const int k = (L + 1) % 3;
            atomicAdd(&a.ctl->acc_n[k], (unsigned long long)cn);
            atomicAdd(&a.ctl->acc_mo[k], cmo);
            atomicAdd(&a.ctl->acc_mi[k], cmi);
        }
    }
};

// Append mode for a top-down level: the frontier's push edges are no more
// than the bitmap's words, so the next queue is built by the claims rather
// than by scanning the whole next-frontier bitmap.
__device__ __forceinline__ bool td_append(const BfsArgs &a, int64_t mf) { return mf <= a.nwords; }

// Rows per warp for the short-row pass (a power of two up to 32): at least
// as many as spread the frontier over the warps available, and, when the
// frontier is small, as many as fill about one 128-edge step at the mean push
// degree -- the latency per warp is the same either way, and fewer warps
// means fewer appends and counter atomics on the level's shared words (each
// warp's land on the same few addresses, where L2 serialises them).
__device__ __forceinline__ int rows_per_warp(int64_t qlen, int64_t mf, int64_t nwarps) {
    const int64_t mean = qlen > 0 ? max((int64_t)1, mf / qlen) : 1;
    const int64_t per_warp = max((int64_t)128, mf / max(nwarps, (int64_t)1));
    int G = 1;
    while (G < 32 && ((int64_t)G * nwarps < qlen || (int64_t)(2 * G) * mean <= per_warp)) G <<= 1;
    return G;
}

// Big-row counter: entry count in the top 26 bits, chunk total in the low 38.
// One atomicAdd of (1 << 38 | chunks) gives a row its index and chunk base
// together, so chunk bases grow with the index and can be binary-searched.
constexpr int kBigShift = 38;
constexpr unsigned long long kBigMask = (1ull << kBigShift) - 1;

// qknown >= 0: the queue's length, already read by the caller.
template <bool kPersist>
__device__ void td_phase(const BfsArgs &a, int L, Range r, int64_t mf, bool append,
                         bool lazy = false, int64_t qknown = -1) {
    LazyCounts lc;
    const int32_t *Q = (L & 1) ? a.q1 : a.q0;
    int32_t *NQ = (L & 1) ? a.q0 : a.q1;
    unsigned long long *nq_slot = &a.ctl->qn[(L + 1) % 3];
    unsigned claimed = 0;
    uint32_t *N = (L & 1) ? a.bm0 : a.bm1;
    const int64_t qlen = qknown >= 0 ? qknown : (int64_t)ld_state<kPersist>(&a.ctl->qn[L % 3]);
    unsigned long long *big_slot = &a.ctl->nbig[L % 3];
    __shared__ int64_t s_ex[kMaxBlock / 32][32];
    __shared__ int64_t s_st[kMaxBlock / 32][32];
    __shared__ int32_t s_ou[kMaxBlock / 32][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t gw = (int64_t)r.bid * wpb + wib;
    const int64_t nwarps = (int64_t)r.nblk * wpb;
    const int G = rows_per_warp(qlen, mf, nwarps);
    const int64_t stride = nwarps * G;
    unsigned bypassed = 0;
    for (int64_t cb = gw * G; cb < qlen; cb += stride) {
        const int64_t i = cb + lane;
        int32_t u = (lane < G && i < qlen) ? ld_state<kPersist>(Q + i) : -1;
        if (u >= 0) ALB_CHECK_ID(u, a.n, -1, &a.ctl->err);
        int64_t st = 0, d = 0;
        int32_t ou = 0;
        if (u >= 0) {
            st = __ldg(a.prow + u);
            d = __ldg(a.prow + u + 1) - st;
            ou = __ldg(a.perm + u);
            if (d > kBigRow) {  // pushed in chunks by all warps in td_big_phase
                const unsigned long long nch = (unsigned long long)((d + kBigChunk - 1) / kBigChunk);
                const unsigned long long old = atomicAdd(big_slot, (1ull << kBigShift) | nch);
                const int64_t idx = (int64_t)(old >> kBigShift);
                a.big[idx] = u;
                a.big_base[idx] = (int64_t)(old & kBigMask);
                d = 0;
            }
        }
        const int64_t inc = warp_inclusive_scan(d);
        const int64_t T = __shfl_sync(kFull, inc, 31);
        s_ex[wib][lane] = inc - d;
        s_st[wib][lane] = st;
        s_ou[wib][lane] = ou;
        __syncwarp();
        // the loop bound is warp-uniform (lanes past T carry no edge) so that
        // append mode can flush its claims with warp collectives
        for (int64_t eb = 0; eb < T; eb += 128) {
            const int64_t e0 = eb + lane;
            int32_t v[4];
            uint32_t ou4[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int64_t e = e0 + 32 * k;
                v[k] = -1;
                ou4[k] = 0;
                if (e < T) {
                    int j = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1)
                        if (s_ex[wib][j + step] <= e) j += step;
                    v[k] = __ldg(a.pcol + s_st[wib][j] + (e - s_ex[wib][j]));
                    ALB_CHECK_ID(v[k], a.n, -1, &a.ctl->err);
                    ou4[k] = (uint32_t)s_ou[wib][j];
                }
            }
            if (lazy) {
                push_edges4_lazy(a, L, v, ou4, bypassed, claimed);
                const unsigned cl = claimed;
                lc.load(a, v, cl);
                flush_claims(a, NQ, nq_slot, v, claimed);
                lc.add(cl);
            } else {
                push_edges4(a, N, v, ou4, kPersist, bypassed, append, claimed);
                if (append) flush_claims(a, NQ, nq_slot, v, claimed);
            }
        }
        __syncwarp();
    }
    // the level's counters and the bypass statistic, combined in the block
    // first: one atomic per block and counter instead of one per warp (each
    // warp's would land on the same few words, where L2 serialises them)
    __shared__ unsigned long long s_c[4];
    if (threadIdx.x < 4) s_c[threadIdx.x] = 0;
    __syncthreads();
    const unsigned long long cn = warp_sum((unsigned long long)lc.n), cmo = warp_sum(lc.mo),
                             cmi = warp_sum(lc.mi), cb = warp_sum((unsigned long long)bypassed);
    if ((threadIdx.x & 31) == 0) {
        if (cn) atomicAdd(&s_c[0], cn);
        if (cmo) atomicAdd(&s_c[1], cmo);
        if (cmi) atomicAdd(&s_c[2], cmi);
        if (cb) atomicAdd(&s_c[3], cb);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int k = (L + 1) % 3;
        if (s_c[0]) {
            atomicAdd(&a.ctl->acc_n[k], s_c[0]);
            atomicAdd(&a.ctl->acc_mo[k], s_c[1]);
            atomicAdd(&a.ctl->acc_mi[k], s_c[2]);
        }
        if (s_c[3]) atomicAdd(&a.ctl->acc_stat[k][kStEdgesBypassed], s_c[3]);
    }
}

// Long frontier rows, kBigChunk edges per chunk, chunks spread over all
// warps. Each warp takes a contiguous run of chunks: it finds the row of its
// first chunk by binary search over the chunk bases (monotone in the list
// index) and walks forward from there.
template <bool kPersist>
__device__ void td_big_phase(const BfsArgs &a, int L, Range r, bool append, bool lazy = false) {
    const unsigned long long ctr = ld_state<kPersist>(&a.ctl->nbig[L % 3]);
    if (ctr == 0) return;
    const int64_t nbig = (int64_t)(ctr >> kBigShift);
    const int64_t total = (int64_t)(ctr & kBigMask);
    uint32_t *N = (L & 1) ? a.bm0 : a.bm1;
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t gw = (int64_t)r.bid * wpb + (threadIdx.x >> 5);
    const int64_t nwarps = (int64_t)r.nblk * wpb;
    const int64_t per = (total + nwarps - 1) / nwarps;
    const int64_t k0 = gw * per, k1 = min(total, k0 + per);
    unsigned bypassed = 0;
    int32_t *NQ = (L & 1) ? a.q0 : a.q1;
    unsigned long long *nq_slot = &a.ctl->qn[(L + 1) % 3];
    unsigned claimed = 0;
    LazyCounts lc;
    if (k0 >= k1) {
        add_stat(a, L, kStEdgesBypassed, bypassed);  // keeps every lane at the shuffle
        return;
    }
    int64_t lo = 0, hi = nbig - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (ld_state<kPersist>(a.big_base + mid) <= k0) lo = mid;
        else hi = mid - 1;
    }
    int64_t base = ld_state<kPersist>(a.big_base + lo);
    int64_t next = lo + 1 < nbig ? ld_state<kPersist>(a.big_base + lo + 1) : total;
    int32_t u = ld_state<kPersist>(a.big + lo);
    int64_t st = __ldg(a.prow + u), d = __ldg(a.prow + u + 1) - st;
    uint32_t ou = (uint32_t)__ldg(a.perm + u);
    for (int64_t k = k0; k < k1; k++) {
        while (k >= next) {  // the run crosses into the next long row
            lo++;
            base = next;
            next = lo + 1 < nbig ? ld_state<kPersist>(a.big_base + lo + 1) : total;
            u = ld_state<kPersist>(a.big + lo);
            st = __ldg(a.prow + u);
            d = __ldg(a.prow + u + 1) - st;
            ou = (uint32_t)__ldg(a.perm + u);
        }
        const int64_t c = k - base;
        const int64_t e1 = min(d, (c + 1) * kBigChunk);
        static_assert(kBigChunk == 128, "four edges per lane per chunk");
        int32_t v[4];
        uint32_t ou4[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int64_t e = c * kBigChunk + 32 * q + lane;
            v[q] = e < e1 ? __ldg(a.pcol + st + e) : -1;
            if (v[q] >= 0) ALB_CHECK_ID(v[q], a.n, -1, &a.ctl->err);
            ou4[q] = ou;
        }
        if (lazy) {
            push_edges4_lazy(a, L, v, ou4, bypassed, claimed);
            const unsigned cl = claimed;
            lc.load(a, v, cl);
            flush_claims(a, NQ, nq_slot, v, claimed);
            lc.add(cl);
        } else {
            push_edges4(a, N, v, ou4, kPersist, bypassed, append, claimed);
            if (append) flush_claims(a, NQ, nq_slot, v, claimed);
        }
    }
    if (lazy) lc.flush(a, L);
    add_stat(a, L, kStEdgesBypassed, bypassed);
}

// After a top-down level: clear the old frontier over its queue; compact the
// new frontier bitmap N into the next queue (thread per word, prefix sums in
// the warp, one atomic per warp), recording levels and counters and marking
// the new vertices visited (each word by the one thread that owns it).
template <bool kPersist>
__device__ void td_finish_phase(const BfsArgs &a, int L, Range r, bool append) {
    const int32_t *Q = (L & 1) ? a.q1 : a.q0;
    int32_t *NQ = (L & 1) ? a.q0 : a.q1;
    uint32_t *F = (L & 1) ? a.bm1 : a.bm0;
    const uint32_t *N = (L & 1) ? a.bm0 : a.bm1;
    const int64_t qlen = (int64_t)ld_state<kPersist>(&a.ctl->qn[L % 3]);
    unsigned long long *nq_slot = &a.ctl->qn[(L + 1) % 3];
    const int lane = threadIdx.x & 31;
    const int64_t tid = (int64_t)r.bid * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)r.nblk * blockDim.x;
    for (int64_t i = tid; i < qlen; i += nth) F[ld_state<kPersist>(Q + i) >> 5] = 0;
    const int32_t lvl = L + 1;
    unsigned cn = 0, full = 0;
    unsigned long long cmo = 0, cmi = 0;
    if (append) {  // the claims built the next queue: walk it
        const int64_t nq = (int64_t)ld_state<kPersist>(nq_slot);
        for (int64_t i = tid; i < nq; i += nth) {
            const int32_t v = ld_state<kPersist>(NQ + i);
            const uint32_t bit = 1u << (v & 31);
            const uint32_t old = atomicOr(a.vis + (v >> 5), bit);
            full += (old != kFull && (old | bit) == kFull);
            a.level_pos[v] = lvl;
            cn++;
            cmo += (unsigned long long)__ldg(a.odeg + v);
            cmi += (unsigned long long)__ldg(a.ideg + v);
        }
    }
    // the loop bound is warp-uniform so that every lane reaches the shuffles
    for (int64_t w0 = append ? a.nwords : (tid & ~31ll); w0 < a.nwords; w0 += nth) {
        const int64_t w = w0 + lane;
        uint32_t m = w < a.nwords ? ld_bits<kPersist>(N + w) : 0u;
        const int cnt = __popc(m);
        const int inc = warp_inclusive_scan(cnt);
        const int tot = __shfl_sync(kFull, inc, 31);
        if (tot == 0) continue;
        unsigned long long base = 0;
        if (lane == 31) base = atomicAdd(nq_slot, (unsigned long long)tot);
        base = __shfl_sync(kFull, base, 31);
        if (m) {
            const uint32_t old = ld_bits<kPersist>(a.vis + w);
            a.vis[w] = old | m;
            full += (old != kFull && (old | m) == kFull);
        }
        int64_t pos = (int64_t)base + inc - cnt;
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            const int32_t v = (int32_t)(w * 32 + b);
            if (ALB_CHECK_POS(pos, a.n, &a.ctl->err)) NQ[pos] = v;
            pos++;
            a.level_pos[v] = lvl;
            cn++;
            cmo += (unsigned long long)__ldg(a.odeg + v);
            cmi += (unsigned long long)__ldg(a.ideg + v);
        }
    }
    cn = warp_sum(cn);
    full = warp_sum(full);
    cmo = warp_sum(cmo);
    cmi = warp_sum(cmi);
    if (lane == 0 && (cn || full)) {
        const int k = (L + 1) % 3;
        if (cn) {
            atomicAdd(&a.ctl->acc_n[k], (unsigned long long)cn);
            atomicAdd(&a.ctl->acc_mo[k], cmo);
            atomicAdd(&a.ctl->acc_mi[k], cmi);
        }
        if (full) atomicAdd(&a.ctl->acc_full[k], (unsigned long long)full);
    }
}

// Rebuilds the bitmaps after a run of lazy levels (see push_edges4_lazy):
// visited = the initial mask | every position with a level, frontier (of
// level L) = the positions at level L, next frontier cleared; the words with
// an unvisited row are counted into acc_active[L % 3]. A warp takes 32 words
// (1024 positions) at a time: lane l loads position 32k + l of word k for
// every k before any ballot, so 32 loads per lane are in flight together,
// and lane k then writes word k (coalesced stores).
__device__ void materialize_phase(const BfsArgs &a, int L, Range r) {
    uint32_t *F = (L & 1) ? a.bm1 : a.bm0;
    uint32_t *N = (L & 1) ? a.bm0 : a.bm1;
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t gw = (int64_t)r.bid * wpb + (threadIdx.x >> 5);
    const int64_t nwarps = (int64_t)r.nblk * wpb;
    unsigned active = 0;
    for (int64_t w0 = gw * 32; w0 < a.nwords; w0 += nwarps * 32) {
        int32_t lp[32];
#pragma unroll
        for (int k = 0; k < 32; k++) {
            const int64_t p = (w0 + k) * 32 + lane;
            lp[k] = p < a.n ? __ldcg(a.level_pos + p) : -1;
        }
        uint32_t vb = 0, fb = 0;
#pragma unroll
        for (int k = 0; k < 32; k++) {
            const uint32_t v = __ballot_sync(kFull, lp[k] >= 0);
            const uint32_t f = __ballot_sync(kFull, lp[k] == L);
            if (lane == k) {
                vb = v;
                fb = f;
            }
        }
        const int64_t w = w0 + lane;
        if (w < a.nwords) {
            const uint32_t vis = __ldg(a.vinit + w) | vb;
            a.vis[w] = vis;
            F[w] = fb;
            N[w] = 0;
            active += vis != kFull;
        }
    }
    active = warp_sum(active);
    if (lane == 0 && active) atomicAdd(&a.ctl->acc_active[L % 3], (unsigned long long)active);
}

// Frontier word read by the bottom-up pull: from the staged shared-memory
// copy (kSmemF) or from global memory.
template <bool kSmemF, bool kPersist>
__device__ __forceinline__ uint32_t ld_front(const uint32_t *F, int32_t w) {
    if constexpr (kSmemF)
        return F[w];
    else
        return ld_bits<kPersist>(F + w);
}

// Bottom-up pull. kBypass: skip words whose rows are all visited.
// kEarly: stop each row at its first frontier source or its padding.
// Fs: where the frontier words are read (the global bitmap, or its copy in
// shared memory when kSmemF).
// Words per run of the bottom-up pull (a warp's unit of work from the
// level's counter): one visited word per lane.
constexpr int64_t kBuRun = 32;
constexpr int kBuWords = 2;  // words a warp scans at a time

template <bool kPersist, bool kBypass, bool kEarly, bool kSmemF = false>
__device__ void bu_phase(const BfsArgs &a, int L, Range r, const uint32_t *Fs = nullptr) {
    const uint32_t *F = kSmemF ? Fs : ((L & 1) ? a.bm1 : a.bm0);
    uint32_t *N = (L & 1) ? a.bm0 : a.bm1;
    const int lane = threadIdx.x & 31;
    (void)r;  // words are handed out by the level's counter, not by block index
    const int32_t C = a.C, log2C = a.log2C;
    const int32_t lvl = L + 1;
    unsigned cn = 0, full = 0;
    unsigned long long cmo = 0, cmi = 0, bytes = 0;
    unsigned n_wbyp = 0, n_rows = 0, n_grp = 0, n_gtot = 0;
    const uint64_t pol = l2_evict_first();
    constexpr int kW = kPersist ? 1 : kBuWords;
    // Words come in runs of kBuRun from the level's counter. Lane l holds the
    // visited mask of word l of the run (one coalesced load, the next run's
    // requested one run ahead; only the warp that takes a word writes its
    // mask during the level). With kBypass the run's fully visited words are
    // skipped together: their next-frontier words are cleared by one store
    // per lane and only the other words are walked, one at a time.
    unsigned long long *ctr = &a.ctl->work[L % 3];
    auto grab = [&]() {
        unsigned long long v = 0;
        if (lane == 0) v = atomicAdd(ctr, (unsigned long long)kBuRun);
        return (int64_t)__shfl_sync(kFull, v, 0);
    };
    auto run_vis = [&](int64_t rw) {
        return rw + lane < a.nwords ? ld_bits<kPersist>(a.vis + rw + lane) : kFull;
    };
    int64_t cur = grab(), nxt = grab();
    uint32_t vcur = run_vis(cur), vnxt = run_vis(nxt);
    while (cur < a.nwords) {
        unsigned todo;
        if (kBypass) {
            const bool valid = cur + lane < a.nwords;
            const bool full_w = valid && vcur == kFull;
            if (full_w) N[cur + lane] = 0;
            n_wbyp += full_w;
            todo = __ballot_sync(kFull, valid && !full_w);
        } else {
            todo = __ballot_sync(kFull, cur + lane < a.nwords);
        }
        const int64_t base_w = cur;
        const uint32_t vrun = vcur;
        cur = nxt;
        vcur = vnxt;
        if (cur < a.nwords) {
            nxt = grab();
            vnxt = run_vis(nxt);
        }
      // kW words at a time (kBuWords; one in the persistent kernel, whose
      // 80-register budget more would overflow): lane l scans row l of each,
      // their geometry, first column groups and frontier words requested
      // together, so that each lane keeps that many times the loads in flight
      // (a word costs a few dependent round trips whatever its rows' lengths).
      while (todo) {
        int qs[kW];
        int nr = 0;  // words taken (warp-uniform)
#pragma unroll
        for (int t = 0; t < kW; t++) {
            qs[t] = todo ? __ffs(todo) - 1 : qs[0];
            nr += todo != 0;
            todo &= todo - 1;
        }
        int64_t w[kW];
        uint32_t vis[kW];
        int32_t p[kW], ng[kW], found[kW];
        bool active[kW], long_cand[kW];
        const int4 *cp[kW];
        int4 c[kW];
#pragma unroll
        for (int t = 0; t < kW; t++) {
            w[t] = base_w + qs[t];
            vis[t] = __shfl_sync(kFull, vrun, qs[t]);
            p[t] = (int32_t)(w[t] * 32 + lane);
            found[t] = -1;
        }
        int32_t wd[kW];
        int64_t so[kW];
#pragma unroll
        for (int t = 0; t < kW; t++) {
            // rows past n are preset visited; clamp their slice index
            const int64_t sl = (int64_t)(p[t] < a.n ? p[t] : a.n - 1) >> log2C;
            wd[t] = t < nr ? __ldg(a.width + sl) : 0;
            so[t] = t < nr ? __ldg(a.slice_off + sl) : 0;
        }
#pragma unroll
        for (int t = 0; t < kW; t++) {
            active[t] = t < nr && !((vis[t] >> lane) & 1u);
            ng[t] = active[t] ? (wd[t] + 3) >> 2 : 0;
            n_rows += ng[t] > 0;
            n_gtot += ng[t];
            cp[t] = a.col4 + (so[t] >> 2) + (p[t] & (C - 1));
            // group j+1 is requested before group j's frontier tests, so each
            // lane keeps column loads in flight while it waits on the bitmap
            c[t] = make_int4(p[t], p[t], p[t], p[t]);
            if (active[t] && ng[t] > 0) c[t] = ld_stream(cp[t], pol);
        }
        // an unvisited row whose first entry is padding is a long row (rows
        // without sources start visited): the long-row pass has run already
#pragma unroll
        for (int t = 0; t < kW; t++) long_cand[t] = active[t] && c[t].x == p[t];
        for (int32_t j = 0;; j++) {
            bool any = false;
#pragma unroll
            for (int t = 0; t < kW; t++) {
                active[t] = active[t] && (j < ng[t]);
                any = any || active[t];
            }
            if (!__any_sync(kFull, any)) break;
            int4 nx[kW];
            uint32_t ff[kW][4];
#pragma unroll
            for (int t = 0; t < kW; t++) {
                nx[t] = make_int4(p[t], p[t], p[t], p[t]);
                if (!active[t]) continue;
                bytes += 32;  // four columns and the four frontier words they select
                n_grp++;
                if (j + 1 < ng[t]) nx[t] = ld_stream(cp[t] + (int64_t)(j + 1) * C, pol);
                ALB_CHECK_ID4(c[t], a.nwords * 32, p[t], &a.ctl->err);
                ff[t][0] = ld_front<kSmemF, kPersist>(F, c[t].x >> 5);
                ff[t][1] = ld_front<kSmemF, kPersist>(F, c[t].y >> 5);
                ff[t][2] = ld_front<kSmemF, kPersist>(F, c[t].z >> 5);
                ff[t][3] = ld_front<kSmemF, kPersist>(F, c[t].w >> 5);
            }
#pragma unroll
            for (int t = 0; t < kW; t++) {
                if (!active[t]) continue;
                const int32_t cc[4] = {c[t].x, c[t].y, c[t].z, c[t].w};
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if (!active[t]) break;
                    if (kEarly && cc[k] == p[t]) {
                        active[t] = false;  // padding: end of row
                    } else if ((ff[t][k] >> (cc[k] & 31)) & 1u) {
                        if (found[t] < 0) found[t] = cc[k];
                        if (kEarly) active[t] = false;
                    }
                }
                c[t] = nx[t];
            }
        }
        for (int t = 0; t < nr; t++) {
            bool reached = found[t] >= 0;
            bool by_long = false;
            if (long_cand[t] && !reached && a.nlong)
                by_long = reached = ld_state<kPersist>(a.parent_pos + p[t]) != kFull;
            const unsigned nm = __ballot_sync(kFull, reached);
            if (lane == 0) {
                N[w[t]] = nm;
                if (nm) {
                    a.vis[w[t]] = vis[t] | nm;
                    full += (vis[t] != kFull && (vis[t] | nm) == kFull);
                }
            }
            if (reached) {
                a.level_pos[p[t]] = lvl;
                if (!by_long) a.parent_pos[p[t]] = (uint32_t)__ldg(a.perm + found[t]);
                bytes += 20;  // level, parent, the parent's id, two degrees
                cn++;
                cmo += (unsigned long long)__ldg(a.odeg + p[t]);
                cmi += (unsigned long long)__ldg(a.ideg + p[t]);
            }
        }
      }
    }
    add_stat(a, L, kStWordsBypassed, n_wbyp);
    add_stat(a, L, kStRowsScanned, n_rows);
    add_stat(a, L, kStGroupsRead, n_grp);
    add_stat(a, L, kStGroupsTotal, n_gtot);
    cn = warp_sum(cn);
    cmo = warp_sum(cmo);
    cmi = warp_sum(cmi);
    bytes = warp_sum(bytes);
    if (lane == 0 && (cn || full || bytes)) {
        const int k = (L + 1) % 3;
        if (cn) {
            atomicAdd(&a.ctl->acc_n[k], (unsigned long long)cn);
            atomicAdd(&a.ctl->acc_mo[k], cmo);
            atomicAdd(&a.ctl->acc_mi[k], cmi);
        }
        if (full) atomicAdd(&a.ctl->acc_full[k], (unsigned long long)full);
        if (bytes) atomicAdd(&a.ctl->acc_bytes[k], bytes);
    }
}

// Bottom-up pull of the long rows (kept out of the slices). Rows are in
// source-id order, so a row's parent is its first frontier source.
// Head pass: one warp per unvisited long row scans its first kLongChunk
// sources, 32 per step; a hit there is the row's first frontier source. A row
// with no hit in its head and more sources left goes on the continuation list
// (packed counter in nbig[L % 3]: rows << kBigShift | chunks), whose
// kLongChunk-source chunks the tail pass spreads over all warps; their hits
// meet in parent_pos[p] by atomicMin. The slice pass that follows sees
// parent_pos[p] set and records the row as reached. Both run before bu_phase.
// First frontier source among sources [st, en) of one long row (-1 if
// none), 128 per step: each lane loads four source ids, then their four
// frontier words, before testing any; the earliest hit is the lowest lane of
// the first 32-source group with one.
template <bool kPersist, bool kEarly>
__device__ __forceinline__ int32_t long_scan(const BfsArgs &a, const uint32_t *F, int64_t st,
                                             int64_t en, unsigned long long &bytes) {
    const int lane = threadIdx.x & 31;
    int32_t found = -1;
    for (int64_t e0 = st; e0 < en; e0 += 128) {
        int32_t c[4];
        uint32_t f[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int64_t e = e0 + 32 * u + lane;
            c[u] = e < en ? __ldg(a.lcol + e) : -1;
            if (c[u] >= 0) ALB_CHECK_ID(c[u], a.n, -1, &a.ctl->err);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) f[u] = c[u] >= 0 ? ld_bits<kPersist>(F + (c[u] >> 5)) : 0u;
        bytes += 8 * (unsigned long long)min((int64_t)128, en - e0);
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const bool hit = c[u] >= 0 && ((f[u] >> (c[u] & 31)) & 1u);
            const unsigned m = __ballot_sync(kFull, hit);
            if (m && found < 0) found = __shfl_sync(kFull, c[u], __ffs(m) - 1);
        }
        if (kEarly && found >= 0) break;
    }
    return found;
}

template <bool kPersist, bool kEarly>
__device__ void bu_long_phase(const BfsArgs &a, int L, Range r) {
    if (a.nlong == 0) return;
    const uint32_t *F = (L & 1) ? a.bm1 : a.bm0;
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t nwarps = (int64_t)r.nblk * wpb;
    unsigned long long *cont = &a.ctl->nbig[L % 3];
    unsigned long long bytes = 0;
    // rows stay strided over the warps (row gw + k * nwarps goes to warp gw),
    // but a warp loads the position, visited bit and offsets of its next 32
    // rows at once, one per lane, then scans the unvisited ones
    const int64_t gw = (int64_t)r.bid * wpb + (threadIdx.x >> 5);
    for (int64_t i0 = gw; i0 < a.nlong; i0 += 32 * nwarps) {
        const int64_t i = i0 + lane * nwarps;
        int32_t p_l = 0;
        int64_t st_l = 0, en_l = 0;
        bool todo_l = false;
        if (i < a.nlong) {
            p_l = __ldg(a.lrow + i);
            st_l = __ldg(a.lptr + i);
            en_l = __ldg(a.lptr + i + 1);
            todo_l = !((ld_bits<kPersist>(a.vis + (p_l >> 5)) >> (p_l & 31)) & 1u);
        }
        unsigned todo = __ballot_sync(kFull, todo_l);
        while (todo) {
            const int b = __ffs(todo) - 1;
            todo &= todo - 1;
            const int32_t p = __shfl_sync(kFull, p_l, b);
            const int64_t st = __shfl_sync(kFull, st_l, b), en = __shfl_sync(kFull, en_l, b);
            const int64_t hen = min(en, st + kLongChunk);
            bytes += 24;
            const int32_t found = long_scan<kPersist, kEarly>(a, F, st, hen, bytes);
            if (lane == 0) {
                if (found >= 0) {
                    atomicMin(a.parent_pos + p, (uint32_t)__ldg(a.perm + found));
                } else if (hen < en) {
                    const unsigned long long nch =
                        (unsigned long long)((en - hen + kLongChunk - 1) / kLongChunk);
                    const unsigned long long old = atomicAdd(cont, (1ull << kBigShift) | nch);
                    const int64_t idx = (int64_t)(old >> kBigShift);
                    a.big[idx] = (int32_t)(i0 + b * nwarps);
                    a.big_base[idx] = (int64_t)(old & kBigMask);
                }
            }
        }
    }
    if (lane == 0 && bytes) atomicAdd(&a.ctl->acc_bytes[(L + 1) % 3], bytes);
}

// Tail pass over the continuation list: chunk k of list entry j covers
// sources [lptr[i] + (1 + k - big_base[j]) * kLongChunk, ...) of long row
// i = big[j]; the entry is found by binary search over big_base.
template <bool kPersist, bool kEarly>
__device__ void bu_long_tail_phase(const BfsArgs &a, int L, Range r) {
    const unsigned long long ctr = ld_state<kPersist>(&a.ctl->nbig[L % 3]);
    if (ctr == 0) return;
    const int64_t nrows = (int64_t)(ctr >> kBigShift);
    const int64_t total = (int64_t)(ctr & kBigMask);
    const uint32_t *F = (L & 1) ? a.bm1 : a.bm0;
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t nwarps = (int64_t)r.nblk * wpb;
    unsigned long long bytes = 0;
    for (int64_t k = (int64_t)r.bid * wpb + (threadIdx.x >> 5); k < total; k += nwarps) {
        int64_t lo = 0, hi = nrows - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (ld_state<kPersist>(a.big_base + mid) <= k) lo = mid;
            else hi = mid - 1;
        }
        const int32_t i = ld_state<kPersist>(a.big + lo);
        const int32_t p = __ldg(a.lrow + i);
        const int64_t c = k - ld_state<kPersist>(a.big_base + lo);
        const int64_t st = __ldg(a.lptr + i) + (1 + c) * kLongChunk;
        const int64_t en = min(__ldg(a.lptr + i + 1), st + kLongChunk);
        bytes += 24;
        const int32_t found = long_scan<kPersist, kEarly>(a, F, st, en, bytes);
        if (found >= 0 && lane == 0) atomicMin(a.parent_pos + p, (uint32_t)__ldg(a.perm + found));
    }
    if (lane == 0 && bytes) atomicAdd(&a.ctl->acc_bytes[(L + 1) % 3], bytes);
}

// Algorithmic bytes of the level that just ran (see alb_level_rec).
__host__ __device__ inline int64_t level_bytes(const BfsCtl &c, int dir, unsigned long long nn,
                                               unsigned long long counted) {
    if (dir == ALB_DIR_TOPDOWN) return 20 * c.nf + 8 * c.mf + 12 * (int64_t)nn;
    return (int64_t)counted + 12 * c.nwords;
}

// The level's bypass statistics (slot k) into its trace record.
template <class Ctl>
__device__ inline void write_stats(alb_level_rec &r, Ctl &c, int k) {
    r.words_bypassed = (int64_t)c.acc_stat[k][kStWordsBypassed];
    r.rows_scanned = (int64_t)c.acc_stat[k][kStRowsScanned];
    r.groups_read = (int64_t)c.acc_stat[k][kStGroupsRead];
    r.groups_bypassed =
        (int64_t)c.acc_stat[k][kStGroupsTotal] - (int64_t)c.acc_stat[k][kStGroupsRead];
    r.edges_bypassed = (int64_t)c.acc_stat[k][kStEdgesBypassed];
}

// Level rollover from the accumulators of slot (L+1)%3 (values read with
// coherent loads by the caller).
__host__ __device__ inline void roll(BfsCtl &c, int dir, unsigned long long nn,
                                     unsigned long long mo, unsigned long long mi,
                                     unsigned long long fl) {
    c.prev_nf = c.nf;
    c.nf = (int64_t)nn;
    c.mf = (int64_t)mo;
    c.nu -= (int64_t)nn;
    c.mu -= (int64_t)mi;
    c.active_words -= (int64_t)fl;
    c.reached += (int64_t)nn;
    c.edges += (int64_t)mo;
    c.q_valid = dir == ALB_DIR_TOPDOWN;
    c.n_dirty = dir != ALB_DIR_TOPDOWN;
    c.prev_dir = dir;
    if (dir == ALB_DIR_TOPDOWN)
        c.levels_td++;
    else
        c.levels_bu++;
    c.level++;
    if (nn == 0 || c.level >= c.level_cap || c.err) c.done = 1;
}

// ---------------------------------------------------- standalone kernels

__global__ void k_init_bulk(BfsArgs a) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t str = (int64_t)gridDim.x * blockDim.x;
    for (int64_t p = tid; p < a.n; p += str) {
        a.level_pos[p] = -1;
        a.parent_pos[p] = 0xFFFFFFFFu;
    }
    for (int64_t w = tid; w < a.nwords; w += str) {
        a.vis[w] = a.vinit[w];
        a.bm0[w] = 0;
        a.bm1[w] = 0;
    }
}

struct InitParams {
    int32_t root, policy, trace_cap, level_cap;
    float alpha, beta, mean_deg, skew;
    int64_t n_live, m_in, active0;
};

__global__ void k_init_root(BfsArgs a, InitParams ip) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int32_t rp = a.inv[ip.root];
    const uint32_t bit = 1u << (rp & 31);
    const uint32_t old = a.vis[rp >> 5];
    a.vis[rp >> 5] = old | bit;
    a.bm0[rp >> 5] |= bit;
    a.q0[0] = rp;
    a.level_pos[rp] = 0;
    a.parent_pos[rp] = (uint32_t)ip.root;
    BfsCtl c;
    memset(&c, 0, sizeof(c));
    c.level = 0;
    c.dir = -1;
    c.prev_dir = -1;
    c.q_valid = 1;
    c.n_dirty = 0;
    c.policy = ip.policy;
    c.alpha = ip.alpha;
    c.beta = ip.beta;
    c.n = a.n;
    c.nwords = a.nwords;
    c.nf = 1;
    c.mf = a.odeg[rp];
    c.prev_nf = 0;
    const bool live = a.ideg[rp] > 0;  // discoverable by a pull
    c.nu = ip.n_live - (live ? 1 : 0);
    c.mu = ip.m_in - a.ideg[rp];
    c.active_words = ip.active0 - ((old != kFull && (old | bit) == kFull) ? 1 : 0);
    c.reached = 1;
    c.edges = a.odeg[rp];
    c.qn[0] = 1;
    c.trace_cap = ip.trace_cap;
    c.level_cap = ip.level_cap;
    c.feat_mean_deg = ip.mean_deg;
    c.feat_skew = ip.skew;
    *a.ctl = c;
    *a.bar = 0;
}

__global__ void k_decide(BfsArgs a, int forced, cudaGraphConditionalHandle sw) {
    if (threadIdx.x >= 32) return;
    const BfsCtl c = *a.ctl;
    const int dir = decide_warp(a, c, forced);
    if (threadIdx.x == 0) {
        a.ctl->dir = dir;
        record_trace(a, c, dir);
        // zero the slots the next level will accumulate into
        const int k = (c.level + 2) % 3;
        a.ctl->acc_n[k] = 0;
        a.ctl->acc_mo[k] = 0;
        a.ctl->acc_mi[k] = 0;
        a.ctl->acc_full[k] = 0;
        a.ctl->acc_bytes[k] = 0;
        for (int i = 0; i < kStatN; i++) a.ctl->acc_stat[k][i] = 0;
        a.ctl->acc_active[k] = 0;
        a.ctl->nbig[k] = 0;
        a.ctl->work[k] = 0;
        a.ctl->qn[k] = 0;
        unsigned branch;
        if (dir == ALB_DIR_TOPDOWN)
            branch = (!c.q_valid || c.n_dirty) ? 1u : 0u;
        else
            branch = dir == ALB_DIR_BOTTOMUP ? 2u : 3u;
        a.ctl->branch = (int32_t)branch;
        if (sw) cudaGraphSetConditional(sw, branch);
    }
}

__global__ void k_prep(BfsArgs a) {
    const BfsCtl *c = a.ctl;
    const int L = c->level;
    prep_phase<false>(a, L, !c->q_valid, c->n_dirty != 0, Range{(int)blockIdx.x, (int)gridDim.x});
}

__global__ void k_td(BfsArgs a) {
    const int64_t mf = a.ctl->mf;
    td_phase<false>(a, a.ctl->level, Range{(int)blockIdx.x, (int)gridDim.x}, mf,
                    td_append(a, mf));
}

__global__ void k_td_big(BfsArgs a) {
    td_big_phase<false>(a, a.ctl->level, Range{(int)blockIdx.x, (int)gridDim.x},
                        td_append(a, a.ctl->mf));
}

__global__ void k_td_finish(BfsArgs a) {
    td_finish_phase<false>(a, a.ctl->level, Range{(int)blockIdx.x, (int)gridDim.x},
                           td_append(a, a.ctl->mf));
}

// The slice pass runs with kBuBlock threads whatever the loop's block size:
// the bound holds it at 64 registers (4 blocks, 32 warps per SM; it scans
// two words at a time).
constexpr unsigned kBuBlock = 256;

template <bool kBypass, bool kEarly>
__global__ void __launch_bounds__(kBuBlock, 4) k_bu(BfsArgs a) {
    bu_phase<false, kBypass, kEarly>(a, a.ctl->level, Range{(int)blockIdx.x, (int)gridDim.x});
}

// The slice pass with the frontier bitmap staged in shared memory: one CTA
// of kBuSmemBlock threads per SM copies the whole bitmap (nwords * 4 bytes,
// at most kSmemFrontierMax) with one bulk copy completing on an mbarrier,
// then gathers frontier words from shared memory. The wait is bounded: past
// kBulkWaitNs it records ALB_ERR_TIMEOUT and the CTA leaves.
constexpr unsigned kBuSmemBlock = 1024;
constexpr int64_t kSmemFrontierMax = 192 * 1024;
constexpr uint64_t kBulkWaitNs = 2ull * 1000 * 1000 * 1000;

template <bool kBypass, bool kEarly>
__global__ void __launch_bounds__(kBuSmemBlock, 1) k_bu_smem(BfsArgs a) {
    extern __shared__ __align__(16) uint32_t s_front[];
    __shared__ __align__(8) uint64_t s_bar;
    const int L = a.ctl->level;
    const uint32_t *F = (L & 1) ? a.bm1 : a.bm0;
    const uint32_t bytes = (uint32_t)(((a.nwords * 4) + 15) & ~15ll);
    if (threadIdx.x == 0) {
        mbar_init(&s_bar, 1);
        // (short_bulk: a test hook expecting bytes the copy never delivers)
        mbar_expect_tx(&s_bar, bytes + (a.short_bulk ? 16u : 0u));
        bulk_g2s(s_front, F, bytes, &s_bar);
    }
    __syncthreads();  // the barrier is initialised before anyone waits on it
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(&s_bar, 0)) {
        if (globaltimer_ns() - t0 > a.bulk_ns) {
            if (threadIdx.x == 0) atomicExch(&a.ctl->err, ALB_ERR_TIMEOUT);
            // the copy may still be writing this CTA's shared memory: stay
            // resident until it lands (second, longer bound) before leaving
            const uint64_t t1 = globaltimer_ns();
            while (!mbar_try_wait(&s_bar, 0) && globaltimer_ns() - t1 < 4 * a.bulk_ns)
                __nanosleep(1024);
            return;
        }
    }
    bu_phase<false, kBypass, kEarly, true>(a, L, Range{(int)blockIdx.x, (int)gridDim.x}, s_front);
}

template <bool kEarly>
__global__ void k_bu_long(BfsArgs a) {
    bu_long_phase<false, kEarly>(a, a.ctl->level, Range{(int)blockIdx.x, (int)gridDim.x});
}

template <bool kEarly>
__global__ void k_bu_long_tail(BfsArgs a) {
    bu_long_tail_phase<false, kEarly>(a, a.ctl->level, Range{(int)blockIdx.x, (int)gridDim.x});
}

__global__ void k_end(BfsArgs a, cudaGraphConditionalHandle wh) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    BfsCtl c = *a.ctl;
    const int k = (c.level + 1) % 3;
    if (a.trace && c.level < c.trace_cap) {
        a.trace[c.level].bytes = level_bytes(c, c.dir, c.acc_n[k], c.acc_bytes[k]);
        write_stats(a.trace[c.level], c, k);
    }
    c.launches += 2 + (c.branch == 1 ? 4 : 3);  // decide, end, steps
    roll(c, c.dir, c.acc_n[k], c.acc_mo[k], c.acc_mi[k], c.acc_full[k]);
    if (c.level < c.trace_cap) c.trace_len = c.level;
    else c.trace_len = c.trace_cap;
    *a.ctl = c;
    if (wh) cudaGraphSetConditional(wh, c.done ? 0u : 1u);
}

__global__ void k_scatter(BfsArgs a, int32_t *level, int32_t *parent) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t str = (int64_t)gridDim.x * blockDim.x;
    for (int64_t p = tid; p < a.n; p += str) {
        const int32_t v = a.perm[p];
        if (level) level[v] = a.level_pos[p];
        if (parent) parent[v] = (int32_t)a.parent_pos[p];
    }
}

// ------------------------------------------------------ persistent kernel

// Grid barrier of the persistent kernel: one 64-bit arrival counter that is
// never reset. A block's arrival (an acquire-release atomicAdd, which also
// publishes the block's writes) returns the count before it; the barrier it
// belongs to ends when the count reaches the next multiple of the block
// count, so the last arrival itself releases everyone -- no reset, no second
// word, one round trip on the critical path. Waits are bounded by
// a.barrier_ns: on expiry the block records ALB_ERR_TIMEOUT and sets bit 62,
// which puts the count past every target, so every waiter leaves at once and
// reads the failure from the same word. (withhold_level: a test hook under
// which one block skips its arrival at level L's barriers and leaves.)
__device__ __forceinline__ unsigned long long atom_add_acq_rel(unsigned long long *p,
                                                               unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v)
                 : "memory");
    return old;
}

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// The level's counters as they stand after a barrier, read by thread 0
// right after its wait (all five loads in one round trip) and shared with
// the block by the barrier's closing __syncthreads: nbig[L % 3] (long frontier
// rows) and the (L + 1) % 3 accumulators that roll() consumes.
struct LevelSums {
    unsigned long long nbig, n, mo, mi, full;
    unsigned long long qn;  // qn[(L + 1) % 3]: the next level's queue, when it was built
};

__device__ bool grid_sync(const BfsArgs &a, unsigned nblocks, int L, LevelSums *sums = nullptr) {
    BfsCtl *ctl = a.ctl;
    if (a.withhold_level >= 0 && L == a.withhold_level && (int)blockIdx.x == a.withhold_block)
        return false;
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned long long old = atom_add_acq_rel(a.bar, 1ull);
        bool ok = !(old & kBarFailed);
        if (ok) {
            const unsigned long long target = (old / nblocks + 1) * nblocks;
            if (old + 1 != target) {
                const uint64_t t0 = globaltimer_ns();
                unsigned long long cur;
                while ((cur = ld_acquire(a.bar)) < target) {
                    if (globaltimer_ns() - t0 > a.barrier_ns) {
                        atomicExch(&ctl->err, ALB_ERR_TIMEOUT);
                        atomicOr(a.bar, kBarFailed);
                        cur = kBarFailed;
                        break;
                    }
                }
                ok = !(cur & kBarFailed);
            }
        }
        if (ok && sums) {
            const volatile BfsCtl *g = ctl;
            const int k = (L + 1) % 3;
            sums->nbig = g->nbig[L % 3];
            sums->n = g->acc_n[k];
            sums->mo = g->acc_mo[k];
            sums->mi = g->acc_mi[k];
            sums->full = g->acc_full[k];
            sums->qn = g->qn[k];
        }
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    return s_ok != 0;
}

// One block of kPersistBlock threads per SM: a grid barrier then waits for
// as few arrivals as the SM count.
constexpr unsigned kPersistBlock = 768;

__global__ void __launch_bounds__(kPersistBlock, 1) k_persistent(BfsArgs a) {
    __shared__ BfsCtl c;
    __shared__ int s_dir;
    __shared__ LevelSums s_sums;
    // the current level's queue length when the last level's closing barrier
    // read it (-1: read it from the control block)
    __shared__ int64_t s_qlen;
    // the selector network, read once per launch instead of once per level
    __shared__ __align__(16) float s_mlp[kMlpParams + 1];
    const unsigned nb = gridDim.x;
    const Range r{(int)blockIdx.x, (int)gridDim.x};
    if (threadIdx.x == 0) {
        c = *a.ctl;  // written by an earlier launch
        s_qlen = -1;
    }
    if (a.mlp)
        for (int i = threadIdx.x; i <= kMlpParams; i += blockDim.x) s_mlp[i] = a.mlp[i];
    __syncthreads();
    while (true) {
        if (threadIdx.x < 32) {
            const int dir = decide_warp(a, c, -1, s_mlp);
            if (threadIdx.x == 0) {
                s_dir = dir;
                if (blockIdx.x == 0) {
                    record_trace(a, c, dir);
                    const int k = (c.level + 2) % 3;
                    a.ctl->acc_n[k] = 0;
                    a.ctl->acc_mo[k] = 0;
                    a.ctl->acc_mi[k] = 0;
                    a.ctl->acc_full[k] = 0;
                    a.ctl->acc_bytes[k] = 0;
                    for (int i = 0; i < kStatN; i++) a.ctl->acc_stat[k][i] = 0;
                    a.ctl->acc_active[k] = 0;
                    a.ctl->nbig[k] = 0;
                    a.ctl->work[k] = 0;
                    a.ctl->qn[k] = 0;
                }
            }
        }
        __syncthreads();
        const int dir = s_dir;
        const int L = c.level;
        bool ok = true;
        // small top-down levels run lazily: one barrier per level, the
        // bitmaps rebuilt when a level that reads them comes (materialize)
        const bool lazy = dir == ALB_DIR_TOPDOWN && td_append(a, c.mf);
        if (c.lazy && !lazy) {
            materialize_phase(a, L, r);
            ok = grid_sync(a, nb, L);
            if (threadIdx.x == 0) {
                c.active_words = (int64_t) * (volatile unsigned long long *)&a.ctl->acc_active[L % 3];
                c.lazy = 0;
                c.q_valid = 1;  // the lazy levels' claims built the queue
                c.n_dirty = 0;
            }
            __syncthreads();
        }
        if (!ok) {
            // a barrier gave up: every block leaves below
        } else if (dir == ALB_DIR_TOPDOWN) {
            int64_t qk = s_qlen;
            if (!c.q_valid || c.n_dirty) {
                prep_phase<true>(a, L, !c.q_valid, c.n_dirty != 0, r);
                ok = grid_sync(a, nb, L);
                qk = -1;  // the queue was rebuilt
            }
            const bool app = td_append(a, c.mf);
            if (ok) {
                td_phase<true>(a, L, r, c.mf, app, lazy, qk);
                ok = grid_sync(a, nb, L, &s_sums);
            }
            if (ok && s_sums.nbig) {
                td_big_phase<true>(a, L, r, app, lazy);
                ok = grid_sync(a, nb, L, &s_sums);
            }
            if (ok && !lazy) {
                td_finish_phase<true>(a, L, r, app);
                ok = grid_sync(a, nb, L, &s_sums);
            }
        } else if (dir == ALB_DIR_BOTTOMUP) {
            if (a.nlong) {
                bu_long_phase<true, true>(a, L, r);
                ok = grid_sync(a, nb, L, &s_sums);
                if (ok && s_sums.nbig) {
                    bu_long_tail_phase<true, true>(a, L, r);
                    ok = grid_sync(a, nb, L);
                }
            }
            if (ok) {
                bu_phase<true, true, true>(a, L, r);
                ok = grid_sync(a, nb, L, &s_sums);
            }
        } else {
            if (a.nlong) {
                bu_long_phase<true, false>(a, L, r);
                ok = grid_sync(a, nb, L, &s_sums);
                if (ok && s_sums.nbig) {
                    bu_long_tail_phase<true, false>(a, L, r);
                    ok = grid_sync(a, nb, L);
                }
            }
            if (ok) {
                bu_phase<true, false, false>(a, L, r);
                ok = grid_sync(a, nb, L, &s_sums);
            }
        }
        if (!ok) break;
        if (threadIdx.x == 0) {
            // the level's last barrier read its counters into s_sums
            const int k = (L + 1) % 3;
            if (blockIdx.x == 0 && a.trace && L < c.trace_cap) {
                volatile BfsCtl *g = a.ctl;
                a.trace[L].bytes = level_bytes(c, dir, s_sums.n, g->acc_bytes[k]);
                write_stats(a.trace[L], *g, k);
            }
            roll(c, dir, s_sums.n, s_sums.mo, s_sums.mi, s_sums.full);
            c.dir = dir;
            if (lazy) c.lazy = 1;
            // a top-down level built the next queue before its last barrier
            s_qlen = dir == ALB_DIR_TOPDOWN ? (int64_t)s_sums.qn : -1;
        }
        __syncthreads();
        if (c.done) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // publish the rolling fields (accumulators and barrier stay as they are)
        BfsCtl *g = a.ctl;
        g->level = c.level;
        g->dir = c.dir;
        g->prev_dir = c.prev_dir;
        g->q_valid = c.q_valid;
        g->n_dirty = c.n_dirty;
        g->done = c.done;
        g->levels_td = c.levels_td;
        g->levels_bu = c.levels_bu;
        g->nf = c.nf;
        g->mf = c.mf;
        g->prev_nf = c.prev_nf;
        g->nu = c.nu;
        g->mu = c.mu;
        g->active_words = c.active_words;
        g->reached = c.reached;
        g->edges = c.edges;
        g->trace_len = c.level < c.trace_cap ? c.level : c.trace_cap;
    }
}

// ------------------------------------------------------------- host side

}  // namespace alb

struct alb::CachedLoop {
    int block = 0;
    uint64_t bulk_ns = 0;  // the wait settings baked into the kernel nodes
    int32_t short_bulk = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace alb {

alb_status bfs_scratch_alloc(alb_graph *g) {
    BfsScratch &b = g->bfs;
    if (b.ready) return ALB_OK;
    const int64_t n = g->n, nw = g->sell.nwords;
    // the three bitmaps in one allocation (one L2 window covers them), each
    // padded to 16 bytes: k_bu_smem copies a frontier bitmap whole
    const int64_t nw16 = (nw + 3) & ~3ll;
    ALB_TRY(dmalloc((void **)&b.bits, sizeof(uint32_t) * 3 * nw16, "bitmaps"));
    b.bm0 = b.bits;
    b.bm1 = b.bits + nw16;
    b.vis = b.bits + 2 * nw16;
    b.win = cudaAccessPolicyWindow{};
    if (nw * 4 > kSmemFrontierMax) {
        // the frontier is gathered from global memory: keep the bitmaps in a
        // persisting L2 window (the column stream is marked evict-first) so
        // a level's gathers do not miss on lines the previous level wrote
        int maxwin = 0, maxpers = 0;
        cudaDeviceGetAttribute(&maxwin, cudaDevAttrMaxAccessPolicyWindowSize, g->device);
        cudaDeviceGetAttribute(&maxpers, cudaDevAttrMaxPersistingL2CacheSize, g->device);
        const size_t bytes = sizeof(uint32_t) * 3 * (size_t)nw16;
        if (maxwin > 0 && maxpers > 0) {
            const size_t win = std::min(bytes, (size_t)maxwin);
            const size_t pers = std::min(win, (size_t)maxpers);
            size_t cur = 0;
            cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize);
            if (cur < pers && cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, pers) != cudaSuccess)
                cudaGetLastError();
            cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize);
            if (cur > 0) {
                b.win.base_ptr = b.bits;
                b.win.num_bytes = win;
                b.win.hitRatio = std::min(1.0f, (float)cur / (float)win);
                b.win.hitProp = cudaAccessPropertyPersisting;
                b.win.missProp = cudaAccessPropertyStreaming;
            }
        }
    }
    ALB_TRY(dmalloc((void **)&b.q0, sizeof(int32_t) * n, "frontier queue"));
    ALB_TRY(dmalloc((void **)&b.q1, sizeof(int32_t) * n, "frontier queue"));
    ALB_TRY(dmalloc((void **)&b.big, sizeof(int32_t) * n, "long-row list"));
    ALB_TRY(dmalloc((void **)&b.big_base, sizeof(int64_t) * n, "long-row chunk bases"));
    ALB_TRY(dmalloc((void **)&b.level_pos, sizeof(int32_t) * n, "levels"));
    ALB_TRY(dmalloc((void **)&b.parent_pos, sizeof(uint32_t) * n, "parents"));
    ALB_TRY(dmalloc((void **)&b.ctl, sizeof(BfsCtl), "level control"));
    ALB_TRY(dmalloc((void **)&b.bar, 256, "grid barrier"));
    b.trace_cap = (int32_t)std::min<int64_t>(n + 2, 1 << 16);
    ALB_TRY(dmalloc((void **)&b.trace, sizeof(alb_level_rec) * b.trace_cap, "level trace"));
    ALB_CK(cudaMallocHost((void **)&b.h_ctl, sizeof(BfsCtl)));
    b.ready = true;
    return ALB_OK;
}

void bfs_scratch_free(alb_graph *g) {
    BfsScratch &b = g->bfs;
    dfree(b.bits);
    dfree(b.q0);
    dfree(b.q1);
    dfree(b.big);
    dfree(b.big_base);
    dfree(b.level_pos);
    dfree(b.parent_pos);
    dfree(b.out_level);
    dfree(b.out_parent);
    dfree(b.ctl);
    dfree(b.bar);
    dfree(b.trace);
    if (b.h_ctl) cudaFreeHost(b.h_ctl);
    b = BfsScratch();
}

void loop_cache_free(alb_graph *g) {
    if (!g->loop) return;
    if (g->loop->exec) cudaGraphExecDestroy(g->loop->exec);
    if (g->loop->graph) cudaGraphDestroy(g->loop->graph);
    delete g->loop;
    g->loop = nullptr;
}

extern const float *selector_device_params(int which);
extern bool selector_host_params(int which, float *out);

float skew_of(const Sell &s, int64_t n) {
    const double mean = n > 0 ? (double)s.m_in / (double)n : 0.0;
    return mean > 0 ? (float)std::log2(1.0 + (double)s.max_deg / mean) : 0.0f;
}

BfsArgs make_args(alb_graph *g) {
    const Sell &s = g->sell;
    const BfsScratch &b = g->bfs;
    BfsArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = g->n;
    a.nslices = s.nslices;
    a.nwords = s.nwords;
    a.C = s.C;
    a.log2C = s.log2C;
    a.perm = s.perm;
    a.inv = s.inv;
    a.ideg = s.ideg;
    a.odeg = s.odeg;
    a.width = s.width;
    a.slice_off = s.slice_off;
    a.col4 = (const int4 *)s.col;
    a.prow = s.prow;
    a.pcol = s.pcol;
    a.nlong = s.nlong;
    a.lrow = s.lrow;
    a.lptr = s.lptr;
    a.lcol = s.lcol;
    a.vinit = s.vinit;
    a.bm0 = b.bm0;
    a.bm1 = b.bm1;
    a.vis = b.vis;
    a.q0 = b.q0;
    a.q1 = b.q1;
    a.big = b.big;
    a.big_base = b.big_base;
    a.level_pos = b.level_pos;
    a.parent_pos = b.parent_pos;
    a.ctl = b.ctl;
    a.bar = b.bar;
    a.trace = b.trace;
    a.mlp = selector_device_params(0);
    const DeviceWaits dw = device_waits(kBarrierTimeoutNs, kBulkWaitNs);
    a.barrier_ns = dw.barrier_ns;
    a.bulk_ns = dw.bulk_ns;
    a.withhold_level = dw.withhold_level;
    a.withhold_block = dw.withhold_block;
    a.short_bulk = dw.short_bulk;
    return a;
}

namespace {

struct Launch {
    unsigned grid;
    unsigned block;
    int sms;
};

Launch level_launch(const alb_graph *g, int block) {
    // every level kernel is a grid-stride loop: fill the GPU once
    const int per_sm = std::max(1, 2048 / block);
    return Launch{(unsigned)(g->num_sms * per_sm), (unsigned)block, g->num_sms};
}

Launch with_block(const Launch &w, unsigned block) { return Launch{w.grid, block, w.sms}; }

// The same launch with as many blocks as are resident at once for func (its
// registers can allow fewer than 2048 threads per SM): a grid-stride kernel
// then runs in one wave instead of leaving a partial second wave.
Launch fit(const void *func, const Launch &w) {
    const int per = resident_blocks(func, (int)w.block);
    if (per <= 0) return w;
    return Launch{(unsigned)(w.sms * per), w.block, w.sms};
}

alb_status add_kernel_node(cudaGraph_t graph, cudaGraphNode_t *node, const cudaGraphNode_t *deps,
                           size_t ndeps, void *func, Launch l, void **args, size_t smem = 0,
                           const cudaAccessPolicyWindow *win = nullptr) {
    cudaKernelNodeParams p;
    std::memset(&p, 0, sizeof(p));
    p.func = func;
    p.gridDim = dim3(l.grid);
    p.blockDim = dim3(l.block);
    p.sharedMemBytes = (unsigned)smem;
    p.kernelParams = args;
    ALB_CK(cudaGraphAddKernelNode(node, graph, deps, ndeps, &p));
    if (win) {
        cudaKernelNodeAttrValue v = {};
        v.accessPolicyWindow = *win;
        ALB_CK(cudaGraphKernelNodeSetAttribute(*node, cudaKernelNodeAttributeAccessPolicyWindow, &v));
    }
    return ALB_OK;
}

// The bottom-up slice pass of a level: the staged-frontier kernel when the
// bitmap fits in shared memory, else the kernel that gathers from global.
struct BuSlices {
    void *func;
    Launch l;
    size_t smem;
};

template <bool kBypass, bool kEarly>
BuSlices bu_slices(const BfsArgs &a, const Launch &wide) {
    if (a.nwords * 4 <= kSmemFrontierMax) {
        void *f = (void *)k_bu_smem<kBypass, kEarly>;
        cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kSmemFrontierMax);
        const size_t sm = (size_t)((a.nwords * 4 + 15) & ~15ll);
        return {f, Launch{(unsigned)wide.sms, kBuSmemBlock, wide.sms}, sm};
    }
    void *f = (void *)k_bu<kBypass, kEarly>;
    return {f, fit(f, with_block(wide, kBuBlock)), 0};
}

template <bool kBypass, bool kEarly>
void launch_bu_slices(const BfsArgs &a, const Launch &wide, cudaStream_t st) {
    const BuSlices b = bu_slices<kBypass, kEarly>(a, wide);
    void *args[] = {(void *)&a};
    cudaLaunchKernel(b.func, dim3(b.l.grid), dim3(b.l.block), args, b.smem, st);
}

// while (!done) { decide; switch { td | prep+td | bu | bu-nobypass }; end }
alb_status build_loop_graph(alb_graph *g, int block) {
    loop_cache_free(g);
    CachedLoop *cl = new CachedLoop();
    g->loop = cl;
    cl->block = block;
    BfsArgs a = make_args(g);
    cl->bulk_ns = a.bulk_ns;
    cl->short_bulk = a.short_bulk;
    const Launch wide = level_launch(g, block);
    const Launch one{1, 32, g->num_sms};
    const BuSlices bu2 = bu_slices<true, true>(a, wide), bu3 = bu_slices<false, false>(a, wide);
    // every level kernel carries the bitmaps' L2 window (when there is one)
    const cudaAccessPolicyWindow *W = g->bfs.win.num_bytes > 0 ? &g->bfs.win : nullptr;
    ALB_CK(cudaGraphCreate(&cl->graph, 0));
    cudaGraphConditionalHandle wh;
    ALB_CK(cudaGraphConditionalHandleCreate(&wh, cl->graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
    wp.conditional.handle = wh;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    ALB_CK(cudaGraphAddNode(&wnode, cl->graph, nullptr, nullptr, 0, &wp));
    cudaGraph_t body = wp.conditional.phGraph_out[0];

    cudaGraphConditionalHandle sh;
    ALB_CK(cudaGraphConditionalHandleCreate(&sh, body, 0, cudaGraphCondAssignDefault));
    int forced = -1;
    void *dargs[] = {&a, &forced, &sh};
    cudaGraphNode_t ndecide;
    ALB_TRY(add_kernel_node(body, &ndecide, nullptr, 0, (void *)k_decide, one, dargs, 0, W));
    cudaGraphNodeParams sp = {cudaGraphNodeTypeConditional};
    sp.conditional.handle = sh;
    sp.conditional.type = cudaGraphCondTypeSwitch;
    sp.conditional.size = 4;
    cudaGraphNode_t nswitch;
    ALB_CK(cudaGraphAddNode(&nswitch, body, &ndecide, nullptr, 1, &sp));
    void *aargs[] = {&a};
    {  // 0: top-down, queue ready
        cudaGraph_t b0 = sp.conditional.phGraph_out[0];
        cudaGraphNode_t t, bg, f;
        ALB_TRY(add_kernel_node(b0, &t, nullptr, 0, (void *)k_td, fit((const void *)k_td, wide),
                                aargs, 0, W));
        ALB_TRY(add_kernel_node(b0, &bg, &t, 1, (void *)k_td_big,
                                fit((const void *)k_td_big, wide), aargs, 0, W));
        ALB_TRY(add_kernel_node(b0, &f, &bg, 1, (void *)k_td_finish, wide, aargs, 0, W));
    }
    {  // 1: compaction / clear, then top-down
        cudaGraph_t b1 = sp.conditional.phGraph_out[1];
        cudaGraphNode_t pr, t, bg, f;
        ALB_TRY(add_kernel_node(b1, &pr, nullptr, 0, (void *)k_prep, wide, aargs, 0, W));
        ALB_TRY(add_kernel_node(b1, &t, &pr, 1, (void *)k_td, fit((const void *)k_td, wide),
                                aargs, 0, W));
        ALB_TRY(add_kernel_node(b1, &bg, &t, 1, (void *)k_td_big,
                                fit((const void *)k_td_big, wide), aargs, 0, W));
        ALB_TRY(add_kernel_node(b1, &f, &bg, 1, (void *)k_td_finish, wide, aargs, 0, W));
    }
    {  // 2: the long rows (head, tail), then bottom-up with bypass
        cudaGraphNode_t b, l, t;
        ALB_TRY(add_kernel_node(sp.conditional.phGraph_out[2], &l, nullptr, 0,
                                (void *)k_bu_long<true>,
                                fit((const void *)k_bu_long<true>, wide), aargs, 0, W));
        ALB_TRY(add_kernel_node(sp.conditional.phGraph_out[2], &t, &l, 1,
                                (void *)k_bu_long_tail<true>,
                                fit((const void *)k_bu_long_tail<true>, wide), aargs, 0, W));
        ALB_TRY(add_kernel_node(sp.conditional.phGraph_out[2], &b, &t, 1,
                                bu2.func, bu2.l, aargs, bu2.smem, W));
    }
    {  // 3: the long rows (head, tail), then bottom-up without bypass
        cudaGraphNode_t b, l, t;
        ALB_TRY(add_kernel_node(sp.conditional.phGraph_out[3], &l, nullptr, 0,
                                (void *)k_bu_long<false>,
                                fit((const void *)k_bu_long<false>, wide), aargs, 0, W));
        ALB_TRY(add_kernel_node(sp.conditional.phGraph_out[3], &t, &l, 1,
                                (void *)k_bu_long_tail<false>,
                                fit((const void *)k_bu_long_tail<false>, wide), aargs, 0, W));
        ALB_TRY(add_kernel_node(sp.conditional.phGraph_out[3], &b, &t, 1,
                                bu3.func, bu3.l, aargs, bu3.smem, W));
    }
    void *eargs[] = {&a, &wh};
    cudaGraphNode_t nend;
    ALB_TRY(add_kernel_node(body, &nend, &nswitch, 1, (void *)k_end, one, eargs, 0, W));
    ALB_CK(cudaGraphInstantiate(&cl->exec, cl->graph, 0));
    return ALB_OK;
}

// Grid-stride level kernel launched with its resident grid.
void launch_fit(void *f, const BfsArgs &a, const Launch &wide, cudaStream_t st) {
    const Launch l = fit(f, wide);
    void *args[] = {(void *)&a};
    cudaLaunchKernel(f, dim3(l.grid), dim3(l.block), args, 0, st);
}

void launch_step(const BfsArgs &a, const Launch &wide, cudaStream_t st, int dir, const BfsCtl &h) {
    if (dir == ALB_DIR_TOPDOWN) {
        if (!h.q_valid || h.n_dirty) k_prep<<<wide.grid, wide.block, 0, st>>>(a);
        launch_fit((void *)k_td, a, wide, st);
        launch_fit((void *)k_td_big, a, wide, st);
        k_td_finish<<<wide.grid, wide.block, 0, st>>>(a);
    } else if (dir == ALB_DIR_BOTTOMUP) {
        launch_fit((void *)k_bu_long<true>, a, wide, st);
        launch_fit((void *)k_bu_long_tail<true>, a, wide, st);
        launch_bu_slices<true, true>(a, wide, st);
    } else {
        launch_fit((void *)k_bu_long<false>, a, wide, st);
        launch_fit((void *)k_bu_long_tail<false>, a, wide, st);
        launch_bu_slices<false, false>(a, wide, st);
    }
}

alb_status run_host_loop(alb_graph *g, const BfsArgs &a, const alb_bfs_opts &o,
                         std::vector<float> &step_us) {
    const Launch wide = level_launch(g, o.block);
    cudaStream_t st = g->stream;
    BfsCtl *h = g->bfs.h_ctl;
    step_us.clear();
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (o.trace) {
        ALB_CK(cudaEventCreate(&e0));
        ALB_CK(cudaEventCreate(&e1));
    }
    float mlp[kMlpParams];
    const bool have_mlp = o.policy == ALB_POLICY_LEARNED && selector_host_params(0, mlp);
    (void)a;
    ALB_CK(cudaMemcpyAsync(h, a.ctl, sizeof(BfsCtl), cudaMemcpyDeviceToHost, st));
    ALB_CK(cudaStreamSynchronize(st));
    while (!h->done) {
        int dir;
        if (have_mlp) {
            float f[kMlpIn], out[kMlpOut];
            level_features(*h, f);
            mlp_forward_host(mlp, f, out);
            dir = argmin3(out);
        } else {
            dir = rule_dir(*h);
        }
        k_decide<<<1, 32, 0, st>>>(a, dir, 0);
        if (e0) cudaEventRecord(e0, st);
        launch_step(a, wide, st, dir, *h);
        if (e1) cudaEventRecord(e1, st);
        k_end<<<1, 32, 0, st>>>(a, 0);
        ALB_CK(cudaGetLastError());
        ALB_CK(cudaMemcpyAsync(h, a.ctl, sizeof(BfsCtl), cudaMemcpyDeviceToHost, st));
        ALB_CK(cudaStreamSynchronize(st));
        if (e0) {
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            step_us.push_back(ms * 1000.0f);
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return ALB_OK;
}

alb_status run_persistent(alb_graph *g, const BfsArgs &a) {
    int per_sm = 0;
    ALB_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persistent, kPersistBlock, 0));
    if (per_sm < 1) return fail(ALB_ERR_CUDA, "persistent kernel does not fit on an SM");
    const unsigned grid = (unsigned)(per_sm * g->num_sms);
    BfsArgs args = a;
    void *kargs[] = {&args};
    ALB_CK(cudaLaunchCooperativeKernel((void *)k_persistent, dim3(grid), dim3(kPersistBlock), kargs,
                                       0, g->stream));
    return ALB_OK;
}


alb_status bfs_impl(alb_graph *g, int32_t root, const alb_bfs_opts &o, int32_t *d_level,
                    int32_t *d_parent, alb_stats *st) {
    ALB_TRY(bfs_scratch_alloc(g));
    const BfsArgs a = make_args(g);
    const Sell &s = g->sell;
    cudaStream_t stream = g->stream;
    InitParams ip;
    ip.root = root;
    ip.policy = o.policy;
    ip.trace_cap = o.trace ? g->bfs.trace_cap : 0;
    ip.level_cap = (int32_t)std::min<int64_t>(g->n + 1, INT32_MAX - 1);
    ip.alpha = o.alpha;
    ip.beta = o.beta;
    ip.mean_deg = g->n > 0 ? (float)((double)s.m_in / (double)g->n) : 0.f;
    ip.skew = skew_of(s, g->n);
    ip.n_live = g->n - s.zero_in;
    ip.m_in = s.m_in;
    ip.active0 = s.active0;
    const Launch wide = level_launch(g, 256);
    ALB_CK(cudaEventRecord(g->ev0, stream));
    k_init_bulk<<<wide.grid, wide.block, 0, stream>>>(a);
    k_init_root<<<1, 32, 0, stream>>>(a, ip);
    ALB_CK(cudaGetLastError());
    // the bitmaps' L2 window applies to the level loop's launches on the
    // stream (the CUDA-graph loop carries it on its kernel nodes); it is
    // removed again before the stream is handed back
    const bool win = g->bfs.win.num_bytes > 0 && o.loop != ALB_LOOP_GRAPH;
    if (win) {
        cudaStreamAttrValue v = {};
        v.accessPolicyWindow = g->bfs.win;
        ALB_CK(cudaStreamSetAttribute(stream, cudaStreamAttributeAccessPolicyWindow, &v));
    }
    std::vector<float> step_us;
    alb_status lrc = ALB_OK;
    if (o.loop == ALB_LOOP_HOST) {
        lrc = run_host_loop(g, a, o, step_us);
    } else if (o.loop == ALB_LOOP_PERSISTENT) {
        lrc = run_persistent(g, a);
    } else {
        if (!g->loop || g->loop->block != o.block || g->loop->bulk_ns != a.bulk_ns ||
            g->loop->short_bulk != a.short_bulk)
            lrc = build_loop_graph(g, o.block);
        if (lrc == ALB_OK && cudaGraphLaunch(g->loop->exec, stream) != cudaSuccess)
            lrc = fail(ALB_ERR_CUDA, "cudaGraphLaunch: %s", cudaGetErrorString(cudaGetLastError()));
    }
    if (win) {
        cudaStreamAttrValue v = {};
        v.accessPolicyWindow.num_bytes = 0;
        cudaStreamSetAttribute(stream, cudaStreamAttributeAccessPolicyWindow, &v);
    }
    ALB_TRY(lrc);
    if (d_level || d_parent) k_scatter<<<wide.grid, wide.block, 0, stream>>>(a, d_level, d_parent);
    ALB_CK(cudaGetLastError());
    ALB_CK(cudaEventRecord(g->ev1, stream));
    ALB_CK(cudaMemcpyAsync(g->bfs.h_ctl, a.ctl, sizeof(BfsCtl), cudaMemcpyDeviceToHost, stream));
    ALB_CK(cudaStreamSynchronize(stream));
    const BfsCtl &c = *g->bfs.h_ctl;
    if (c.err) return fail(c.err, "BFS aborted on the device (code %d)", c.err);
    if (!c.done) return fail(ALB_ERR_DEVICE, "BFS level loop ended without finishing");
    float ms = 0;
    ALB_CK(cudaEventElapsedTime(&ms, g->ev0, g->ev1));
    g->last_trace_valid = false;
    if (o.trace) {
        const int32_t cnt = std::min(c.trace_len, g->bfs.trace_cap);
        g->last_trace.resize((size_t)cnt);
        if (cnt)
            ALB_CK(cudaMemcpy(g->last_trace.data(), g->bfs.trace, sizeof(alb_level_rec) * cnt,
                              cudaMemcpyDeviceToHost));
        for (int32_t i = 0; i < cnt && i < (int32_t)step_us.size(); i++)
            g->last_trace[i].step_us = step_us[i];
        g->last_trace_valid = true;
    }
    if (st) {
        st->num_levels = c.level;
        st->levels_topdown = c.levels_td;
        st->levels_bottomup = c.levels_bu;
        st->pushed_roots = 0;
        st->reached = c.reached;
        st->edges = c.edges;
        st->ms = ms;
        // init_bulk + init_root (+ scatter), plus the loop's own launches
        st->kernels = 2 + ((d_level || d_parent) ? 1 : 0) +
                      (o.loop == ALB_LOOP_PERSISTENT ? 1 : c.launches);
    }
    return ALB_OK;
}

// Launch the step kernels of one variant for the current level.

// Device copies of the state a level step mutates (restored between variants).
struct LevelSnapshot {
    uint32_t *vis = nullptr, *b0 = nullptr, *b1 = nullptr;
    BfsCtl *ctl = nullptr;
    ~LevelSnapshot() {
        dfree(vis);
        dfree(b0);
        dfree(b1);
        dfree(ctl);
    }
};

alb_status profile_impl(alb_graph *g, int32_t root, const alb_bfs_opts &o, int32_t cap,
                        alb_level_profile *out, int32_t *count) {
    ALB_TRY(bfs_scratch_alloc(g));
    const BfsArgs a = make_args(g);
    const Sell &s = g->sell;
    cudaStream_t st = g->stream;
    const int64_t nw = s.nwords;
    LevelSnapshot snap;
    ALB_TRY(dmalloc((void **)&snap.vis, 4 * nw, "snapshot"));
    ALB_TRY(dmalloc((void **)&snap.b0, 4 * nw, "snapshot"));
    ALB_TRY(dmalloc((void **)&snap.b1, 4 * nw, "snapshot"));
    ALB_TRY(dmalloc((void **)&snap.ctl, sizeof(BfsCtl), "snapshot"));
    InitParams ip;
    std::memset(&ip, 0, sizeof(ip));
    ip.root = root;
    ip.policy = o.policy;
    ip.trace_cap = 0;
    ip.level_cap = (int32_t)std::min<int64_t>(g->n + 1, INT32_MAX - 1);
    ip.alpha = o.alpha;
    ip.beta = o.beta;
    ip.mean_deg = g->n > 0 ? (float)((double)s.m_in / (double)g->n) : 0.f;
    ip.skew = skew_of(s, g->n);
    ip.n_live = g->n - s.zero_in;
    ip.m_in = s.m_in;
    ip.active0 = s.active0;
    const Launch wide = level_launch(g, o.block);
    k_init_bulk<<<wide.grid, wide.block, 0, st>>>(a);
    k_init_root<<<1, 32, 0, st>>>(a, ip);
    ALB_CK(cudaGetLastError());
    BfsCtl *h = g->bfs.h_ctl;
    ALB_CK(cudaMemcpyAsync(h, a.ctl, sizeof(BfsCtl), cudaMemcpyDeviceToHost, st));
    ALB_CK(cudaStreamSynchronize(st));
    cudaEvent_t e0, e1;
    ALB_CK(cudaEventCreate(&e0));
    ALB_CK(cudaEventCreate(&e1));
    auto save = [&](bool back) -> alb_status {
        auto cp = [&](void *dst, const void *src, size_t bytes) {
            return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
        };
        cudaError_t e = back ? cp(a.vis, snap.vis, 4 * nw) : cp(snap.vis, a.vis, 4 * nw);
        if (e == cudaSuccess) e = back ? cp(a.bm0, snap.b0, 4 * nw) : cp(snap.b0, a.bm0, 4 * nw);
        if (e == cudaSuccess) e = back ? cp(a.bm1, snap.b1, 4 * nw) : cp(snap.b1, a.bm1, 4 * nw);
        if (e == cudaSuccess)
            e = back ? cp(a.ctl, snap.ctl, sizeof(BfsCtl)) : cp(snap.ctl, a.ctl, sizeof(BfsCtl));
        if (e != cudaSuccess) return fail(ALB_ERR_CUDA, "profile snapshot: %s", cudaGetErrorString(e));
        return ALB_OK;
    };
    int32_t cnt = 0;
    alb_status rc = ALB_OK;
    while (!h->done && rc == ALB_OK) {
        const BfsCtl hc = *h;
        alb_level_profile prof;
        std::memset(&prof, 0, sizeof(prof));
        rc = save(false);
        for (int v = 0; v < 3 && rc == ALB_OK; v++) {
            if (v) rc = save(true);
            k_decide<<<1, 32, 0, st>>>(a, v, 0);
            cudaEventRecord(e0, st);
            launch_step(a, wide, st, v, hc);
            cudaEventRecord(e1, st);
            cudaError_t e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) rc = fail(ALB_ERR_CUDA, "profile step: %s", cudaGetErrorString(e));
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            prof.us[v] = ms * 1000.f;
        }
        if (rc != ALB_OK) break;
        int best = 0;
        for (int v = 1; v < 3; v++)
            if (prof.us[v] < prof.us[best]) best = v;
        rc = save(true);
        if (rc != ALB_OK) break;
        k_decide<<<1, 32, 0, st>>>(a, best, 0);
        launch_step(a, wide, st, best, hc);
        k_end<<<1, 32, 0, st>>>(a, 0);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, a.ctl, sizeof(BfsCtl), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            rc = fail(ALB_ERR_CUDA, "profile level: %s", cudaGetErrorString(e));
            break;
        }
        prof.best = best;
        prof.rec.dir = best;
        prof.rec.level = hc.level;
        prof.rec.nf = hc.nf;
        prof.rec.mf = hc.mf;
        prof.rec.nu = hc.nu;
        prof.rec.mu = hc.mu;
        prof.rec.active_slices = hc.active_words;
        prof.rec.step_us = prof.us[best];
        level_features(hc, prof.feat);
        if (cnt < cap && out) out[cnt] = prof;
        cnt++;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != ALB_OK) return rc;
    *count = cnt;
    return ALB_OK;
}

alb_status check_bfs_args(alb_graph *g, int32_t root, const alb_bfs_opts *o, alb_bfs_opts &out) {
    if (!g) return fail(ALB_ERR_INVALID, "BFS: graph is NULL");
    if (!g->sell.built) return fail(ALB_ERR_STATE, "BFS: call alb_sell_build first");
    if (root < 0 || root >= g->n)
        return fail(ALB_ERR_INVALID, "BFS: root %d outside [0, %lld)", root, (long long)g->n);
    alb_bfs_opts_default(&out);
    if (o) out = *o;
    if (out.policy < ALB_POLICY_BEAMER || out.policy > ALB_POLICY_BOTTOMUP_NOBYPASS)
        return fail(ALB_ERR_INVALID, "BFS: unknown policy %d", out.policy);
    if (out.loop < ALB_LOOP_HOST || out.loop > ALB_LOOP_PERSISTENT)
        return fail(ALB_ERR_INVALID, "BFS: unknown loop mode %d", out.loop);
    if (!(out.block == 128 || out.block == 256 || out.block == 512 || out.block == 1024))
        return fail(ALB_ERR_UNSUPPORTED, "BFS: block must be 128, 256, 512 or 1024");
    if (!(out.alpha > 0) || !(out.beta > 0))
        return fail(ALB_ERR_INVALID, "BFS: alpha and beta must be positive");
    return ALB_OK;
}

}  // namespace
}  // namespace alb

using namespace alb;

extern "C" {

void alb_bfs_opts_default(alb_bfs_opts *o) {
    if (!o) return;
    o->policy = ALB_POLICY_BEAMER;
    o->loop = ALB_LOOP_GRAPH;
    o->alpha = 14.0f;
    o->beta = 24.0f;
    o->block = 256;
    o->trace = 0;
}

alb_status alb_bfs_device(alb_graph *g, int32_t root, const alb_bfs_opts *o, int32_t *d_level,
                          int32_t *d_parent, alb_stats *st) {
    alb_bfs_opts oo;
    ALB_TRY(check_bfs_args(g, root, o, oo));
    ALB_CK(cudaSetDevice(g->device));
    try {
        return bfs_impl(g, root, oo, d_level, d_parent, st);
    } catch (const std::bad_alloc &) {
        return fail(ALB_ERR_OOM, "alb_bfs_device: host allocation failed");
    }
}

alb_status alb_bfs(alb_graph *g, int32_t root, const alb_bfs_opts *o, int32_t *level,
                   int32_t *parent, alb_stats *st) {
    alb_bfs_opts oo;
    ALB_TRY(check_bfs_args(g, root, o, oo));
    ALB_CK(cudaSetDevice(g->device));
    BfsScratch &b = g->bfs;
    ALB_TRY(bfs_scratch_alloc(g));
    if (level && !b.out_level) ALB_TRY(dmalloc((void **)&b.out_level, sizeof(int32_t) * g->n, "level output"));
    if (parent && !b.out_parent)
        ALB_TRY(dmalloc((void **)&b.out_parent, sizeof(int32_t) * g->n, "parent output"));
    alb_status rc;
    try {
        rc = bfs_impl(g, root, oo, level ? b.out_level : nullptr, parent ? b.out_parent : nullptr, st);
    } catch (const std::bad_alloc &) {
        rc = fail(ALB_ERR_OOM, "alb_bfs: host allocation failed");
    }
    if (rc != ALB_OK) return rc;
    if (level)
        ALB_CK(cudaMemcpyAsync(level, b.out_level, sizeof(int32_t) * g->n, cudaMemcpyDeviceToHost, g->stream));
    if (parent)
        ALB_CK(cudaMemcpyAsync(parent, b.out_parent, sizeof(int32_t) * g->n, cudaMemcpyDeviceToHost,
                               g->stream));
    ALB_CK(cudaStreamSynchronize(g->stream));
    return ALB_OK;
}

alb_status alb_bfs_profile(alb_graph *g, int32_t root, const alb_bfs_opts *o, int32_t cap,
                           alb_level_profile *out, int32_t *count) {
    alb_bfs_opts oo;
    ALB_TRY(check_bfs_args(g, root, o, oo));
    if (!count || (cap > 0 && !out)) return fail(ALB_ERR_INVALID, "alb_bfs_profile: bad output");
    ALB_CK(cudaSetDevice(g->device));
    try {
        return profile_impl(g, root, oo, cap, out, count);
    } catch (const std::bad_alloc &) {
        return fail(ALB_ERR_OOM, "alb_bfs_profile: host allocation failed");
    }
}

alb_status alb_level_trace(const alb_graph *g, int32_t cap, alb_level_rec *out, int32_t *count) {
    if (!g || !count || (cap > 0 && !out)) return fail(ALB_ERR_INVALID, "alb_level_trace: bad arguments");
    if (!g->last_trace_valid) return fail(ALB_ERR_STATE, "alb_level_trace: last BFS ran without trace");
    const int32_t n = (int32_t)g->last_trace.size();
    *count = n;
    const int32_t k = std::min(n, std::max(cap, 0));
    if (k) std::memcpy(out, g->last_trace.data(), sizeof(alb_level_rec) * k);
    return ALB_OK;
}

}  // extern "C"
