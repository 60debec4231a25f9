// Bit-parallel multi-source BFS: up to 64 roots per uint64 word, one pass
// over the SELL-C-sigma matrix per level for all roots. No counterpart in the
// reference (bfs/src/bfs_SELLCSv2.c runs one root from row 0).
//
// Per position p (sorted-position space, as in bfs.cu):
//   V[p]     roots that have visited p (unused root bits preset)
//   S[l][p]  roots whose level-l frontier contains p. S[l] is both the
//            frontier of level l and the record of level l: a root's level at
//            p is the l whose S[l][p] holds its bit, so the int32 output is
//            written once, at the end, as full 256-byte rows.
//   D        one bit per position: V[p] == ~0 (the bypass test)
//   A[l & 1] one bit per position: S[l][p] != 0. The 2 MB-per-2^24-vertex
//            bitmap stays in L2 where the 8-byte frontier words do not, and a
//            bottom-up gather fetches S[l][c] only when c's bit is set.
//
// bottom-up (k_ms_bu): warp per 32 positions; a full D word is skipped; each
//   lane ORs S[l] over its row with 16-byte column loads and stops when every
//   root has visited or reached it ((acc | V) == ~0) or at the row padding.
// top-down (k_ms_td): warp-cooperative push over the frontier queue; targets
//   receive atomicOr(S[l+1][v], S[l][u] & ~V[v]) (64-bit atomics); the first
//   writer of a target appends it to the next queue.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "graph.h"
#include "selector.cuh"

namespace alb {

constexpr uint64_t kAll = ~0ull;
// Packed list counters (rows << kMsBigShift | chunks), as in bfs.cu.
constexpr int kMsBigShift = 38;
constexpr unsigned long long kMsBigMask = (1ull << kMsBigShift) - 1;

struct MsCtl {
    int32_t level, dir, prev_dir, q_valid, done, err, policy, base;  // base: level of S[0]
    float alpha, beta;
    int32_t levels_td, levels_bu;
    int64_t n, nwords;
    int64_t nf, mf, prev_nf, nu, mu, active_words;
    int64_t pairs, edges;  // (vertex, root) pairs reached; sum of their push degrees
    unsigned long long acc_n[3], acc_mo[3], acc_mi[3], acc_full[3], acc_bits[3], acc_edges[3],
        qn[3], acc_bytes[3], acc_done[3], nbig[3], work[3];
    int64_t launches;
    float feat_mean_deg, feat_skew;
    // set for the next level by k_ms_end (and for level 0 by k_ms_roots):
    // frontier-nonzero filter on/off, the CUDA-graph switch branch, and
    // whether the snapshot store must be flushed before the level runs
    int32_t filt, branch, need_flush, level_cap;
    int64_t m_in;
    // Roots whose frontier is small (or empty) at a bottom-up level: the pull
    // does not wait for their bits (a row stops once every other root is
    // accounted for) and a push over their frontier finds their new rows.
    // Chosen by k_ms_end from per-root frontier counts sampled on every
    // kSampleStride-th bitmap word (MsSample, filled by k_ms_sample).
    unsigned long long tmask;
    int32_t grab;  // words per run of the bottom-up pull (8 .. 32)
    // budget of estimated push edges for all tmask roots together (0: off)
    int64_t push_budget;
    unsigned long long used;  // root bits in use
    int32_t pushed_roots;     // sum of popc(tmask) over the levels
    int32_t gtrace_on;        // graph loop: record each level in MsArgs::gtrace
};
static_assert(sizeof(MsCtl) % 8 == 0, "k_ms_end moves the control block in 8-byte words");

// Level records of the CUDA-graph loop (the benchmarked form), written on the
// device: start (k_ms_branch) and end (k_ms_end) %globaltimer stamps, the
// level's algorithmic bytes, its direction, and the frontier and unvisited
// counts it started from.
constexpr int kGTraceCap = 1 << 14;
constexpr int kGTraceW = 8;

// Rows and push degrees of each root's sampled frontier. Kept beside the
// control block (same allocation) so that k_ms_end's copy of it stays small.
struct MsSample {
    unsigned int rows[64];
    unsigned long long deg[64];
};

// Per-root frontier sampling: one bitmap word (32 rows) in kSampleStride.
constexpr int kSampleStride = 32;
constexpr int kSampleMinDiv = 1024;
// Default push budget (all tmask roots together): m_in / kPushDiv estimated
// push edges.
constexpr int kPushDiv = 64;

// Branches of the CUDA-graph level loop's switch node.
// kBrBUWide: the unfiltered pull two column groups at a time, at the first
// bottom-up level after a top-down one (prev_td), where rows scan longest
// before every root is accounted for; at later levels rows stop sooner and
// the second group is mostly fetched for nothing.
enum MsBranch { kBrTD = 0, kBrBUFilt, kBrBU, kBrBUWide, kBrBUNBFilt, kBrBUNB, kBrCount };

__host__ __device__ inline int ms_branch_of(int dir, int filt, bool prev_td) {
    if (dir == ALB_DIR_TOPDOWN) return kBrTD;
    if (dir == ALB_DIR_BOTTOMUP) return filt ? kBrBUFilt : (prev_td ? kBrBUWide : kBrBU);
    return filt ? kBrBUNBFilt : kBrBUNB;
}

struct MsArgs {
    int64_t n, nwords, npad;
    int32_t C, log2C, K;
    int32_t sigma;  // sort window: perm maps each aligned window of sigma rows to itself
    const int32_t *perm, *inv, *ideg, *odeg, *width;
    const int64_t *slice_off;
    const int4 *col4;
    const int64_t *prow;
    const int32_t *pcol;
    int64_t nlong;  // rows kept out of the slices, pulled in chunks
    const int32_t *lrow;
    const int64_t *lptr;
    const int32_t *lcol;
    uint64_t *V;
    uint64_t *S;  // K slots of npad words
    uint32_t *D;
    uint32_t *A;  // 2 x nwords: frontier-nonzero bitmaps by level parity
    int32_t *q0, *q1;
    int32_t *big;  // frontier rows longer than kBigRow (top-down)
    int64_t *big_base;
    MsCtl *ctl;
    MsSample *smp;  // directly after *ctl
    int32_t long_row;  // rows with more sources than this are the long rows
    const float *mlp;
    long long *gtrace;  // kGTraceCap x kGTraceW level records (MsCtl::gtrace_on)
};

__device__ __forceinline__ uint32_t *nz_bits(const MsArgs &a, int L) {
    return a.A + (int64_t)(L & 1) * a.nwords;
}

__device__ __forceinline__ uint64_t *slot(const MsArgs &a, int j) { return a.S + (int64_t)j * a.npad; }

// Level kernels take the slot index j and the filter flag from the host loop,
// or read them from the control block when launched by the CUDA-graph loop
// (passed as -1).
__device__ __forceinline__ int ms_j(const MsArgs &a, int j) {
    return j >= 0 ? j : a.ctl->level - a.ctl->base;
}
__device__ __forceinline__ int ms_filt(const MsArgs &a, int filt) {
    return filt >= 0 ? filt : a.ctl->filt;
}

// Initial state, thread per position: a warp covers one bitmap word (npad and
// the grid stride are multiples of 32), so the done word comes from a ballot.
__global__ void k_ms_init(MsArgs a, uint64_t unused) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t str = (int64_t)gridDim.x * blockDim.x;
    uint64_t *S0 = a.S;
    for (int64_t p = tid; p < a.npad; p += str) {
        const bool live = p < a.n && __ldg(a.ideg + p) > 0;
        a.V[p] = live ? unused : kAll;
        S0[p] = 0;
        const unsigned dead = __ballot_sync(kFull, !live);
        if ((threadIdx.x & 31) == 0) {
            const int64_t w = p >> 5;
            a.D[w] = dead;
            a.A[w] = 0;
            a.A[a.nwords + w] = 0;
        }
    }
}

struct MsInit {
    int32_t roots[64];
    int32_t nroots, policy, level_cap;
    float alpha, beta, mean_deg, skew;
    int64_t n_live, m_in, active0, push_budget;
    int32_t grab;
    int32_t gtrace;  // record the graph loop's levels
};

// One block of 64 threads: thread i seeds root i; thread 0 fills the control block.
__global__ void k_ms_roots(MsArgs a, MsInit in) {
    __shared__ unsigned long long s_nf, s_mf, s_pairs, s_edges, s_done_mi, s_full, s_done_v;
    const int i = threadIdx.x;
    if (i == 0) s_nf = s_mf = s_pairs = s_edges = s_done_mi = s_full = s_done_v = 0;
    a.smp->rows[i] = 0;
    a.smp->deg[i] = 0;
    __syncthreads();
    if (i < in.nroots) {
        const int32_t p = a.inv[in.roots[i]];
        const uint64_t bit = 1ull << i;
        const unsigned long long oldv = atomicOr((unsigned long long *)a.V + p, bit);
        const unsigned long long olds = atomicOr((unsigned long long *)a.S + p, bit);
        if (olds == 0) {
            a.q0[atomicAdd(&s_nf, 1ull)] = p;
            atomicAdd(&s_mf, (unsigned long long)a.odeg[p]);
            atomicOr(a.A + (p >> 5), 1u << (p & 31));  // level 0: A[0]
        }
        // bit i belongs to root i alone, so every root counts once (its bit
        // may already be set in V when p has no sources: V starts full there)
        (void)oldv;
        atomicAdd(&s_pairs, 1ull);
        atomicAdd(&s_edges, (unsigned long long)a.odeg[p]);
    }
    __syncthreads();
    // positions whose every root bit is now set
    if (i < in.nroots) {
        const int32_t p = a.inv[in.roots[i]];
        if (a.V[p] == kAll) {
            const unsigned long long old = atomicOr(&a.D[p >> 5], 1u << (p & 31));
            if (!(old & (1u << (p & 31)))) {
                atomicAdd(&s_done_v, 1ull);
                atomicAdd(&s_done_mi, (unsigned long long)a.ideg[p]);
                if ((old | (1u << (p & 31))) == kFull) atomicAdd(&s_full, 1ull);
            }
        }
    }
    __syncthreads();
    if (i == 0) {
        MsCtl c;
        memset(&c, 0, sizeof(c));
        c.dir = -1;
        c.prev_dir = -1;
        c.q_valid = 1;
        c.policy = in.policy;
        c.alpha = in.alpha;
        c.beta = in.beta;
        c.n = a.n;
        c.nwords = a.nwords;
        c.nf = (int64_t)s_nf;
        c.mf = (int64_t)s_mf;
        c.nu = in.n_live - (int64_t)s_done_v;
        c.mu = in.m_in - (int64_t)s_done_mi;
        c.active_words = in.active0 - (int64_t)s_full;
        c.pairs = (int64_t)s_pairs;
        c.edges = (int64_t)s_edges;
        c.qn[0] = s_nf;
        c.feat_mean_deg = in.mean_deg;
        c.feat_skew = in.skew;
        c.m_in = in.m_in;
        c.level_cap = in.level_cap;
        c.push_budget = in.push_budget;
        c.grab = in.grab;
        c.used = in.nroots >= 64 ? kAll : (1ull << in.nroots) - 1;
        c.gtrace_on = in.gtrace;
        c.done = c.nf == 0;
        // level 0's direction: the rule of later levels (the learned policy
        // falls back to Beamer here: no level has run yet)
        BfsCtl fc;
        memset(&fc, 0, sizeof(fc));
        fc.n = c.n;
        fc.nwords = c.nwords;
        fc.nf = c.nf;
        fc.mf = c.mf;
        fc.nu = c.nu;
        fc.mu = c.mu;
        fc.prev_dir = -1;
        fc.policy = in.policy == ALB_POLICY_LEARNED ? ALB_POLICY_BEAMER : in.policy;
        fc.alpha = in.alpha;
        fc.beta = in.beta;
        c.dir = rule_dir(fc);
        c.filt = c.mf < c.m_in / 8;
        c.branch = ms_branch_of(c.dir, c.filt, false);
        *a.ctl = c;
    }
}

// Words of a bottom-up level in runs of `grab` words (8 to 32, set by the
// host from the word count: about three runs per resident warp) taken from
// the level's counter (dynamic distribution, as WordRuns). The done words of
// a run are loaded together, one per lane, a run ahead of use. kSkip: words
// whose rows are all done are not yielded; their next-frontier words and
// nonzero bits are cleared when the run comes up, one coalesced store per
// word, so a warp does not walk them one dependent round trip at a time (at
// late levels most words are such). Call from all lanes of a warp.
__device__ __forceinline__ int64_t grab_n(unsigned long long *ctr, int step) {
    unsigned long long v = 0;
    if ((threadIdx.x & 31) == 0) v = atomicAdd(ctr, (unsigned long long)step);
    return (int64_t)__shfl_sync(kFull, v, 0);
}

template <bool kSkip>
struct MsWords {
    int64_t cur, nxt;     // first word of the current run and of the next one
    uint32_t dcur, dnxt;  // lane l < step: done word of word cur + l / nxt + l
    unsigned left;        // words of the current run not yet yielded
    int step;             // words per run (<= 32)
    __device__ __forceinline__ uint32_t load(const MsArgs &a, int64_t r) const {
        const int l = threadIdx.x & 31;
        return (l < step && r + l < a.nwords) ? __ldg(a.D + r + l) : kFull;
    }
    __device__ __forceinline__ unsigned prep(const MsArgs &a, uint64_t *N, uint32_t *An) const {
        const int l = threadIdx.x & 31;
        const bool valid = l < step && cur + l < a.nwords;
        const unsigned all = __ballot_sync(kFull, valid);
        if (!kSkip) return all;
        unsigned full = __ballot_sync(kFull, valid && dcur == kFull);
        while (full) {
            const int q = __ffs(full) - 1;
            full &= full - 1;
            N[(cur + q) * 32 + l] = 0;
            if (l == 0) An[cur + q] = 0;
        }
        return __ballot_sync(kFull, valid && dcur != kFull);
    }
    __device__ __forceinline__ void start(const MsArgs &a, uint64_t *N, uint32_t *An,
                                          unsigned long long *ctr) {
        step = a.ctl->grab;
        cur = grab_n(ctr, step);
        nxt = grab_n(ctr, step);
        dcur = load(a, cur);
        dnxt = load(a, nxt);
        left = prep(a, N, An);
    }
    // the next word (a.nwords when the level's words are exhausted) and its
    // done word
    __device__ __forceinline__ int64_t next(const MsArgs &a, uint64_t *N, uint32_t *An,
                                            unsigned long long *ctr, uint32_t &d) {
        while (!left) {
            if (cur >= a.nwords) {
                d = kFull;
                return a.nwords;
            }
            cur = nxt;
            dcur = dnxt;
            if (cur < a.nwords) {
                nxt = grab_n(ctr, step);
                dnxt = load(a, nxt);
            }
            left = prep(a, N, An);
        }
        const int q = __ffs(left) - 1;
        left &= left - 1;
        d = __shfl_sync(kFull, dcur, q);
        return cur + q;
    }
};

// Bottom-up over S[j] -> S[j+1]. kBypass: skip words whose 32 positions are
// done; kEarly: stop a row once every root is accounted for, or at padding.
// kFilt: test the nonzero bitmap before each 8-byte frontier fetch. It pays
// when few sources are in the frontier (the fetches it saves miss L2) and
// costs a dependent round trip per group when most are, so the host picks it
// from the frontier's share of all entries.
// Launched with kMsBuBlock threads; the bound keeps it at 48 registers
// (5 blocks, 40 warps per SM) without spills.
constexpr int kMsBuBlock = 256;

// kWide (with !kFilt): two column groups per step, eight frontier fetches in
// flight per lane, at four blocks per SM.
template <bool kBypass, bool kEarly, bool kFilt, bool kWide = false>
__global__ void __launch_bounds__(kMsBuBlock, kWide ? 4 : 5) k_ms_bu(MsArgs a, int j) {
    j = ms_j(a, j);
    const uint64_t *F = slot(a, j);
    uint64_t *N = slot(a, j + 1);
    const int lane = threadIdx.x & 31;
    const int L = a.ctl->level;
    const int k = (L + 1) % 3;
    const uint64_t tm = a.ctl->tmask;
    const uint32_t *Az = nz_bits(a, L);
    uint32_t *An = nz_bits(a, L + 1);
    // per-thread counts fit 32 bits; degree sums and bytes need 64
    unsigned cn = 0, cbits = 0, cfull = 0, cdone = 0;
    unsigned long long cmo = 0, cmi = 0, cedges = 0, bytes = 0;
    const uint64_t pol = l2_evict_first();
    // words come in runs from the level's counter (MsWords, done words
    // skipped when kBypass). Software pipeline over words: the visited words
    // and slice geometry are requested one word ahead, so their latency
    // overlaps the current word's column loads and gathers.
    unsigned long long *ctr = &a.ctl->work[L % 3];
    MsWords<kBypass> it;
    it.start(a, N, An, ctr);
    auto geometry = [&](int64_t ww, uint32_t dd, uint64_t &vv, int32_t &wdv, int64_t &sov) {
        vv = kAll;
        wdv = 0;
        sov = 0;
        if (ww < a.nwords && !(kBypass && dd == kFull)) {
            const int64_t pw = ww * 32 + lane;
            // rows past n (padding of the last word) are preset visited;
            // their slice index is clamped so the loads stay in bounds
            const int64_t sw = (pw < a.n ? pw : a.n - 1) >> a.log2C;
            vv = __ldg(a.V + pw);
            wdv = __ldg(a.width + sw);
            sov = __ldg(a.slice_off + sw);
        }
    };
    uint32_t d, d1 = kFull;
    int64_t w = it.next(a, N, An, ctr, d);
    int64_t w1 = w < a.nwords ? it.next(a, N, An, ctr, d1) : a.nwords;
    uint64_t vis_c;
    int32_t wd_c;
    int64_t so_c;
    geometry(w, d, vis_c, wd_c, so_c);
    while (w < a.nwords) {
        uint64_t vis1;
        int32_t wd1;
        int64_t so1;
        geometry(w1, d1, vis1, wd1, so1);
        const int64_t p = w * 32 + lane;
        if (kBypass && d == kFull) {  // not reached: MsWords clears these words
            N[p] = 0;
            if (lane == 0) An[w] = 0;
        } else {
            bytes += 8;  // V[p]
            const uint64_t vis = vis_c;
            // roots in tmask are found by the push over their frontier
            const uint64_t visx = vis | tm;
            bool active = visx != kAll;
            int32_t ng = active ? (wd_c + 3) >> 2 : 0;
            const int4 *cp = a.col4 + (so_c >> 2) + (p & (a.C - 1));
            uint64_t acc = 0;
            // group g+1 is requested before group g's frontier fetches, so each
            // lane keeps a column load in flight while it waits on the gathers
            const int32_t pp = (int32_t)p;
            if (kWide && !kFilt) {
                const int4 pad = make_int4(pp, pp, pp, pp);
                int4 c0 = pad, c1 = pad;
                if (active && ng > 0) c0 = ld_stream(cp, pol);
                if (active && ng > 1) c1 = ld_stream(cp + a.C, pol);
                for (int32_t g = 0;; g += 2) {
                    active = active && g < ng;
                    if (!__any_sync(kFull, active)) break;
                    if (!active) continue;
                    int4 n0 = pad, n1 = pad;
                    if (g + 2 < ng) n0 = ld_stream(cp + (int64_t)(g + 2) * a.C, pol);
                    if (g + 3 < ng) n1 = ld_stream(cp + (int64_t)(g + 3) * a.C, pol);
                    ALB_CHECK_ID4(c0, a.npad, pp, &a.ctl->err);
                    ALB_CHECK_ID4(c1, a.npad, pp, &a.ctl->err);
                    // past the row's last group c1 is padding (p itself)
                    acc |= __ldg(F + c0.x) | __ldg(F + c0.y) | __ldg(F + c0.z) | __ldg(F + c0.w) |
                           __ldg(F + c1.x) | __ldg(F + c1.y) | __ldg(F + c1.z) | __ldg(F + c1.w);
                    bytes += g + 1 < ng ? 96 : 48;
                    if (kEarly && (c1.w == pp || (acc | visx) == kAll)) active = false;
                    c0 = n0;
                    c1 = n1;
                }
                ng = 0;  // the single-group loop below has nothing left
            }
            int4 c = make_int4(pp, pp, pp, pp);
            if (active && ng > 0) c = ld_stream(cp, pol);
            for (int32_t g = 0;; g++) {
                active = active && g < ng;
                if (!__any_sync(kFull, active)) break;
                if (!active) continue;
                int4 nx = make_int4(pp, pp, pp, pp);
                if (g + 1 < ng) nx = ld_stream(cp + (int64_t)(g + 1) * a.C, pol);
                // padding entries hold p itself: S[j][p] only has bits already in
                // V[p], so OR-ing it changes nothing
                ALB_CHECK_ID4(c, a.npad, pp, &a.ctl->err);
                if (kFilt) {
                    const uint32_t z0 = __ldg(Az + (c.x >> 5)), z1 = __ldg(Az + (c.y >> 5)),
                                   z2 = __ldg(Az + (c.z >> 5)), z3 = __ldg(Az + (c.w >> 5));
                    const bool h0 = (z0 >> (c.x & 31)) & 1u, h1 = (z1 >> (c.y & 31)) & 1u,
                               h2 = (z2 >> (c.z & 31)) & 1u, h3 = (z3 >> (c.w & 31)) & 1u;
                    if (h0) acc |= __ldg(F + c.x);
                    if (h1) acc |= __ldg(F + c.y);
                    if (h2) acc |= __ldg(F + c.z);
                    if (h3) acc |= __ldg(F + c.w);
                    // four columns, four bitmap words, the frontier words fetched
                    bytes += 32 + 8 * (h0 + h1 + h2 + h3);
                } else {
                    acc |= __ldg(F + c.x) | __ldg(F + c.y) | __ldg(F + c.z) | __ldg(F + c.w);
                    bytes += 48;  // four columns and their four frontier words
                }
                if (kEarly && (c.w == pp || (acc | visx) == kAll)) active = false;
                c = nx;
            }
            const uint64_t nb = acc & ~vis;
            N[p] = nb;
            const unsigned nzm = __ballot_sync(kFull, nb != 0);
            if (lane == 0) An[w] = nzm;
            bool done_now = false;
            if (nb) {
                const uint64_t nv = vis | nb;
                a.V[p] = nv;
                const int pc = __popcll(nb);
                const int32_t od = __ldg(a.odeg + p);
                bytes += 12;  // V[p] written, push degree
                cn++;
                cbits += pc;
                cmo += od;
                cedges += (unsigned long long)pc * od;
                if (nv == kAll) {
                    done_now = true;
                    cdone++;
                    cmi += __ldg(a.ideg + p);
                }
            }
            const unsigned dm = __ballot_sync(kFull, done_now);
            if (lane == 0 && dm) {
                a.D[w] = d | dm;
                cfull += (d != kFull && (d | dm) == kFull);
            }
        }
        w = w1;
        d = d1;
        vis_c = vis1;
        wd_c = wd1;
        so_c = so1;
        w1 = w1 < a.nwords ? it.next(a, N, An, ctr, d1) : a.nwords;
    }
    cn = warp_sum(cn);
    cbits = warp_sum(cbits);
    cmo = warp_sum(cmo);
    cmi = warp_sum(cmi);
    cedges = warp_sum(cedges);
    cdone = warp_sum(cdone);
    bytes = warp_sum(bytes);
    if (lane == 0) {
        if (cn) {
            atomicAdd(&a.ctl->acc_n[k], (unsigned long long)cn);
            atomicAdd(&a.ctl->acc_bits[k], (unsigned long long)cbits);
            atomicAdd(&a.ctl->acc_mo[k], cmo);
            atomicAdd(&a.ctl->acc_mi[k], cmi);
            atomicAdd(&a.ctl->acc_edges[k], cedges);
            if (cdone) atomicAdd(&a.ctl->acc_done[k], (unsigned long long)cdone);
        }
        if (cfull) atomicAdd(&a.ctl->acc_full[k], (unsigned long long)cfull);
        if (bytes) atomicAdd(&a.ctl->acc_bytes[k], bytes);
    }
}

__device__ __forceinline__ uint64_t warp_or64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v |= __shfl_xor_sync(kFull, v, o);
    return v;
}

// Long rows (kept out of the slices), head pass: one warp per long row some
// root has not visited ORs the frontier words of its first kLongChunk
// sources, 32 per step (fetched where the nonzero bitmap has a bit when filt
// is set), and stops once every root is accounted for. New bits go into N[p]
// by atomicOr (the slice pass wrote 0 there). A row still missing roots with
// sources left joins the continuation list (nbig[L % 3], big, big_base) for
// k_ms_bu_long_tail; k_ms_bu_long_fin folds N[p] into the state.
// Sources [st, en) of one long row, 128 per step: each lane loads four
// source ids, then their four frontier words, all before using any of them,
// and keeps a private OR; the warp combines the lanes once per step.
template <bool kEarly>
__device__ __forceinline__ uint64_t ms_long_scan(const MsArgs &a, const uint64_t *F,
                                                 const uint32_t *Az, int filt, int64_t st,
                                                 int64_t en, uint64_t acc, uint64_t vis,
                                                 unsigned long long &bytes) {
    const int lane = threadIdx.x & 31;
    uint64_t mine = 0;
    for (int64_t e0 = st; e0 < en; e0 += 128) {
        int32_t c[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int64_t e = e0 + 32 * u + lane;
            c[u] = e < en ? __ldg(a.lcol + e) : -1;
            if (c[u] >= 0) ALB_CHECK_ID(c[u], a.n, -1, &a.ctl->err);
        }
        int fetched = 0;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (c[u] >= 0 && (!filt || ((__ldg(Az + (c[u] >> 5)) >> (c[u] & 31)) & 1u))) {
                mine |= __ldg(F + c[u]);
                fetched++;
            }
        }
        // columns (and bitmap words when filtering), frontier words fetched
        const int64_t ne = min((int64_t)128, en - e0);
        bytes += (filt ? 8 : 4) * ne + 8 * (unsigned long long)warp_sum(fetched);
        if (kEarly && ((acc | warp_or64(mine)) | vis) == kAll) break;
    }
    return acc | warp_or64(mine);
}

// Counters of the long rows folded in one level (per thread).
struct MsLongCounts {
    unsigned long long cn = 0, cbits = 0, cmo = 0, cmi = 0, cfull = 0, cedges = 0, cdone = 0;
    unsigned long long bytes = 0;  // algorithmic bytes, where the kernel counts them here
    __device__ void flush(const MsArgs &a, int k) {
        cn = warp_sum(cn);
        cbits = warp_sum(cbits);
        cmo = warp_sum(cmo);
        cmi = warp_sum(cmi);
        cfull = warp_sum(cfull);
        cedges = warp_sum(cedges);
        cdone = warp_sum(cdone);
        bytes = warp_sum(bytes);
        if ((threadIdx.x & 31) == 0 && bytes) atomicAdd(&a.ctl->acc_bytes[k], bytes);
        if ((threadIdx.x & 31) == 0 && (cn | cbits | cdone)) {
            atomicAdd(&a.ctl->acc_n[k], cn);
            atomicAdd(&a.ctl->acc_bits[k], cbits);
            atomicAdd(&a.ctl->acc_mo[k], cmo);
            atomicAdd(&a.ctl->acc_mi[k], cmi);
            atomicAdd(&a.ctl->acc_edges[k], cedges);
            if (cdone) atomicAdd(&a.ctl->acc_done[k], cdone);
            if (cfull) atomicAdd(&a.ctl->acc_full[k], cfull);
        }
    }
};

// Long row p reached by the roots nb (not in vis) this level: visited word,
// nonzero and done bitmaps, counters. One thread per row.
__device__ __forceinline__ void ms_long_fold(const MsArgs &a, int32_t p, uint64_t nb, uint64_t vis,
                                             uint32_t *An, MsLongCounts &c) {
    const uint64_t nv = vis | nb;
    a.V[p] = nv;
    const uint32_t bit = 1u << (p & 31);
    atomicOr(An + (p >> 5), bit);
    const int pc = __popcll(nb);
    const int32_t od = __ldg(a.odeg + p);
    c.cn++;
    c.cbits += pc;
    c.cmo += od;
    c.cedges += (unsigned long long)pc * od;
    if (nv == kAll) {
        c.cdone++;
        c.cmi += __ldg(a.ideg + p);
        const uint32_t od2 = atomicOr(a.D + (p >> 5), bit);
        c.cfull += (od2 != kFull && (od2 | bit) == kFull);
    }
}

// Head pass over the long rows: a warp loads the position, visited word and
// offsets of 32 of its rows at once (one per lane), then scans the first
// kLongChunk sources of every one some root has not visited. A row settled
// by its head (every root accounted for, or no sources left) is folded in
// here; the rest go on the continuation list for k_ms_bu_long_tail with their
// new bits ORed into N[p], and k_ms_bu_long_fin folds them in.
template <bool kEarly>
__global__ void k_ms_bu_long(MsArgs a, int j, int filt) {
    j = ms_j(a, j);
    filt = ms_filt(a, filt);
    if (a.nlong == 0) return;
    const uint64_t *F = slot(a, j);
    uint64_t *N = slot(a, j + 1);
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    const int L = a.ctl->level;
    const uint64_t tm = a.ctl->tmask;  // roots the push handles: not waited for
    const uint32_t *Az = nz_bits(a, L);
    uint32_t *An = nz_bits(a, L + 1);
    unsigned long long *cont = &a.ctl->nbig[L % 3];
    unsigned long long bytes = 0;
    MsLongCounts cnt;
    // rows stay strided over the warps (row gw + k * nwarps goes to warp gw),
    // but a warp loads the metadata of its next 32 rows at once, one per lane
    const int64_t gw = blockIdx.x * wpb + (threadIdx.x >> 5);
    for (int64_t i0 = gw; i0 < a.nlong; i0 += 32 * nwarps) {
        const int64_t i = i0 + lane * nwarps;
        int32_t p_l = 0;
        uint64_t vis_l = kAll;
        int64_t st_l = 0, en_l = 0;
        if (i < a.nlong) {
            p_l = __ldg(a.lrow + i);
            st_l = __ldg(a.lptr + i);
            en_l = __ldg(a.lptr + i + 1);
            vis_l = __ldg(a.V + p_l);
        }
        unsigned todo = __ballot_sync(kFull, (vis_l | tm) != kAll);
        while (todo) {
            const int b = __ffs(todo) - 1;
            todo &= todo - 1;
            const int32_t p = __shfl_sync(kFull, p_l, b);
            const uint64_t vis = __shfl_sync(kFull, vis_l, b);
            const int64_t st = __shfl_sync(kFull, st_l, b), en = __shfl_sync(kFull, en_l, b);
            const int64_t hen = min(en, st + kLongChunk);
            bytes += 24;
            const uint64_t acc =
                ms_long_scan<kEarly>(a, F, Az, filt, st, hen, 0ull, vis | tm, bytes);
            const uint64_t nb = acc & ~vis;
            if (lane == 0) {
                if ((acc | vis | tm) != kAll && hen < en) {
                    if (nb) atomicOr((unsigned long long *)N + p, (unsigned long long)nb);
                    const unsigned long long nch =
                        (unsigned long long)((en - hen + kLongChunk - 1) / kLongChunk);
                    const unsigned long long old = atomicAdd(cont, (1ull << kMsBigShift) | nch);
                    const int64_t idx = (int64_t)(old >> kMsBigShift);
                    a.big[idx] = (int32_t)(i0 + b * nwarps);
                    a.big_base[idx] = (int64_t)(old & kMsBigMask);
                } else if (nb) {
                    N[p] = nb;  // the slice pass wrote 0 here
                    ms_long_fold(a, p, nb, vis, An, cnt);
                }
            }
        }
    }
    cnt.flush(a, (L + 1) % 3);
    if (lane == 0 && bytes) atomicAdd(&a.ctl->acc_bytes[(L + 1) % 3], bytes);
}

// Tail pass: chunk k of continuation entry jj covers sources
// [lptr[i] + (1 + k - big_base[jj]) * kLongChunk, ...) of long row i = big[jj];
// the scan starts from the bits N[p] already holds so it can stop early.
template <bool kEarly>
__global__ void k_ms_bu_long_tail(MsArgs a, int j, int filt) {
    j = ms_j(a, j);
    filt = ms_filt(a, filt);
    const int L = a.ctl->level;
    const unsigned long long ctr = a.ctl->nbig[L % 3];
    if (ctr == 0) return;
    const int64_t nrows = (int64_t)(ctr >> kMsBigShift);
    const int64_t total = (int64_t)(ctr & kMsBigMask);
    const uint64_t *F = slot(a, j);
    uint64_t *N = slot(a, j + 1);
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    const uint32_t *Az = nz_bits(a, L);
    const uint64_t tm = a.ctl->tmask;  // roots the push handles: not waited for
    unsigned long long bytes = 0;
    for (int64_t k = blockIdx.x * wpb + (threadIdx.x >> 5); k < total; k += nwarps) {
        int64_t lo = 0, hi = nrows - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (a.big_base[mid] <= k) lo = mid;
            else hi = mid - 1;
        }
        const int32_t i = a.big[lo];
        const int32_t p = __ldg(a.lrow + i);
        const uint64_t vis = __ldg(a.V + p);
        const uint64_t have = __ldcg((const unsigned long long *)N + p);
        if ((have | vis | tm) == kAll) continue;
        const int64_t st = __ldg(a.lptr + i) + (1 + k - a.big_base[lo]) * kLongChunk;
        const int64_t en = min(__ldg(a.lptr + i + 1), st + kLongChunk);
        bytes += 24;
        const uint64_t acc = ms_long_scan<kEarly>(a, F, Az, filt, st, en, have, vis | tm, bytes);
        const uint64_t nb = acc & ~vis & ~have;
        if (lane == 0 && nb) atomicOr((unsigned long long *)N + p, (unsigned long long)nb);
    }
    if (lane == 0 && bytes) atomicAdd(&a.ctl->acc_bytes[(L + 1) % 3], bytes);
}

// Long rows on the continuation list: thread per entry folds N[p] (head and
// tail bits) into the state.
__global__ void k_ms_bu_long_fin(MsArgs a, int j) {
    j = ms_j(a, j);
    const int L = a.ctl->level;
    const unsigned long long ctr = a.ctl->nbig[L % 3];
    if (ctr == 0) return;
    const int64_t nrows = (int64_t)(ctr >> kMsBigShift);
    const uint64_t *N = slot(a, j + 1);
    uint32_t *An = nz_bits(a, L + 1);
    MsLongCounts cnt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nrows;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t p = __ldg(a.lrow + a.big[e]);
        const uint64_t nb = N[p];
        if (nb) ms_long_fold(a, p, nb, a.V[p], An, cnt);
    }
    cnt.flush(a, (L + 1) % 3);
}

// Frontier-nonzero bitmap A[M & 1] -> queue of level M (M = L + ahead):
// thread per bitmap word, prefix sums within the warp, one atomic per warp.
// ahead = 0 rebuilds the current queue before a top-down level that follows
// a bottom-up one; ahead = 1 builds the next queue after a top-down level
// (whose pushes only mark the bitmap, so no atomic counter is shared by
// every claim).
__global__ void k_ms_compact(MsArgs a, int ahead) {
    if (ahead == 0 && a.ctl->q_valid) return;  // the queue already lists the frontier
    const int M = a.ctl->level + ahead;
    const uint32_t *Az = nz_bits(a, M);
    int32_t *Q = (M & 1) ? a.q1 : a.q0;
    unsigned long long *qslot = &a.ctl->qn[M % 3];
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // warp-uniform bound: every lane reaches the shuffles
    for (int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) & ~31ll; w0 < a.nwords;
         w0 += stride) {
        const int64_t w = w0 + lane;
        uint32_t m = w < a.nwords ? __ldg(Az + w) : 0u;
        const int64_t cnt = __popc(m);
        const int64_t inc = warp_inclusive_scan(cnt);
        const int64_t total = __shfl_sync(kFull, inc, 31);
        if (total == 0) continue;
        unsigned long long base = 0;
        if (lane == 31) base = atomicAdd(qslot, (unsigned long long)total);
        base = __shfl_sync(kFull, base, 31);
        int64_t o = (int64_t)base + inc - cnt;
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            Q[o++] = (int32_t)(w * 32 + b);
        }
    }
}

// Push of the roots in tmask during a bottom-up level (after the pull): the
// roots nb reach v (nb: the edge's roots not in v's visited word as read).
// The new roots are claimed on V[v] itself (atomicOr), so concurrent pushers
// and the pull's own discoveries are never counted twice, and the level's
// state and counters are updated in place.
__device__ __forceinline__ void ms_tclaim(const MsArgs &a, uint64_t *N, uint32_t *An, int32_t v,
                                          uint64_t nb, MsLongCounts &c) {
    if (!nb) return;
    const uint32_t bit = 1u << (v & 31);
    const uint64_t oldv = atomicOr((unsigned long long *)a.V + v, (unsigned long long)nb);
    nb &= ~oldv;
    if (!nb) return;
    const uint64_t oldn = atomicOr((unsigned long long *)N + v, (unsigned long long)nb);
    c.bytes += 16;  // V and N words written
    const int pc = __popcll(nb);
    const int32_t od = __ldg(a.odeg + v);
    c.cbits += pc;
    c.cedges += (unsigned long long)pc * od;
    if (oldn == 0) {  // v enters the next frontier
        c.cn++;
        c.cmo += od;
        atomicOr(An + (v >> 5), bit);
    }
    if ((oldv | nb) == kAll) {
        c.cdone++;
        c.cmi += __ldg(a.ideg + v);
        const uint32_t od2 = atomicOr(a.D + (v >> 5), bit);
        c.cfull += (od2 != kFull && (od2 | bit) == kFull);
    }
}

// Four pushed edges per lane (v[k] < 0: none), roots f[k] reaching v[k]
// this level: the done words and the target words of all four are requested
// before the first atomic, so one lane keeps eight loads in flight instead
// of two. Top-down (kPush false): only two small words are read per edge,
// v's done bit (D, 1 bit per row, stays in L2) and N[v] (so that the many
// pushes into a hub stop issuing atomics once its word holds their bits); f
// is ORed in without masking by V[v], and k_ms_td_finish removes the roots
// that had already visited v. A push that finds N[v] empty marks v in the
// next nonzero bitmap An (setting a bit is idempotent, so racing pushers need
// no claim); the next queue is compacted from An afterwards. kPush: the push
// of the tmask roots, ms_tclaim against V (D can change during that kernel
// and is read through L2).
template <bool kPush>
__device__ __forceinline__ void ms_push4(const MsArgs &a, uint64_t *N, uint32_t *An,
                                         const int32_t (&v)[4], const uint64_t (&f)[4],
                                         MsLongCounts &c) {
    uint32_t dw[4];
    uint64_t cur[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        dw[k] = kFull;
        cur[k] = 0;
        if (v[k] >= 0) {
            dw[k] = kPush ? __ldcg(a.D + (v[k] >> 5)) : __ldg(a.D + (v[k] >> 5));
            cur[k] = __ldcg((const unsigned long long *)(kPush ? a.V : N) + v[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (v[k] < 0 || ((dw[k] >> (v[k] & 31)) & 1u)) continue;  // every root has visited v
        if (kPush) {
            c.bytes += 16;  // column, done bit, visited probe
            ms_tclaim(a, N, An, v[k], f[k] & ~cur[k], c);
        } else if (f[k] & ~cur[k]) {
            atomicOr((unsigned long long *)N + v[k], (unsigned long long)f[k]);
            if (!cur[k]) atomicOr(An + (v[k] >> 5), 1u << (v[k] & 31));
        }
    }
}

// Top-down push over the frontier queue. kPush: the push of a bottom-up
// level's tmask roots, over the queue k_ms_tq built (next-parity queue and
// counters, which that level leaves unused), with the state updated in place.
template <bool kPush>
__global__ void k_ms_td(MsArgs a, int j) {
    j = ms_j(a, j);
    const uint64_t *F = slot(a, j);
    uint64_t *N = slot(a, j + 1);
    const int L = a.ctl->level;
    const uint64_t tm = kPush ? a.ctl->tmask : kAll;
    if (kPush && !tm) return;
    const int qp = kPush ? L + 1 : L;
    const int32_t *Q = (qp & 1) ? a.q1 : a.q0;
    const int64_t qlen = (int64_t)a.ctl->qn[qp % 3];
    uint32_t *An = nz_bits(a, L + 1);
    unsigned long long *big_slot = &a.ctl->nbig[qp % 3];
    MsLongCounts cnt;
    __shared__ int64_t s_ex[32][32];
    __shared__ int64_t s_st[32][32];
    __shared__ uint64_t s_f[32][32];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    int G = 32;  // frontier rows per warp: enough to keep every warp busy
    while (G > 1 && (int64_t)(G >> 1) * nwarps >= qlen) G >>= 1;
    const int64_t stride = nwarps * G;
    for (int64_t cb = (blockIdx.x * wpb + wib) * G; cb < qlen; cb += stride) {
        const int64_t i = cb + lane;
        int32_t u = (lane < G && i < qlen) ? Q[i] : -1;
        if (u >= 0) ALB_CHECK_ID(u, a.n, -1, &a.ctl->err);
        int64_t st = 0, d = 0;
        uint64_t f = 0;
        if (u >= 0) {
            st = __ldg(a.prow + u);
            d = __ldg(a.prow + u + 1) - st;
            f = __ldg(F + u) & tm;
            if (kPush) cnt.bytes += 20;  // queue entry, row offsets, frontier word
            if (d > kBigRow) {  // pushed in chunks by all warps in k_ms_td_big
                const unsigned long long nch = (unsigned long long)((d + kBigChunk - 1) / kBigChunk);
                const unsigned long long old = atomicAdd(big_slot, (1ull << kMsBigShift) | nch);
                const int64_t idx = (int64_t)(old >> kMsBigShift);
                a.big[idx] = u;
                a.big_base[idx] = (int64_t)(old & kMsBigMask);
                d = 0;
            }
        }
        const int64_t inc = warp_inclusive_scan(d);
        const int64_t T = __shfl_sync(kFull, inc, 31);
        s_ex[wib][lane] = inc - d;
        s_st[wib][lane] = st;
        s_f[wib][lane] = f;
        __syncwarp();
        for (int64_t e0 = lane; e0 < T; e0 += 128) {
            int32_t v[4];
            uint64_t ff[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int64_t e = e0 + 32 * k;
                v[k] = -1;
                ff[k] = 0;
                if (e < T) {
                    int jj = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1)
                        if (s_ex[wib][jj + step] <= e) jj += step;
                    v[k] = __ldg(a.pcol + s_st[wib][jj] + (e - s_ex[wib][jj]));
                    ALB_CHECK_ID(v[k], a.n, -1, &a.ctl->err);
                    ff[k] = s_f[wib][jj];
                }
            }
            ms_push4<kPush>(a, N, An, v, ff, cnt);
        }
        __syncwarp();
    }
    if (kPush) cnt.flush(a, (L + 1) % 3);
}

// Long frontier rows in kBigChunk-edge chunks over all warps. Each warp
// takes a contiguous run of chunks: it finds the row of its first chunk by
// binary search over the chunk bases (monotone in the list index) and walks
// forward from there.
template <bool kPush>
__global__ void k_ms_td_big(MsArgs a, int j) {
    j = ms_j(a, j);
    const int L = a.ctl->level;
    const unsigned long long ctr = a.ctl->nbig[(kPush ? L + 1 : L) % 3];
    if (ctr == 0) return;
    const uint64_t tm = kPush ? a.ctl->tmask : kAll;
    const int64_t nbig = (int64_t)(ctr >> kMsBigShift);
    const int64_t total = (int64_t)(ctr & kMsBigMask);
    const uint64_t *F = slot(a, j);
    uint64_t *N = slot(a, j + 1);
    uint32_t *An = nz_bits(a, L + 1);
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t gw = blockIdx.x * wpb + (threadIdx.x >> 5);
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    const int64_t per = (total + nwarps - 1) / nwarps;
    const int64_t k0 = gw * per, k1 = min(total, k0 + per);
    if (k0 >= k1) return;  // warp-uniform: whole warps leave
    MsLongCounts cnt;
    int64_t lo = 0, hi = nbig - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (a.big_base[mid] <= k0) lo = mid;
        else hi = mid - 1;
    }
    int64_t base = a.big_base[lo];
    int64_t next = lo + 1 < nbig ? a.big_base[lo + 1] : total;
    int32_t u = a.big[lo];
    int64_t st = __ldg(a.prow + u), d = __ldg(a.prow + u + 1) - st;
    uint64_t f = __ldg(F + u) & tm;
    for (int64_t k = k0; k < k1; k++) {
        while (k >= next) {  // the run crosses into the next long row
            lo++;
            base = next;
            next = lo + 1 < nbig ? a.big_base[lo + 1] : total;
            u = a.big[lo];
            st = __ldg(a.prow + u);
            d = __ldg(a.prow + u + 1) - st;
            f = __ldg(F + u) & tm;
        }
        const int64_t c = k - base;
        const int64_t e1 = min(d, (c + 1) * kBigChunk);
        static_assert(kBigChunk == 128, "four edges per lane per chunk");
        int32_t v[4];
        uint64_t ff[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int64_t e = c * kBigChunk + 32 * q + lane;
            v[q] = e < e1 ? __ldg(a.pcol + st + e) : -1;
            if (v[q] >= 0) ALB_CHECK_ID(v[q], a.n, -1, &a.ctl->err);
            ff[q] = f;
        }
        ms_push4<kPush>(a, N, An, v, ff, cnt);
    }
    if (kPush) cnt.flush(a, (L + 1) % 3);
}

// After a top-down level: fold the new frontier words into V and count.
__global__ void k_ms_td_finish(MsArgs a, int j) {
    j = ms_j(a, j);
    uint64_t *N = slot(a, j + 1);
    const int L = a.ctl->level;
    const int32_t *NQ = (L & 1) ? a.q0 : a.q1;
    const int64_t nqlen = (int64_t)a.ctl->qn[(L + 1) % 3];
    const int k = (L + 1) % 3;
    unsigned long long cn = 0, cbits = 0, cmo = 0, cmi = 0, cfull = 0, cedges = 0, cdone = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nqlen;
         i += (int64_t)gridDim.x * blockDim.x) {
        int32_t v = NQ[i];
        ALB_CHECK_ID(v, a.n, -1, &a.ctl->err);
        if (v < 0) continue;
        const uint64_t raw = N[v];
        const uint64_t old = a.V[v];  // only this thread writes V[v] in this kernel
        const uint64_t nb = raw & ~old;  // the pushes did not mask by V
        if (nb != raw) N[v] = nb;
        if (!nb) {  // reached only by roots that had visited it: not in the frontier
            atomicAnd(nz_bits(a, L + 1) + (v >> 5), ~(1u << (v & 31)));
            continue;
        }
        const uint64_t nv = old | nb;
        a.V[v] = nv;
        const int pc = __popcll(nb);
        const int32_t od = __ldg(a.odeg + v);
        cn++;
        cbits += pc;
        cmo += od;
        cedges += (unsigned long long)pc * od;
        if (nv == kAll && old != kAll) {
            cdone++;
            cmi += __ldg(a.ideg + v);
            const uint32_t bit = 1u << (v & 31);
            const uint32_t od2 = atomicOr(a.D + (v >> 5), bit);
            cfull += (od2 != kFull && (od2 | bit) == kFull);
        }
    }
    cn = warp_sum(cn);
    cbits = warp_sum(cbits);
    cmo = warp_sum(cmo);
    cmi = warp_sum(cmi);
    cfull = warp_sum(cfull);
    cedges = warp_sum(cedges);
    cdone = warp_sum(cdone);
    if ((threadIdx.x & 31) == 0 && (cn || cfull)) {
        atomicAdd(&a.ctl->acc_done[k], cdone);
        atomicAdd(&a.ctl->acc_n[k], cn);
        atomicAdd(&a.ctl->acc_bits[k], cbits);
        atomicAdd(&a.ctl->acc_mo[k], cmo);
        atomicAdd(&a.ctl->acc_mi[k], cmi);
        atomicAdd(&a.ctl->acc_edges[k], cedges);
        if (cfull) atomicAdd(&a.ctl->acc_full[k], cfull);
    }
}

// Per-root size of the frontier level L produced (S[j+1]) for k_ms_end's
// choice of pushed roots, in rows and push degrees (MsSample). The long rows
// are counted exactly (they carry most of the degree in a skewed graph); the
// others on one bitmap word in every kSampleStride, scaled by the stride. The
// sampled word's offset inside its stride cycles with the stride index: rows
// are sorted by length inside sigma windows, and a fixed offset would sample
// one rank of length only. Warp per sampled word or per 32 long rows; lane i
// keeps roots i and i + 32.
constexpr int kSampleBlock = 256;

// dir: the direction level L ran (-1: the one in the control block).
__global__ void __launch_bounds__(kSampleBlock) k_ms_sample(MsArgs a, int j, int dir) {
    __shared__ unsigned s_cnt[64];
    __shared__ unsigned long long s_deg[64];
    // the graph loop's pass after the last level: no next slot to read
    if (a.ctl->done) return;
    // only a top-down level can be followed by a level with pushed roots
    if (dir < 0) dir = a.ctl->dir;
    if (a.ctl->push_budget <= 0 || dir != ALB_DIR_TOPDOWN) return;
    // a frontier under n / kSampleMinDiv rows is not sampled: every root's
    // estimate stays 0, and a bottom-up level after it pushes all of them
    // (a push over so few rows is cheaper than any pull)
    const int L0 = a.ctl->level;
    if ((int64_t)a.ctl->acc_n[(L0 + 1) % 3] * kSampleMinDiv < a.n) return;
    j = ms_j(a, j);
    const int L = a.ctl->level;
    const uint64_t *N = slot(a, j + 1);
    const uint32_t *An = nz_bits(a, L + 1);
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < 64) {
        s_cnt[threadIdx.x] = 0;
        s_deg[threadIdx.x] = 0;
    }
    __syncthreads();
    unsigned c0 = 0, c1 = 0;
    unsigned long long d0 = 0, d1 = 0, bytes = 0;
    const int64_t nsamp = (a.nwords + kSampleStride - 1) / kSampleStride;
    const int64_t ntask = nsamp + (a.nlong + 31) / 32;
    const int64_t wpb = blockDim.x >> 5;
    for (int64_t t = blockIdx.x * wpb + (threadIdx.x >> 5); t < ntask; t += (int64_t)gridDim.x * wpb) {
        uint64_t x = 0;
        int32_t od = 0;
        unsigned wt;
        if (t < nsamp) {
            const int64_t w = min(t * kSampleStride + ((t * 13) & (kSampleStride - 1)), a.nwords - 1);
            const uint32_t m = __ldg(An + w);
            if (lane == 0) bytes += 4;
            if (!m) continue;  // warp-uniform
            const int64_t p = w * 32 + lane;
            // long rows (long_row > 0) are counted below
            if (((m >> lane) & 1u) && (a.long_row <= 0 || __ldg(a.ideg + p) <= a.long_row)) {
                x = __ldcg((const unsigned long long *)N + p);
                od = __ldg(a.odeg + p);
                bytes += 16;  // length, frontier word, push degree
            }
            wt = kSampleStride;
        } else {
            const int64_t e = (t - nsamp) * 32 + lane;
            if (e < a.nlong) {
                const int32_t p = __ldg(a.lrow + e);
                x = __ldcg((const unsigned long long *)N + p);
                if (x) od = __ldg(a.odeg + p);
                bytes += x ? 16 : 12;
            }
            wt = 1;
        }
        unsigned m = __ballot_sync(kFull, x != 0);
        while (m) {
            const int q = __ffs(m) - 1;
            m &= m - 1;
            const uint64_t xq = __shfl_sync(kFull, x, q);
            const unsigned long long oq = (unsigned long long)(unsigned)__shfl_sync(kFull, od, q) * wt;
            if ((xq >> lane) & 1ull) {
                c0 += wt;
                d0 += oq;
            }
            if ((xq >> (lane + 32)) & 1ull) {
                c1 += wt;
                d1 += oq;
            }
        }
    }
    if (c0) {
        atomicAdd(&s_cnt[lane], c0);
        atomicAdd(&s_deg[lane], d0);
    }
    if (c1) {
        atomicAdd(&s_cnt[lane + 32], c1);
        atomicAdd(&s_deg[lane + 32], d1);
    }
    bytes = warp_sum(bytes);
    if (lane == 0 && bytes) atomicAdd(&a.ctl->acc_bytes[(L + 1) % 3], bytes);
    __syncthreads();
    if (threadIdx.x < 64 && s_cnt[threadIdx.x]) {
        atomicAdd(&a.smp->rows[threadIdx.x], s_cnt[threadIdx.x]);
        atomicAdd(&a.smp->deg[threadIdx.x], s_deg[threadIdx.x]);
    }
}

// Queue of the rows in level L's frontier that hold a tmask root, for the
// push after a bottom-up level's pull: next-parity queue q[(L + 1) & 1],
// count qn[(L + 1) % 3] (both idle during a bottom-up level). A warp takes 32
// bitmap words at a time and reads the frontier words of the set bits only.
__global__ void k_ms_tq(MsArgs a, int j) {
    const uint64_t tm = a.ctl->tmask;
    if (!tm) return;
    j = ms_j(a, j);
    const int L = a.ctl->level;
    const uint64_t *F = slot(a, j);
    const uint32_t *Az = nz_bits(a, L);
    int32_t *Q = ((L + 1) & 1) ? a.q1 : a.q0;
    unsigned long long *qslot = &a.ctl->qn[(L + 1) % 3];
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long bytes = 0;
    // warp-uniform bound: every lane reaches the ballots
    for (int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) & ~31ll; w0 < a.nwords;
         w0 += stride) {
        const uint32_t mine = w0 + lane < a.nwords ? __ldg(Az + w0 + lane) : 0u;
        bytes += 4 + 8 * __popc(mine);  // bitmap word, the frontier words it selects
        unsigned words = __ballot_sync(kFull, mine != 0);
        while (words) {
            const int q = __ffs(words) - 1;
            words &= words - 1;
            const uint32_t m = __shfl_sync(kFull, mine, q);
            const int64_t p = (w0 + q) * 32 + lane;
            const bool hit = ((m >> lane) & 1u) && (__ldg(F + p) & tm);
            const unsigned hm = __ballot_sync(kFull, hit);
            if (!hm) continue;
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(qslot, (unsigned long long)__popc(hm));
            base = __shfl_sync(kFull, base, 0);
            if (hit) Q[base + __popc(hm & ((1u << lane) - 1u))] = (int32_t)p;
            if (lane == 0) bytes += 4 * __popc(hm);  // queue entries
        }
    }
    bytes = warp_sum(bytes);
    if (lane == 0 && bytes) atomicAdd(&a.ctl->acc_bytes[(L + 1) % 3], bytes);
}

__device__ inline void ms_feature_ctl(const MsCtl &m, BfsCtl &c) {
    memset(&c, 0, sizeof(c));
    c.level = m.level;
    c.n = m.n;
    c.nwords = m.nwords;
    c.nf = m.nf;
    c.mf = m.mf;
    c.prev_nf = m.prev_nf;
    c.nu = m.nu;
    c.mu = m.mu;
    c.active_words = m.active_words;
    c.prev_dir = m.prev_dir;
    c.policy = m.policy;
    c.alpha = m.alpha;
    c.beta = m.beta;
    c.feat_mean_deg = m.feat_mean_deg;
    c.feat_skew = m.feat_skew;
}

// Rollover of level L's counters and the device-side decision for L+1.
// dir: the direction level L ran (-1: the one recorded in the control block,
// as in the CUDA-graph loop). wh: the graph loop's while condition (0 when
// the host drives the loop), cleared when the traversal is done or the
// snapshot store must be flushed before the next level.
static_assert(sizeof(MsCtl) % 8 == 0, "the control block is copied in 8-byte words");

__global__ void k_ms_end(MsArgs a, int dir, cudaGraphConditionalHandle wh) {
    if (threadIdx.x >= 32) return;
    __shared__ MsCtl s;
    __shared__ int s_skip;
    // the control block moves between global and shared memory with all 32
    // lanes (8-byte words), not one thread's serial copy
    constexpr int kCtlWords = (int)(sizeof(MsCtl) / 8);
    for (int w = threadIdx.x; w < kCtlWords; w += 32)
        reinterpret_cast<unsigned long long *>(&s)[w] =
            reinterpret_cast<const unsigned long long *>(a.ctl)[w];
    __syncwarp();
    if (threadIdx.x == 0) {
        MsCtl &c = s;
        s_skip = c.done;  // the graph loop's first pass when nothing is left to do
        if (!c.done) {
            if (dir < 0) dir = c.dir;
            const int k = (c.level + 1) % 3;
            const unsigned long long nn = c.acc_n[k];
            if (c.gtrace_on && c.level < kGTraceCap) {
                long long *r = a.gtrace + (int64_t)c.level * kGTraceW;
                r[1] = (long long)globaltimer_ns();
                r[2] = dir == ALB_DIR_TOPDOWN
                           ? (long long)(20 * c.nf + 16 * c.mf + 16 * (int64_t)nn)
                           : (long long)c.acc_bytes[k] + 8 * a.npad + 8 * a.nwords;
                r[3] = dir;
                r[4] = c.nf;
                r[5] = c.mf;
                r[6] = c.nu;
                r[7] = c.mu;
            }
            c.prev_nf = c.nf;
            c.nf = (int64_t)nn;
            c.mf = (int64_t)c.acc_mo[k];
            c.nu -= (int64_t)c.acc_done[k];  // vertices every root has visited
            c.mu -= (int64_t)c.acc_mi[k];
            c.active_words -= (int64_t)c.acc_full[k];
            c.pairs += (int64_t)c.acc_bits[k];
            c.edges += (int64_t)c.acc_edges[k];
            c.q_valid = dir == ALB_DIR_TOPDOWN;
            c.prev_dir = dir;
            c.dir = dir;
            if (dir == ALB_DIR_TOPDOWN) c.levels_td++; else c.levels_bu++;
            c.level++;
            // kernels of this level in the graph loop: branch, sample and end,
            // plus the branch's steps (six top-down; seven bottom-up, four in
            // kBrBU, which has no push)
            c.launches += 3 + (c.branch == kBrTD ? 6 : c.branch == kBrBU ? 4 : 7);
            if (nn == 0) c.done = 1;
            if (!c.done && c.level >= c.level_cap) {  // cannot happen in a BFS: refuse
                c.done = 1;
                c.err = ALB_ERR_DEVICE;
            }
            // zero the slots level L+1 accumulates into after the next rollover
            const int z = (c.level + 1) % 3;
            c.acc_n[z] = c.acc_mo[z] = c.acc_mi[z] = c.acc_full[z] = c.acc_bits[z] = 0;
            c.acc_edges[z] = c.qn[z] = c.acc_bytes[z] = c.acc_done[z] = c.nbig[z] = c.work[z] = 0;
            // a bottom-up level's push of its tmask roots used the new level's
            // long-row counter and, after a bottom-up level, its queue count
            c.nbig[c.level % 3] = 0;
            if (!c.q_valid) c.qn[c.level % 3] = 0;
        }
    }
    __syncwarp();
    if (s_skip) {  // nothing changed: no write-back
        if (threadIdx.x == 0 && wh) cudaGraphSetConditional(wh, 0);
        return;
    }
    // decide the next level (one warp; the MLP runs here when loaded)
    BfsCtl fc;
    ms_feature_ctl(s, fc);
    int next;
    if (s.policy == ALB_POLICY_LEARNED && a.mlp && a.mlp[kMlpParams] != 0.0f) {
        float f[kMlpIn];
        level_features(fc, f);
        next = mlp_select_warp(a.mlp, f);
    } else {
        next = rule_dir(fc);
    }
    // Roots pushed instead of pulled, at the first bottom-up level after a
    // top-down one (where the roots' frontiers differ most in size: some are
    // still a few rows wide when most cover a good part of the graph): the
    // roots with the smallest estimated push edges, in ascending order while
    // their running sum stays within the budget. Later bottom-up levels pull
    // every root. The samples are cleared for the next level.
    {
        __shared__ unsigned long long s_val[64], s_cum[64];
        const int i = threadIdx.x;
        const int64_t budget = s.push_budget;
        const bool bu = next != ALB_DIR_TOPDOWN && s.dir == ALB_DIR_TOPDOWN && !s.done && budget > 0;
        const unsigned long long e0 = a.smp->deg[i], e1 = a.smp->deg[i + 32];
        unsigned lo = 0, hi = 0;
        if (bu) {
            // rank of roots i and i + 32 by (estimate, root index)
            int r0 = 0, r1 = 0;
            for (int q = 0; q < 32; q++) {
                const unsigned long long a0 = __shfl_sync(kFull, e0, q), a1 = __shfl_sync(kFull, e1, q);
                r0 += (a0 < e0 || (a0 == e0 && q < i)) + (a1 < e0);
                r1 += (a0 <= e1) + (a1 < e1 || (a1 == e1 && q < i));
            }
            s_val[r0] = e0;
            s_val[r1] = e1;
            __syncwarp();
            // running sums in rank order: lane i holds ranks 2i and 2i + 1
            const unsigned long long v0 = s_val[2 * i], v1 = s_val[2 * i + 1];
            unsigned long long inc = v0 + v1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long t = __shfl_up_sync(kFull, inc, o);
                if (i >= o) inc += t;
            }
            s_cum[2 * i] = inc - v1;
            s_cum[2 * i + 1] = inc;
            __syncwarp();
            const unsigned long long lim = (unsigned long long)budget;
            lo = __ballot_sync(kFull, s_cum[r0] <= lim && ((s.used >> i) & 1ull));
            hi = __ballot_sync(kFull, s_cum[r1] <= lim && ((s.used >> (i + 32)) & 1ull));
        }
        a.smp->rows[i] = a.smp->rows[i + 32] = 0;
        a.smp->deg[i] = a.smp->deg[i + 32] = 0;
        if (i == 0) {
            s.tmask = (unsigned long long)lo | ((unsigned long long)hi << 32);
            s.pushed_roots += __popcll(s.tmask);
        }
        __syncwarp();
    }
    if (threadIdx.x == 0) {
        s.dir = next;
        // nonzero-bitmap filter when under 1/8 of all entries point into the frontier
        s.filt = s.mf < s.m_in / 8;
        s.branch = ms_branch_of(next, s.filt, s.prev_dir == ALB_DIR_TOPDOWN);
        s.need_flush = !s.done && (s.level - s.base + 1 >= a.K);
    }
    __syncwarp();
    for (int w = threadIdx.x; w < kCtlWords; w += 32)
        reinterpret_cast<unsigned long long *>(a.ctl)[w] =
            reinterpret_cast<const unsigned long long *>(&s)[w];
    if (threadIdx.x == 0 && wh) cudaGraphSetConditional(wh, (s.done || s.need_flush) ? 0u : 1u);
}

// Graph loop: the level's branch (none once done).
__global__ void k_ms_branch(MsArgs a, cudaGraphConditionalHandle sh) {
    const MsCtl *c = a.ctl;
    if (c->gtrace_on && !c->done && c->level < kGTraceCap)
        a.gtrace[(int64_t)c->level * kGTraceW] = (long long)globaltimer_ns();
    cudaGraphSetConditional(sh, c->done ? (unsigned)kBrCount : (unsigned)c->branch);
}

// After a flush of the snapshot store: slot 0 now holds level `base`.
__global__ void k_ms_set_base(MsArgs a, int base) {
    a.ctl->base = base;
    a.ctl->need_flush = 0;
}

// Before a top-down level: clear the next snapshot slot and nonzero bitmap.
__global__ void k_ms_zero_next(MsArgs a, int j) {
    j = ms_j(a, j);
    const int L = a.ctl->level;
    uint64_t *N = slot(a, j + 1);
    uint32_t *An = nz_bits(a, L + 1);
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t str = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < a.npad / 2; i += str)
        reinterpret_cast<uint4 *>(N)[i] = make_uint4(0u, 0u, 0u, 0u);
    for (int64_t w = tid; w < a.nwords; w += str) An[w] = 0u;
}

// Writes the levels held by snapshot slots [0, nslots) (levels base ..) into
// the vertex-major n x 64 output. Half a warp per position: lane q of the
// half owns roots 4q .. 4q+3 and writes them as one 16-byte store, so a
// position's 256-byte output row is one contiguous burst. The slots are read
// once per position (lane q loads slot q and q+16) and shared with shuffles.
// Each warp takes kExpandUnroll pairs of positions per step and issues all
// their loads before the first shuffle, to keep enough bytes in flight.
// A root's bit is set in exactly one slot, so the slots can be scanned in any
// order. kFirst: the first flush writes every entry (-1 where unreached and
// for root columns >= nroots); later flushes write only the levels found.
constexpr int kExpandUnroll = 4;

template <bool kFirst, bool kVec>
__global__ void k_ms_expand(MsArgs a, int nslots, int base, int nroots, int32_t *out) {
    const int lane = threadIdx.x & 31, q = lane & 15;
    const int64_t total = a.n * 16;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int first_cnt = min(16, nslots);
    // the loop bound is warp-uniform so that every lane reaches the shuffles
    for (int64_t t0 = gw * 32 * kExpandUnroll; t0 < total; t0 += nw * 32 * kExpandUnroll) {
        uint64_t mine[kExpandUnroll];
        int32_t vid[kExpandUnroll];
#pragma unroll
        for (int u = 0; u < kExpandUnroll; u++) {
            const int64_t t = t0 + u * 32 + lane;
            const bool ok = t < total;
            const int64_t p = ok ? t >> 4 : 0;
            mine[u] = (ok && q < nslots) ? __ldcs(a.S + (int64_t)q * a.npad + p) : 0ull;
            vid[u] = ok ? __ldg(a.perm + p) : 0;
        }
#pragma unroll
        for (int u = 0; u < kExpandUnroll; u++) {
            const int64_t t = t0 + u * 32 + lane;
            const bool ok = t < total;
            const int64_t p = ok ? t >> 4 : 0;
            int32_t l[4] = {-1, -1, -1, -1};
            for (int k = 0; k < first_cnt; k++) {
                const uint64_t sv = __shfl_sync(kFull, mine[u], k, 16);
                const uint32_t b = (uint32_t)(sv >> (4 * q)) & 0xFu;
                if (b) {
#pragma unroll
                    for (int r = 0; r < 4; r++)
                        if ((b >> r) & 1u) l[r] = base + k;
                }
            }
            for (int c0 = 16; c0 < nslots; c0 += 16) {  // more than 16 levels held
                const int js = c0 + q;
                const uint64_t m2 =
                    (ok && js < nslots) ? __ldcs(a.S + (int64_t)js * a.npad + p) : 0ull;
                const int cnt = min(16, nslots - c0);
                for (int k = 0; k < cnt; k++) {
                    const uint64_t sv = __shfl_sync(kFull, m2, k, 16);
                    const uint32_t b = (uint32_t)(sv >> (4 * q)) & 0xFu;
                    if (b) {
#pragma unroll
                        for (int r = 0; r < 4; r++)
                            if ((b >> r) & 1u) l[r] = base + c0 + k;
                    }
                }
            }
            if (!ok) continue;
#pragma unroll
            for (int r = 0; r < 4; r++)
                if (4 * q + r >= nroots) l[r] = -1;
            int32_t *o = out + (int64_t)vid[u] * 64 + 4 * q;
            if (kFirst && kVec) {
                __stcs(reinterpret_cast<int4 *>(o), make_int4(l[0], l[1], l[2], l[3]));
            } else {
#pragma unroll
                for (int r = 0; r < 4; r++)
                    if (kFirst || l[r] >= 0) o[r] = l[r];
            }
        }
    }
}

// The same output, one CTA per aligned tile of kExpandTile rows. The sort
// permutes rows only inside sigma windows, so when sigma divides the tile the
// positions of the tile's original ids are the tile's own positions. The CTA
// first reads the tile's slot words (coalesced) and folds them, per
// position, into five words: R = OR of all slots (roots that reached it) and
// M_t = OR of the slots whose index has bit t set, so that root i's slot
// index is the number whose bit t is bit i of M_t. It then writes the tile's
// 256-byte output rows in original-id order, a sequential stream: lane q of a
// half warp turns nibble q of the five words into the levels of roots
// 4q .. 4q+3 with a few integer operations, independent of the slot count.
// First flush, 16-byte aligned output, at most kExpandMaxSlots slots.
constexpr int kExpandTile = 1024;
constexpr int kExpandMaxSlots = 16;
constexpr int kExpandThreads = 512;
constexpr size_t kExpandSmem = (5 * sizeof(uint64_t) + sizeof(int32_t)) * kExpandTile;

// Bit k of the nibble n moves to bit 8k (copies shifted by 0, 7, 14, 21 do
// not overlap for n < 16, so the product has no carries).
__device__ __forceinline__ uint32_t nibble_to_bytes(uint32_t n) {
    return (n * 0x00204081u) & 0x01010101u;
}

__global__ void __launch_bounds__(kExpandThreads) k_ms_expand_tile(MsArgs a, int nslots, int base,
                                                                   int nroots, int32_t *out) {
    extern __shared__ uint64_t s_fold[];  // 5 x kExpandTile words, then kExpandTile positions
    int32_t *s_pos = reinterpret_cast<int32_t *>(s_fold + 5 * kExpandTile);
    const int64_t t0 = (int64_t)blockIdx.x * kExpandTile;
    const int rows = (int)min((int64_t)kExpandTile, a.n - t0);
    for (int r = threadIdx.x; r < kExpandTile; r += blockDim.x) {
        uint64_t m0 = 0, m1 = 0, m2 = 0, m3 = 0, all = 0;
        if (r < rows) {
#pragma unroll 4
            for (int jj = 0; jj < nslots; jj++) {
                const uint64_t w = __ldcs(a.S + (int64_t)jj * a.npad + t0 + r);
                all |= w;
                if (jj & 1) m0 |= w;
                if (jj & 2) m1 |= w;
                if (jj & 4) m2 |= w;
                if (jj & 8) m3 |= w;
            }
            s_pos[r] = (int32_t)((int64_t)__ldg(a.inv + t0 + r) - t0);  // position in the tile
        }
        s_fold[r] = all;
        s_fold[kExpandTile + r] = m0;
        s_fold[2 * kExpandTile + r] = m1;
        s_fold[3 * kExpandTile + r] = m2;
        s_fold[4 * kExpandTile + r] = m3;
    }
    __syncthreads();
    const int q = threadIdx.x & 15;
    const int sh = 4 * q;
    for (int r = threadIdx.x >> 4; r < rows; r += blockDim.x >> 4) {
        const int64_t v = t0 + r;  // original id
        const int pl = s_pos[r];
        if ((unsigned)pl >= (unsigned)rows) {  // not a window permutation: refuse, loudly
            a.ctl->err = ALB_ERR_DEVICE;
            continue;
        }
        const uint32_t reach =
            nibble_to_bytes((uint32_t)(s_fold[pl] >> sh) & 0xFu);
        const uint32_t idx =
            nibble_to_bytes((uint32_t)(s_fold[kExpandTile + pl] >> sh) & 0xFu) |
            (nibble_to_bytes((uint32_t)(s_fold[2 * kExpandTile + pl] >> sh) & 0xFu) << 1) |
            (nibble_to_bytes((uint32_t)(s_fold[3 * kExpandTile + pl] >> sh) & 0xFu) << 2) |
            (nibble_to_bytes((uint32_t)(s_fold[4 * kExpandTile + pl] >> sh) & 0xFu) << 3);
        int32_t l[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const bool hit = ((reach >> (8 * k)) & 1u) && (sh + k < nroots);
            l[k] = hit ? base + (int32_t)((idx >> (8 * k)) & 0xFu) : -1;
        }
        __stcs(reinterpret_cast<int4 *>(out + v * 64 + 4 * q), make_int4(l[0], l[1], l[2], l[3]));
    }
}

struct MsScratch {
    bool ready = false;
    int32_t K = 0;
    uint64_t *V = nullptr, *S = nullptr;
    uint32_t *D = nullptr, *A = nullptr;
    int32_t *q0 = nullptr, *q1 = nullptr, *big = nullptr;
    int64_t *big_base = nullptr;
    MsCtl *ctl = nullptr, *h_ctl = nullptr;
    int32_t *out = nullptr;
    long long *gtrace = nullptr;  // the graph loop's level records
    // CUDA-graph level loop (built for one block size)
    cudaGraph_t lg = nullptr;
    cudaGraphExec_t lexec = nullptr;
    int lblock = 0;
};

}  // namespace alb

namespace alb {

static MsScratch &ms_scratch(alb_graph *g) {
    if (!g->ms) g->ms = new MsScratch();
    return *(MsScratch *)g->ms;
}

void ms_scratch_free(alb_graph *g) {
    if (!g->ms) return;
    MsScratch &m = *(MsScratch *)g->ms;
    dfree(m.V);
    dfree(m.S);
    dfree(m.D);
    dfree(m.A);
    dfree(m.q0);
    dfree(m.q1);
    dfree(m.big);
    dfree(m.big_base);
    dfree(m.ctl);
    dfree(m.out);
    dfree(m.gtrace);
    if (m.h_ctl) cudaFreeHost(m.h_ctl);
    if (m.lexec) cudaGraphExecDestroy(m.lexec);
    if (m.lg) cudaGraphDestroy(m.lg);
    delete (MsScratch *)g->ms;
    g->ms = nullptr;
}

namespace {

void launch_expand(const MsArgs &a, int nslots, int base, bool first, int nroots, int32_t *out,
                   int num_sms, cudaStream_t st) {
    const bool vec = ((uintptr_t)out & 15) == 0;
    auto grid = [&](const void *f) {
        const int per = resident_blocks(f, 256);
        return (unsigned)(num_sms * (per > 0 ? per : 8));
    };
    const bool tiled = first && vec && nslots <= kExpandMaxSlots && a.sigma >= 1 &&
                       a.sigma <= kExpandTile && kExpandTile % a.sigma == 0;
    if (tiled) {
        cudaFuncSetAttribute(k_ms_expand_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kExpandSmem);
        const unsigned tiles = (unsigned)((a.n + kExpandTile - 1) / kExpandTile);
        k_ms_expand_tile<<<tiles, kExpandThreads, kExpandSmem, st>>>(a, nslots, base, nroots,
                                                                      out);
    } else if (first && vec)
        k_ms_expand<true, true><<<grid((const void *)k_ms_expand<true, true>), 256, 0, st>>>(
            a, nslots, base, nroots, out);
    else if (first)
        k_ms_expand<true, false><<<grid((const void *)k_ms_expand<true, false>), 256, 0, st>>>(
            a, nslots, base, nroots, out);
    else
        k_ms_expand<false, false><<<grid((const void *)k_ms_expand<false, false>), 256, 0, st>>>(
            a, nslots, base, nroots, out);
}

alb_status ms_alloc(alb_graph *g, MsScratch &m) {
    if (m.ready) return ALB_OK;
    const Sell &s = g->sell;
    const int64_t npad = s.nwords * 32;
    m.K = 32;
    ALB_TRY(dmalloc((void **)&m.V, sizeof(uint64_t) * npad, "msbfs visited"));
    ALB_TRY(dmalloc((void **)&m.S, sizeof(uint64_t) * npad * m.K, "msbfs frontier snapshots"));
    ALB_TRY(dmalloc((void **)&m.D, sizeof(uint32_t) * s.nwords, "msbfs done bitmap"));
    ALB_TRY(dmalloc((void **)&m.A, sizeof(uint32_t) * 2 * s.nwords, "msbfs frontier-nonzero bitmaps"));
    ALB_TRY(dmalloc((void **)&m.q0, sizeof(int32_t) * npad, "msbfs queue"));
    ALB_TRY(dmalloc((void **)&m.q1, sizeof(int32_t) * npad, "msbfs queue"));
    ALB_TRY(dmalloc((void **)&m.big, sizeof(int32_t) * npad, "msbfs long-row list"));
    ALB_TRY(dmalloc((void **)&m.big_base, sizeof(int64_t) * npad, "msbfs long-row chunk bases"));
    ALB_TRY(dmalloc((void **)&m.ctl, sizeof(MsCtl) + sizeof(MsSample), "msbfs control"));
    ALB_TRY(dmalloc((void **)&m.gtrace, sizeof(long long) * kGTraceCap * kGTraceW,
                    "msbfs level records"));
    ALB_CK(cudaMallocHost((void **)&m.h_ctl, sizeof(MsCtl)));
    m.ready = true;
    return ALB_OK;
}

MsArgs ms_args(alb_graph *g, MsScratch &m) {
    const Sell &s = g->sell;
    MsArgs a;
    std::memset(&a, 0, sizeof(a));
    a.n = g->n;
    a.nwords = s.nwords;
    a.npad = s.nwords * 32;
    a.C = s.C;
    a.log2C = s.log2C;
    a.K = m.K;
    a.sigma = s.sigma;
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
    a.long_row = s.long_row;
    a.lrow = s.lrow;
    a.lptr = s.lptr;
    a.lcol = s.lcol;
    a.V = m.V;
    a.S = m.S;
    a.D = m.D;
    a.A = m.A;
    a.q0 = m.q0;
    a.q1 = m.q1;
    a.big = m.big;
    a.big_base = m.big_base;
    a.ctl = m.ctl;
    a.smp = reinterpret_cast<MsSample *>(m.ctl + 1);
    a.gtrace = m.gtrace;
    return a;
}

}  // namespace

extern const float *selector_device_params(int which);

// Device copies of the state one level mutates (restored between variants).
struct MsSnapshot {
    uint64_t *V = nullptr;
    uint32_t *D = nullptr;
    MsCtl *ctl = nullptr;
    ~MsSnapshot() {
        dfree(V);
        dfree(D);
        dfree(ctl);
    }
};

alb_status ms_snapshot(const MsArgs &a, MsSnapshot &s, cudaStream_t st, bool restore) {
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
    };
    cudaError_t e = restore ? cp(a.V, s.V, 8 * a.npad) : cp(s.V, a.V, 8 * a.npad);
    if (e == cudaSuccess) e = restore ? cp(a.D, s.D, 4 * a.nwords) : cp(s.D, a.D, 4 * a.nwords);
    const size_t cb = sizeof(MsCtl) + sizeof(MsSample);
    if (e == cudaSuccess) e = restore ? cp(a.ctl, s.ctl, cb) : cp(s.ctl, a.ctl, cb);
    if (e != cudaSuccess) return fail(ALB_ERR_CUDA, "msbfs snapshot: %s", cudaGetErrorString(e));
    return ALB_OK;
}

// The level loop as one CUDA graph, decided on the device like the
// single-root loop:
//   while (!done && !need_flush) {
//     k_ms_branch;                    // sets the switch from the control block
//     switch { TD | BU+filter | BU | BU-no-bypass+filter | BU-no-bypass };
//     k_ms_sample;                    // per-root frontier sizes
//     k_ms_end;                       // rollover, next decision, while condition
//   }
// Level kernels get j = -1 and filt = -1 and read both from the control
// block. A flush of the snapshot store ends the loop; the host does it and
// launches the graph again.
struct MsNode {
    void *func;
    unsigned grid, block;
};

alb_status ms_add(cudaGraph_t gr, cudaGraphNode_t *node, const cudaGraphNode_t *dep, MsNode k,
                  void **args) {
    cudaKernelNodeParams p;
    std::memset(&p, 0, sizeof(p));
    p.func = k.func;
    p.gridDim = dim3(k.grid);
    p.blockDim = dim3(k.block);
    p.kernelParams = args;
    ALB_CK(cudaGraphAddKernelNode(node, gr, dep, dep ? 1 : 0, &p));
    return ALB_OK;
}

alb_status build_ms_graph(alb_graph *g, MsScratch &m, MsArgs &a, int block) {
    if (m.lexec) cudaGraphExecDestroy(m.lexec);
    if (m.lg) cudaGraphDestroy(m.lg);
    m.lexec = nullptr;
    m.lg = nullptr;
    const int sms = g->num_sms;
    auto res = [&](const void *f, int b) -> MsNode {
        const int per = resident_blocks(f, b);
        return MsNode{(void *)f, (unsigned)(sms * (per > 0 ? per : std::max(1, 2048 / b))),
                      (unsigned)b};
    };
    const MsNode wide{nullptr, (unsigned)(sms * std::max(1, 2048 / block)), (unsigned)block};
    MsNode tq = wide;
    tq.func = (void *)k_ms_tq;
    ALB_CK(cudaGraphCreate(&m.lg, 0));
    cudaGraphConditionalHandle wh;
    ALB_CK(cudaGraphConditionalHandleCreate(&wh, m.lg, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams wp = {cudaGraphNodeTypeConditional};
    wp.conditional.handle = wh;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    ALB_CK(cudaGraphAddNode(&wnode, m.lg, nullptr, nullptr, 0, &wp));
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    cudaGraphConditionalHandle sh;
    ALB_CK(cudaGraphConditionalHandleCreate(&sh, body, 0, cudaGraphCondAssignDefault));
    void *bargs[] = {&a, &sh};
    cudaGraphNode_t nbranch;
    ALB_TRY(ms_add(body, &nbranch, nullptr, MsNode{(void *)k_ms_branch, 1, 1}, bargs));
    cudaGraphNodeParams sp = {cudaGraphNodeTypeConditional};
    sp.conditional.handle = sh;
    sp.conditional.type = cudaGraphCondTypeSwitch;
    sp.conditional.size = kBrCount;
    cudaGraphNode_t nswitch;
    ALB_CK(cudaGraphAddNode(&nswitch, body, &nbranch, nullptr, 1, &sp));
    int jneg = -1, fneg = -1, ahead0 = 0, ahead1 = 1;
    void *aj[] = {&a, &jneg};
    void *ajf[] = {&a, &jneg, &fneg};
    void *ac0[] = {&a, &ahead0};
    void *ac1[] = {&a, &ahead1};
    auto chain = [&](cudaGraph_t br, std::initializer_list<std::pair<MsNode, void **>> ks)
        -> alb_status {
        cudaGraphNode_t prev = nullptr, cur;
        for (const auto &k : ks) {
            ALB_TRY(ms_add(br, &cur, prev ? &prev : nullptr, k.first, k.second));
            prev = cur;
        }
        return ALB_OK;
    };
    // push: the branch can be the first bottom-up level after a top-down one,
    // the only level whose tmask roots are pushed (kBrBU never is: it is the
    // unfiltered branch of later levels, so its three push launches, which
    // would return at once, are left out)
    auto bu = [&](int br, const void *slices, bool early, bool push) -> alb_status {
        const void *hd = early ? (const void *)k_ms_bu_long<true> : (const void *)k_ms_bu_long<false>;
        const void *tl = early ? (const void *)k_ms_bu_long_tail<true>
                               : (const void *)k_ms_bu_long_tail<false>;
        if (!push)
            return chain(sp.conditional.phGraph_out[br],
                         {{res(slices, kMsBuBlock), aj}, {res(hd, block), ajf},
                          {res(tl, block), ajf}, {res((const void *)k_ms_bu_long_fin, block), aj}});
        return chain(sp.conditional.phGraph_out[br],
                     {{res(slices, kMsBuBlock), aj}, {res(hd, block), ajf}, {res(tl, block), ajf},
                      {res((const void *)k_ms_bu_long_fin, block), aj}, {tq, aj},
                      {res((const void *)k_ms_td<true>, block), aj},
                      {res((const void *)k_ms_td_big<true>, block), aj}});
    };
    MsNode cmp = wide;
    cmp.func = (void *)k_ms_compact;
    MsNode zero = wide;
    zero.func = (void *)k_ms_zero_next;
    ALB_TRY(chain(sp.conditional.phGraph_out[kBrTD],
                  {{cmp, ac0}, {zero, aj}, {res((const void *)k_ms_td<false>, block), aj},
                   {res((const void *)k_ms_td_big<false>, block), aj}, {cmp, ac1},
                   {res((const void *)k_ms_td_finish, block), aj}}));
    ALB_TRY(bu(kBrBUFilt, (const void *)k_ms_bu<true, true, true>, true, true));
    ALB_TRY(bu(kBrBU, (const void *)k_ms_bu<true, true, false>, true, false));
    ALB_TRY(bu(kBrBUWide, (const void *)k_ms_bu<true, true, false, true>, true, true));
    ALB_TRY(bu(kBrBUNBFilt, (const void *)k_ms_bu<false, false, true>, false, true));
    ALB_TRY(bu(kBrBUNB, (const void *)k_ms_bu<false, false, false>, false, true));
    int dneg = -1;
    void *eargs[] = {&a, &dneg, &wh};
    cudaGraphNode_t nsample, nend;
    void *sargs[] = {&a, &jneg, &dneg};
    ALB_TRY(ms_add(body, &nsample, &nswitch, res((const void *)k_ms_sample, kSampleBlock), sargs));
    ALB_TRY(ms_add(body, &nend, &nsample, MsNode{(void *)k_ms_end, 1, 32}, eargs));
    ALB_CK(cudaGraphInstantiate(&m.lexec, m.lg, 0));
    m.lblock = block;
    return ALB_OK;
}

alb_status msbfs_impl(alb_graph *g, const int32_t *roots, int32_t nroots, const alb_bfs_opts &o,
                      int32_t *d_levels, alb_stats *st, std::vector<alb_level_rec> *trace,
                      std::vector<alb_level_profile> *prof = nullptr) {
    MsScratch &m = ms_scratch(g);
    PhaseLog ph("msbfs64_device");
    ALB_TRY(ms_alloc(g, m));
    ph.mark("scratch", g->stream);
    MsArgs a = ms_args(g, m);
    a.mlp = selector_device_params(1);
    const Sell &s = g->sell;
    cudaStream_t stream = g->stream;
    const int block = o.block;
    const unsigned wide = (unsigned)(g->num_sms * std::max(1, 2048 / block));
    MsInit in;
    std::memset(&in, 0, sizeof(in));
    for (int i = 0; i < nroots; i++) in.roots[i] = roots[i];
    in.nroots = nroots;
    in.policy = o.policy;
    in.alpha = o.alpha;
    in.beta = o.beta;
    in.mean_deg = g->n > 0 ? (float)((double)s.m_in / (double)g->n) : 0.f;
    in.skew = skew_of(s, g->n);
    in.n_live = g->n - s.zero_in;
    in.m_in = s.m_in;
    in.active0 = s.active0;
    in.push_budget = s.m_in / kPushDiv;
    {
        // words per run of the pull: about three runs per resident warp, 8 .. 32
        // (RMAT s22: 8 beats 32 by 7 %; s24: 32 beats 8 by 2 %, where longer runs
        // save counter round trips and still leave every warp busy)
        const int per = resident_blocks((const void *)k_ms_bu<true, true, false>, kMsBuBlock);
        const int64_t warps = (int64_t)std::max(per, 1) * (kMsBuBlock / 32) * g->num_sms;
        in.grab = (int32_t)std::max<int64_t>(kGrabWords, std::min<int64_t>(32, s.nwords / (3 * warps)));
    }
    if (const char *e = std::getenv("ALB_MS_PUSH_DIV")) {  // tuning: 0 turns the push off
        const long long dv = std::atoll(e);
        in.push_budget = dv > 0 ? s.m_in / dv : 0;
    }
    const int32_t level_cap = (int32_t)std::min<int64_t>(g->n + 1, INT32_MAX - 1);
    in.level_cap = level_cap;
    // a traced run of the graph loop records its levels on the device, so
    // the trace times the benchmarked form itself
    const bool gtrace = trace && !prof && o.loop == ALB_LOOP_GRAPH;
    in.gtrace = gtrace ? 1 : 0;
    const uint64_t unused = nroots >= 64 ? 0ull : ~((1ull << nroots) - 1);
    ALB_CK(cudaEventRecord(g->ev0, stream));
    k_ms_init<<<wide, 256, 0, stream>>>(a, unused);
    k_ms_roots<<<1, 64, 0, stream>>>(a, in);  // also decides level 0's direction
    ALB_CK(cudaGetLastError());
    int64_t launches = 2;
    MsCtl *h = m.h_ctl;
    int base = 0;      // level held by slot 0
    bool first_flush = true;
    // flush of the snapshot store: write out levels [base, base + K - 1) and
    // restart the store from the current frontier
    auto flush = [&]() -> alb_status {
        if (d_levels) {
            launch_expand(a, m.K - 1, base, first_flush, nroots, d_levels, g->num_sms, stream);
            launches++;
        }
        first_flush = false;
        ALB_CK(cudaMemcpyAsync(a.S, a.S + (int64_t)(m.K - 1) * a.npad, sizeof(uint64_t) * a.npad,
                               cudaMemcpyDeviceToDevice, stream));
        base += m.K - 1;
        k_ms_set_base<<<1, 1, 0, stream>>>(a, base);
        launches++;
        return ALB_OK;
    };
    if (o.loop == ALB_LOOP_GRAPH && (!trace || gtrace) && !prof) {
        // device-driven level loop: the host only steps in for flushes
        if (!m.lexec || m.lblock != block) ALB_TRY(build_ms_graph(g, m, a, block));
        while (true) {
            ALB_CK(cudaGraphLaunch(m.lexec, stream));
            ALB_CK(cudaMemcpyAsync(h, a.ctl, sizeof(MsCtl), cudaMemcpyDeviceToHost, stream));
            ALB_CK(cudaStreamSynchronize(stream));
            if (h->err) return fail(h->err, "msbfs: the device refused the traversal");
            if (h->done || !h->need_flush) break;
            ALB_TRY(flush());
        }
        // per level: counted by k_ms_end from the branch the level took
        launches += h->launches;
        if (gtrace) {
            const int nl = std::min<int>(h->level, kGTraceCap);
            std::vector<long long> rec((size_t)nl * kGTraceW);
            if (nl > 0)
                ALB_CK(cudaMemcpyAsync(rec.data(), m.gtrace, sizeof(long long) * rec.size(),
                                       cudaMemcpyDeviceToHost, stream));
            ALB_CK(cudaStreamSynchronize(stream));
            trace->clear();
            for (int L = 0; L < nl; L++) {
                const long long *r = rec.data() + (size_t)L * kGTraceW;
                alb_level_rec t;
                std::memset(&t, 0, sizeof(t));
                t.level = L;
                t.dir = (int32_t)r[3];
                t.nf = r[4];
                t.mf = r[5];
                t.nu = r[6];
                t.mu = r[7];
                t.t_ns = r[0];
                t.step_us = (float)((r[1] - r[0]) / 1e3);
                t.bytes = r[2];
                trace->push_back(t);
            }
        }
    } else {
        ALB_CK(cudaMemcpyAsync(h, a.ctl, sizeof(MsCtl), cudaMemcpyDeviceToHost, stream));
        ALB_CK(cudaStreamSynchronize(stream));
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (trace) trace->clear();
        if (trace || prof) {
            ALB_CK(cudaEventCreate(&e0));
            ALB_CK(cudaEventCreate(&e1));
        }
        MsSnapshot snap;
        if (prof) {
            prof->clear();
            ALB_TRY(dmalloc((void **)&snap.V, 8 * a.npad, "msbfs snapshot"));
            ALB_TRY(dmalloc((void **)&snap.D, 4 * a.nwords, "msbfs snapshot"));
            ALB_TRY(dmalloc((void **)&snap.ctl, sizeof(MsCtl) + sizeof(MsSample), "msbfs snapshot"));
        }
        while (!h->done && h->level < level_cap) {
            const int L = h->level;
            int j = L - base;
            if (j + 1 >= m.K) {
                ALB_TRY(flush());
                j = 0;
            }
            int dir = h->dir;
            alb_level_rec rec;
            std::memset(&rec, 0, sizeof(rec));
            rec.dir = dir;
            rec.level = L;
            rec.nf = h->nf;
            rec.mf = h->mf;
            rec.nu = h->nu;
            rec.mu = h->mu;
            rec.active_slices = h->active_words;
            rec.step_us = -1.f;
            const bool q_valid = h->q_valid != 0;
            // nonzero-bitmap filter when under 1/8 of all entries point into the frontier
            const int filt = (h->mf < s.m_in / 8) ? 1 : 0;
            // the first bottom-up level after a top-down one pulls two groups at a time
            const bool two_groups = h->prev_dir == ALB_DIR_TOPDOWN;
            auto launch_step = [&](int d) -> alb_status {
                if (d == ALB_DIR_TOPDOWN) {
                    if (!q_valid) {
                        k_ms_compact<<<wide, block, 0, stream>>>(a, 0);
                        launches++;
                    }
                    k_ms_zero_next<<<wide, block, 0, stream>>>(a, j);
                    launch_resident(k_ms_td<false>, block, g->num_sms, stream, a, j);
                    launch_resident(k_ms_td_big<false>, block, g->num_sms, stream, a, j);
                    k_ms_compact<<<wide, block, 0, stream>>>(a, 1);
                    launch_resident(k_ms_td_finish, block, g->num_sms, stream, a, j);
                    launches += 5;
                } else if (d == ALB_DIR_BOTTOMUP) {
                    if (filt)
                        launch_resident(k_ms_bu<true, true, true>, kMsBuBlock, g->num_sms, stream, a, j);
                    else if (two_groups)
                        launch_resident(k_ms_bu<true, true, false, true>, kMsBuBlock, g->num_sms, stream, a, j);
                    else
                        launch_resident(k_ms_bu<true, true, false>, kMsBuBlock, g->num_sms, stream, a, j);
                    launch_resident(k_ms_bu_long<true>, block, g->num_sms, stream, a, j, filt);
                    launch_resident(k_ms_bu_long_tail<true>, block, g->num_sms, stream, a, j, filt);
                    launch_resident(k_ms_bu_long_fin, block, g->num_sms, stream, a, j);
                    launches += 4;
                } else {
                    if (filt)
                        launch_resident(k_ms_bu<false, false, true>, kMsBuBlock, g->num_sms, stream, a, j);
                    else
                        launch_resident(k_ms_bu<false, false, false>, kMsBuBlock, g->num_sms, stream, a, j);
                    launch_resident(k_ms_bu_long<false>, block, g->num_sms, stream, a, j, filt);
                    launch_resident(k_ms_bu_long_tail<false>, block, g->num_sms, stream, a, j, filt);
                    launch_resident(k_ms_bu_long_fin, block, g->num_sms, stream, a, j);
                    launches += 4;
                }
                if (d != ALB_DIR_TOPDOWN && h->prev_dir == ALB_DIR_TOPDOWN) {  // push of the roots in tmask
                    k_ms_tq<<<wide, block, 0, stream>>>(a, j);
                    launch_resident(k_ms_td<true>, block, g->num_sms, stream, a, j);
                    launch_resident(k_ms_td_big<true>, block, g->num_sms, stream, a, j);
                    launches += 3;
                }
                launch_resident(k_ms_sample, kSampleBlock, g->num_sms, stream, a, j, d);
                launches++;
                return ALB_OK;
            };
            if (prof) {
                // time every variant from the same state, then take the fastest
                alb_level_profile pr;
                std::memset(&pr, 0, sizeof(pr));
                ALB_TRY(ms_snapshot(a, snap, stream, false));
                for (int v = 0; v < 3; v++) {
                    if (v) ALB_TRY(ms_snapshot(a, snap, stream, true));
                    ALB_CK(cudaEventRecord(e0, stream));
                    ALB_TRY(launch_step(v));
                    ALB_CK(cudaEventRecord(e1, stream));
                    ALB_CK(cudaStreamSynchronize(stream));
                    float ms = 0;
                    ALB_CK(cudaEventElapsedTime(&ms, e0, e1));
                    pr.us[v] = ms * 1000.f;
                }
                int best = 0;
                for (int v = 1; v < 3; v++)
                    if (pr.us[v] < pr.us[best]) best = v;
                ALB_TRY(ms_snapshot(a, snap, stream, true));
                dir = best;
                pr.best = best;
                pr.rec = rec;
                pr.rec.dir = best;
                pr.rec.step_us = pr.us[best];
                BfsCtl fc;
                std::memset(&fc, 0, sizeof(fc));
                fc.level = L;
                fc.n = h->n;
                fc.nwords = h->nwords;
                fc.nf = h->nf;
                fc.mf = h->mf;
                fc.nu = h->nu;
                fc.mu = h->mu;
                fc.active_words = h->active_words;
                fc.feat_mean_deg = h->feat_mean_deg;
                fc.feat_skew = h->feat_skew;
                level_features(fc, pr.feat);
                prof->push_back(pr);
            }
            if (e0) cudaEventRecord(e0, stream);
            ALB_TRY(launch_step(dir));
            if (e1) cudaEventRecord(e1, stream);
            k_ms_end<<<1, 32, 0, stream>>>(a, dir, 0);
            launches++;
            ALB_CK(cudaGetLastError());
            ALB_CK(cudaMemcpyAsync(h, a.ctl, sizeof(MsCtl), cudaMemcpyDeviceToHost, stream));
            ALB_CK(cudaStreamSynchronize(stream));
            if (trace) {
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                rec.dir = dir;
                rec.step_us = ms * 1000.f;
                const int k = (L + 1) % 3;
                rec.bytes = dir == ALB_DIR_TOPDOWN
                                ? (int64_t)(20 * rec.nf + 16 * rec.mf + 16 * (int64_t)h->acc_n[k])
                                : (int64_t)h->acc_bytes[k] + 8 * a.npad + 8 * a.nwords;
                trace->push_back(rec);
            }
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    }
    if (!h->done) return fail(ALB_ERR_DEVICE, "msbfs: level cap reached");
    if (d_levels) {
        const int nslots = h->level - base;  // slots 0 .. level-base-1 hold levels
        launch_expand(a, std::min(nslots, m.K), base, first_flush, nroots, d_levels, g->num_sms,
                      stream);
        launches++;
    }
    ALB_CK(cudaGetLastError());
    ALB_CK(cudaEventRecord(g->ev1, stream));
    int32_t dev_err = 0;
    if (d_levels)
        ALB_CK(cudaMemcpyAsync(&dev_err, &a.ctl->err, sizeof(int32_t), cudaMemcpyDeviceToHost,
                               stream));
    ALB_CK(cudaStreamSynchronize(stream));
    if (dev_err) return fail(dev_err, "msbfs: level output saw a position outside its tile");
    float ms = 0;
    ALB_CK(cudaEventElapsedTime(&ms, g->ev0, g->ev1));
    if (st) {
        st->num_levels = h->level;
        st->levels_topdown = h->levels_td;
        st->levels_bottomup = h->levels_bu;
        st->pushed_roots = h->pushed_roots;
        st->reached = h->pairs;
        st->edges = h->edges;
        st->ms = ms;
        st->kernels = launches;
    }
    return ALB_OK;
}

}  // namespace alb

using namespace alb;

extern "C" {

alb_status alb_msbfs64_device(alb_graph *g, const int32_t *roots, int32_t nroots,
                              const alb_bfs_opts *o, int32_t *d_levels, alb_stats *st) {
    if (!g || !roots || nroots < 1 || nroots > 64)
        return fail(ALB_ERR_INVALID, "alb_msbfs64: need a graph and 1..64 roots");
    if (!g->sell.built) return fail(ALB_ERR_STATE, "alb_msbfs64: call alb_sell_build first");
    for (int i = 0; i < nroots; i++)
        if (roots[i] < 0 || roots[i] >= g->n)
            return fail(ALB_ERR_INVALID, "alb_msbfs64: root %d outside [0, %lld)", roots[i],
                        (long long)g->n);
    alb_bfs_opts oo;
    alb_bfs_opts_default(&oo);
    if (o) oo = *o;
    if (oo.policy < ALB_POLICY_BEAMER || oo.policy > ALB_POLICY_BOTTOMUP_NOBYPASS)
        return fail(ALB_ERR_INVALID, "alb_msbfs64: unknown policy %d", oo.policy);
    if (!(oo.block == 128 || oo.block == 256 || oo.block == 512 || oo.block == 1024))
        return fail(ALB_ERR_UNSUPPORTED, "alb_msbfs64: block must be 128, 256, 512 or 1024");
    ALB_CK(cudaSetDevice(g->device));
    std::vector<alb_level_rec> tr;
    alb_status rc;
    try {
        rc = msbfs_impl(g, roots, nroots, oo, d_levels, st, oo.trace ? &tr : nullptr);
    } catch (const std::bad_alloc &) {
        rc = fail(ALB_ERR_OOM, "alb_msbfs64: host allocation failed");
    }
    if (rc == ALB_OK && oo.trace) {
        g->last_trace = tr;
        g->last_trace_valid = true;
    }
    return rc;
}

alb_status alb_msbfs64_profile(alb_graph *g, const int32_t *roots, int32_t nroots,
                               const alb_bfs_opts *o, int32_t cap, alb_level_profile *out,
                               int32_t *count) {
    if (!g || !roots || nroots < 1 || nroots > 64 || !count || (cap > 0 && !out))
        return fail(ALB_ERR_INVALID, "alb_msbfs64_profile: bad arguments");
    if (!g->sell.built) return fail(ALB_ERR_STATE, "alb_msbfs64_profile: call alb_sell_build first");
    for (int i = 0; i < nroots; i++)
        if (roots[i] < 0 || roots[i] >= g->n)
            return fail(ALB_ERR_INVALID, "alb_msbfs64_profile: root outside the graph");
    alb_bfs_opts oo;
    alb_bfs_opts_default(&oo);
    if (o) oo = *o;
    ALB_CK(cudaSetDevice(g->device));
    std::vector<alb_level_profile> pr;
    alb_status rc;
    try {
        rc = msbfs_impl(g, roots, nroots, oo, nullptr, nullptr, nullptr, &pr);
    } catch (const std::bad_alloc &) {
        rc = fail(ALB_ERR_OOM, "alb_msbfs64_profile: host allocation failed");
    }
    if (rc != ALB_OK) return rc;
    *count = (int32_t)pr.size();
    for (int32_t i = 0; i < cap && i < (int32_t)pr.size(); i++) out[i] = pr[i];
    return ALB_OK;
}

alb_status alb_msbfs64(alb_graph *g, const int32_t *roots, int32_t nroots, const alb_bfs_opts *o,
                       int32_t *levels, alb_stats *st) {
    if (!g) return fail(ALB_ERR_INVALID, "alb_msbfs64: graph is NULL");
    ALB_CK(cudaSetDevice(g->device));
    PhaseLog ph("msbfs64");
    MsScratch &m = ms_scratch(g);
    // page-locked host levels are written by the expansion itself, across
    // the host link (as fast as a copy, measured: 193 GB/s either way), with
    // no device staging buffer and no separate copy; other host memory goes
    // through a device buffer and one copy
    int32_t *direct = nullptr;
    if (levels) {
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, levels) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
            pa.devicePointer)
            direct = static_cast<int32_t *>(pa.devicePointer);
        cudaGetLastError();
    }
    if (levels && !direct && !m.out) {
        ALB_TRY(dmalloc((void **)&m.out, sizeof(int32_t) * (size_t)g->n * 64, "msbfs levels"));
    }
    ph.mark("out_alloc", g->stream);
    ALB_TRY(alb_msbfs64_device(g, roots, nroots, o, direct ? direct : levels ? m.out : nullptr, st));
    ph.mark("traversal", g->stream);
    if (direct) {
        ALB_CK(cudaStreamSynchronize(g->stream));
    } else if (levels) {
        ALB_CK(cudaMemcpyAsync(levels, m.out, sizeof(int32_t) * (size_t)g->n * 64,
                               cudaMemcpyDeviceToHost, g->stream));
        ALB_CK(cudaStreamSynchronize(g->stream));
    }
    ph.mark("copy_out", g->stream);
    return ALB_OK;
}

}  // extern "C"
