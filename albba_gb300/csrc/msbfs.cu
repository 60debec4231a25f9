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
//
// bottom-up (k_ms_bu): warp per 32 positions; a full D word is skipped; each
//   lane ORs S[l] over its row with 16-byte column loads and stops when every
//   root has visited or reached it ((acc | V) == ~0) or at the row padding.
// top-down (k_ms_td): warp-cooperative push over the frontier queue; targets
//   receive atomicOr(S[l+1][v], S[l][u] & ~V[v]) (64-bit atomics); the first
//   writer of a target appends it to the next queue.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "graph.h"
#include "selector.cuh"

namespace alb {

constexpr uint64_t kAll = ~0ull;

struct MsCtl {
    int32_t level, dir, prev_dir, q_valid, done, err, policy, base;  // base: level of S[0]
    float alpha, beta;
    int32_t levels_td, levels_bu;
    int64_t n, nwords;
    int64_t nf, mf, prev_nf, nu, mu, active_words;
    int64_t pairs, edges;  // (vertex, root) pairs reached; sum of their push degrees
    unsigned long long acc_n[3], acc_mo[3], acc_mi[3], acc_full[3], acc_bits[3], acc_edges[3],
        qn[3], acc_bytes[3], acc_done[3], nbig[3];
    int64_t launches;
    float feat_mean_deg, feat_skew;
};

struct MsArgs {
    int64_t n, nwords, npad;
    int32_t C, log2C, K;
    const int32_t *perm, *inv, *ideg, *odeg, *width;
    const int64_t *slice_off;
    const int4 *col4;
    const int64_t *prow;
    const int32_t *pcol;
    int64_t nlong;  // rows kept out of the slices, pulled one warp each
    const int32_t *lrow;
    const int64_t *lptr;
    const int32_t *lcol;
    uint64_t *V;
    uint64_t *S;  // K slots of npad words
    uint32_t *D;
    int32_t *q0, *q1;
    int32_t *big;  // frontier rows longer than kBigRow (top-down)
    int64_t *big_base;
    MsCtl *ctl;
    const float *mlp;
};

__device__ __forceinline__ uint64_t *slot(const MsArgs &a, int j) { return a.S + (int64_t)j * a.npad; }

__global__ void k_ms_init(MsArgs a, uint64_t unused) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t str = (int64_t)gridDim.x * blockDim.x;
    uint64_t *S0 = a.S;
    for (int64_t p = tid; p < a.npad; p += str) {
        const bool live = p < a.n && a.ideg[p] > 0;
        a.V[p] = live ? unused : kAll;
        S0[p] = 0;
    }
    for (int64_t w = tid; w < a.nwords; w += str) {
        uint32_t d = 0;
        for (int b = 0; b < 32; b++) {
            const int64_t p = w * 32 + b;
            if (!(p < a.n && a.ideg[p] > 0)) d |= 1u << b;
        }
        a.D[w] = d;
    }
}

struct MsInit {
    int32_t roots[64];
    int32_t nroots, policy;
    float alpha, beta, mean_deg, skew;
    int64_t n_live, m_in, active0;
};

// One block of 64 threads: thread i seeds root i; thread 0 fills the control block.
__global__ void k_ms_roots(MsArgs a, MsInit in) {
    __shared__ unsigned long long s_nf, s_mf, s_pairs, s_edges, s_done_mi, s_full, s_done_v;
    const int i = threadIdx.x;
    if (i == 0) s_nf = s_mf = s_pairs = s_edges = s_done_mi = s_full = s_done_v = 0;
    __syncthreads();
    if (i < in.nroots) {
        const int32_t p = a.inv[in.roots[i]];
        const uint64_t bit = 1ull << i;
        const unsigned long long oldv = atomicOr((unsigned long long *)a.V + p, bit);
        const unsigned long long olds = atomicOr((unsigned long long *)a.S + p, bit);
        if (olds == 0) {
            a.q0[atomicAdd(&s_nf, 1ull)] = p;
            atomicAdd(&s_mf, (unsigned long long)a.odeg[p]);
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
        *a.ctl = c;
    }
}

// Bottom-up over S[j] -> S[j+1]. kBypass: skip words whose 32 positions are
// done; kEarly: stop a row once every root is accounted for, or at padding.
template <bool kBypass, bool kEarly>
__global__ void k_ms_bu(MsArgs a, int j) {
    const uint64_t *F = slot(a, j);
    uint64_t *N = slot(a, j + 1);
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t stride = (int64_t)gridDim.x * wpb;
    const int L = a.ctl->level;
    const int k = (L + 1) % 3;
    unsigned long long cn = 0, cbits = 0, cmo = 0, cmi = 0, cfull = 0, cedges = 0, bytes = 0;
    unsigned long long cdone = 0;
    for (int64_t w = blockIdx.x * wpb + (threadIdx.x >> 5); w < a.nwords; w += stride) {
        const uint32_t d = __ldg(a.D + w);
        const int64_t p = w * 32 + lane;
        if (kBypass && d == kFull) {
            N[p] = 0;
            continue;
        }
        bytes += 16;
        const uint64_t vis = __ldg(a.V + p);
        bool active = vis != kAll;
        int32_t ng = 0;
        const int4 *cp = nullptr;
        if (active) {
            const int64_t s = p >> a.log2C;
            ng = (__ldg(a.width + s) + 3) >> 2;
            cp = a.col4 + (__ldg(a.slice_off + s) >> 2) + (p & (a.C - 1));
        }
        uint64_t acc = 0;
        for (int32_t g = 0;; g++) {
            active = active && g < ng;
            if (!__any_sync(kFull, active)) break;
            bytes += 16ull * 32;
            if (!active) continue;
            const int4 c = ld_nc(cp + (int64_t)g * a.C);
            // padding entries hold p itself: S[j][p] only has bits already in
            // V[p], so OR-ing it changes nothing
            acc |= __ldg(F + c.x) | __ldg(F + c.y) | __ldg(F + c.z) | __ldg(F + c.w);
            if (kEarly && (c.w == (int32_t)p || (acc | vis) == kAll)) active = false;
        }
        const uint64_t nb = acc & ~vis;
        N[p] = nb;
        bool done_now = false;
        if (nb) {
            const uint64_t nv = vis | nb;
            a.V[p] = nv;
            const int pc = __popcll(nb);
            const int32_t od = __ldg(a.odeg + p);
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
    cn = warp_sum(cn);
    cbits = warp_sum(cbits);
    cmo = warp_sum(cmo);
    cmi = warp_sum(cmi);
    cedges = warp_sum(cedges);
    cdone = warp_sum(cdone);
    if (lane == 0) {
        if (cn) {
            atomicAdd(&a.ctl->acc_n[k], cn);
            atomicAdd(&a.ctl->acc_bits[k], cbits);
            atomicAdd(&a.ctl->acc_mo[k], cmo);
            atomicAdd(&a.ctl->acc_mi[k], cmi);
            atomicAdd(&a.ctl->acc_edges[k], cedges);
            if (cdone) atomicAdd(&a.ctl->acc_done[k], cdone);
        }
        if (cfull) atomicAdd(&a.ctl->acc_full[k], cfull);
        if (bytes) atomicAdd(&a.ctl->acc_bytes[k], bytes);
    }
}

__device__ __forceinline__ uint64_t warp_or64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v |= __shfl_xor_sync(kFull, v, o);
    return v;
}

// Long rows (kept out of the slices): one warp per row ORs the frontier
// words of 32 sources per step and stops once every root is accounted for.
template <bool kEarly>
__global__ void k_ms_bu_long(MsArgs a, int j) {
    if (a.nlong == 0) return;
    const uint64_t *F = slot(a, j);
    uint64_t *N = slot(a, j + 1);
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    const int L = a.ctl->level;
    const int k = (L + 1) % 3;
    unsigned long long cn = 0, cbits = 0, cmo = 0, cmi = 0, cfull = 0, cedges = 0, bytes = 0;
    unsigned long long cdone = 0;
    for (int64_t i = blockIdx.x * wpb + (threadIdx.x >> 5); i < a.nlong; i += nwarps) {
        const int32_t p = __ldg(a.lrow + i);
        const uint64_t vis = __ldg(a.V + p);
        if (vis == kAll) continue;
        const int64_t st = __ldg(a.lptr + i), en = __ldg(a.lptr + i + 1);
        bytes += 24;
        uint64_t acc = 0;
        for (int64_t e0 = st; e0 < en; e0 += 32) {
            const int64_t e = e0 + lane;
            const uint64_t f = e < en ? __ldg(F + __ldg(a.lcol + e)) : 0ull;
            acc |= warp_or64(f);
            bytes += 128;
            if (kEarly && (acc | vis) == kAll) break;
        }
        const uint64_t nb = acc & ~vis;
        if (lane == 0 && nb) {
            N[p] = nb;  // the slice pass wrote 0 here
            const uint64_t nv = vis | nb;
            a.V[p] = nv;
            const int pc = __popcll(nb);
            const int32_t od = __ldg(a.odeg + p);
            cn++;
            cbits += pc;
            cmo += od;
            cedges += (unsigned long long)pc * od;
            if (nv == kAll) {
                cdone++;
                cmi += __ldg(a.ideg + p);
                const uint32_t bit = 1u << (p & 31);
                const uint32_t od2 = atomicOr(a.D + (p >> 5), bit);
                cfull += (od2 != kFull && (od2 | bit) == kFull);
            }
        }
    }
    if (lane == 0 && (cn || bytes)) {
        if (cn) {
            atomicAdd(&a.ctl->acc_n[k], cn);
            atomicAdd(&a.ctl->acc_bits[k], cbits);
            atomicAdd(&a.ctl->acc_mo[k], cmo);
            atomicAdd(&a.ctl->acc_mi[k], cmi);
            atomicAdd(&a.ctl->acc_edges[k], cedges);
            if (cdone) atomicAdd(&a.ctl->acc_done[k], cdone);
        }
        if (cfull) atomicAdd(&a.ctl->acc_full[k], cfull);
        atomicAdd(&a.ctl->acc_bytes[k], bytes);
    }
}

// S[j] -> queue (positions with a non-empty frontier word).
__global__ void k_ms_compact(MsArgs a, int j) {
    const uint64_t *F = slot(a, j);
    const int L = a.ctl->level;
    int32_t *Q = (L & 1) ? a.q1 : a.q0;
    unsigned long long *qslot = &a.ctl->qn[L % 3];
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t stride = (int64_t)gridDim.x * wpb;
    for (int64_t w = blockIdx.x * wpb + (threadIdx.x >> 5); w < a.nwords; w += stride) {
        const int64_t p = w * 32 + lane;
        const bool f = __ldg(F + p) != 0;
        const unsigned m = __ballot_sync(kFull, f);
        if (!m) continue;
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(qslot, (unsigned long long)__popc(m));
        base = __shfl_sync(kFull, base, 0);
        if (f) Q[base + __popc(m & lanemask_lt())] = (int32_t)p;
    }
}

__device__ __forceinline__ bool ms_push(const MsArgs &a, uint64_t *N, int32_t v, uint64_t f) {
    const uint64_t nb = f & ~__ldg(a.V + v);
    return nb && atomicOr((unsigned long long *)N + v, nb) == 0;
}

__device__ __forceinline__ void ms_append(int32_t *NQ, unsigned long long *nq_slot, bool claimed,
                                          int32_t v) {
    const unsigned cm = __ballot_sync(kFull, claimed);
    if (!cm) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(cm) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(nq_slot, (unsigned long long)__popc(cm));
    base = __shfl_sync(kFull, base, leader);
    if (claimed) NQ[base + __popc(cm & lanemask_lt())] = v;
}

constexpr int kMsBigShift = 38;
constexpr unsigned long long kMsBigMask = (1ull << kMsBigShift) - 1;

__global__ void k_ms_td(MsArgs a, int j) {
    const uint64_t *F = slot(a, j);
    uint64_t *N = slot(a, j + 1);
    const int L = a.ctl->level;
    const int32_t *Q = (L & 1) ? a.q1 : a.q0;
    int32_t *NQ = (L & 1) ? a.q0 : a.q1;
    const int64_t qlen = (int64_t)a.ctl->qn[L % 3];
    unsigned long long *nq_slot = &a.ctl->qn[(L + 1) % 3];
    unsigned long long *big_slot = &a.ctl->nbig[L % 3];
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
        const int32_t u = (lane < G && i < qlen) ? Q[i] : -1;
        int64_t st = 0, d = 0;
        uint64_t f = 0;
        if (u >= 0) {
            st = __ldg(a.prow + u);
            d = __ldg(a.prow + u + 1) - st;
            f = __ldg(F + u);
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
        for (int64_t eb = 0; eb < T; eb += 32) {
            const int64_t e = eb + lane;
            bool claimed = false;
            int32_t v = 0;
            if (e < T) {
                int jj = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (s_ex[wib][jj + step] <= e) jj += step;
                v = __ldg(a.pcol + s_st[wib][jj] + (e - s_ex[wib][jj]));
                claimed = ms_push(a, N, v, s_f[wib][jj]);
            }
            ms_append(NQ, nq_slot, claimed, v);
        }
        __syncwarp();
    }
}

// Long frontier rows in kBigChunk-edge chunks over all warps; a chunk finds
// its row by binary search over the chunk bases (monotone in the index).
__global__ void k_ms_td_big(MsArgs a, int j) {
    const int L = a.ctl->level;
    const unsigned long long ctr = a.ctl->nbig[L % 3];
    if (ctr == 0) return;
    const int64_t nbig = (int64_t)(ctr >> kMsBigShift);
    const int64_t total = (int64_t)(ctr & kMsBigMask);
    const uint64_t *F = slot(a, j);
    uint64_t *N = slot(a, j + 1);
    int32_t *NQ = (L & 1) ? a.q0 : a.q1;
    unsigned long long *nq_slot = &a.ctl->qn[(L + 1) % 3];
    const int lane = threadIdx.x & 31;
    const int64_t wpb = blockDim.x >> 5;
    const int64_t gw = blockIdx.x * wpb + (threadIdx.x >> 5);
    const int64_t nwarps = (int64_t)gridDim.x * wpb;
    for (int64_t k = gw; k < total; k += nwarps) {
        int64_t lo = 0, hi = nbig - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (a.big_base[mid] <= k) lo = mid;
            else hi = mid - 1;
        }
        const int32_t u = a.big[lo];
        const int64_t c = k - a.big_base[lo];
        const int64_t st = __ldg(a.prow + u);
        const int64_t d = __ldg(a.prow + u + 1) - st;
        const uint64_t f = __ldg(F + u);
        const int64_t e1 = min(d, (c + 1) * kBigChunk);
        for (int64_t e = c * kBigChunk + lane; e - lane < e1; e += 32) {
            bool claimed = false;
            int32_t v = 0;
            if (e < e1) {
                v = __ldg(a.pcol + st + e);
                claimed = ms_push(a, N, v, f);
            }
            ms_append(NQ, nq_slot, claimed, v);
        }
    }
}

// After a top-down level: fold the new frontier words into V and count.
__global__ void k_ms_td_finish(MsArgs a, int j) {
    const uint64_t *N = slot(a, j + 1);
    const int L = a.ctl->level;
    const int32_t *NQ = (L & 1) ? a.q0 : a.q1;
    const int64_t nqlen = (int64_t)a.ctl->qn[(L + 1) % 3];
    const int k = (L + 1) % 3;
    unsigned long long cn = 0, cbits = 0, cmo = 0, cmi = 0, cfull = 0, cedges = 0, cdone = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nqlen;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = NQ[i];
        const uint64_t nb = N[v];
        const uint64_t old = a.V[v];  // only this thread writes V[v] in this kernel
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
__global__ void k_ms_end(MsArgs a, int dir) {
    if (threadIdx.x >= 32) return;
    __shared__ MsCtl s;
    if (threadIdx.x == 0) {
        MsCtl c = *a.ctl;
        const int k = (c.level + 1) % 3;
        const unsigned long long nn = c.acc_n[k];
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
        c.launches += 1;
        if (nn == 0) c.done = 1;
        // zero the slots level L+1 accumulates into after the next rollover
        const int z = (c.level + 1) % 3;
        c.acc_n[z] = c.acc_mo[z] = c.acc_mi[z] = c.acc_full[z] = c.acc_bits[z] = 0;
        c.acc_edges[z] = c.qn[z] = c.acc_bytes[z] = c.acc_done[z] = c.nbig[z] = 0;
        s = c;
    }
    __syncwarp();
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
    if (threadIdx.x == 0) {
        s.dir = next;
        *a.ctl = s;
    }
}

// Levels of every (vertex, root) pair from the snapshots S[0..nslots):
// thread (p, i) finds the slot holding bit i of p. Rows of 64 int32 per
// vertex (original id), written whole.
__global__ void k_ms_expand(MsArgs a, int nslots, int base, int first, int nroots, int32_t *out) {
    const int64_t total = a.n * 64;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = t >> 6;
        const int i = (int)(t & 63);
        const uint64_t bit = 1ull << i;
        int32_t lvl = -1;
        for (int jj = 0; jj < nslots; jj++)
            if (__ldg(a.S + (int64_t)jj * a.npad + p) & bit) {
                lvl = base + jj;
                break;
            }
        int32_t *o = out + (int64_t)__ldg(a.perm + p) * 64 + i;
        if (i >= nroots) lvl = -1;
        if (first)
            *o = lvl;
        else if (lvl >= 0)
            *o = lvl;
    }
}

struct MsScratch {
    bool ready = false;
    int32_t K = 0;
    uint64_t *V = nullptr, *S = nullptr;
    uint32_t *D = nullptr;
    int32_t *q0 = nullptr, *q1 = nullptr, *big = nullptr;
    int64_t *big_base = nullptr;
    MsCtl *ctl = nullptr, *h_ctl = nullptr;
    int32_t *out = nullptr;
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
    dfree(m.q0);
    dfree(m.q1);
    dfree(m.big);
    dfree(m.big_base);
    dfree(m.ctl);
    dfree(m.out);
    if (m.h_ctl) cudaFreeHost(m.h_ctl);
    delete (MsScratch *)g->ms;
    g->ms = nullptr;
}

namespace {

alb_status ms_alloc(alb_graph *g, MsScratch &m) {
    if (m.ready) return ALB_OK;
    const Sell &s = g->sell;
    const int64_t npad = s.nwords * 32;
    m.K = 32;
    ALB_TRY(dmalloc((void **)&m.V, sizeof(uint64_t) * npad, "msbfs visited"));
    ALB_TRY(dmalloc((void **)&m.S, sizeof(uint64_t) * npad * m.K, "msbfs frontier snapshots"));
    ALB_TRY(dmalloc((void **)&m.D, sizeof(uint32_t) * s.nwords, "msbfs done bitmap"));
    ALB_TRY(dmalloc((void **)&m.q0, sizeof(int32_t) * npad, "msbfs queue"));
    ALB_TRY(dmalloc((void **)&m.q1, sizeof(int32_t) * npad, "msbfs queue"));
    ALB_TRY(dmalloc((void **)&m.big, sizeof(int32_t) * npad, "msbfs long-row list"));
    ALB_TRY(dmalloc((void **)&m.big_base, sizeof(int64_t) * npad, "msbfs long-row chunk bases"));
    ALB_TRY(dmalloc((void **)&m.ctl, sizeof(MsCtl), "msbfs control"));
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
    a.V = m.V;
    a.S = m.S;
    a.D = m.D;
    a.q0 = m.q0;
    a.q1 = m.q1;
    a.big = m.big;
    a.big_base = m.big_base;
    a.ctl = m.ctl;
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
    if (e == cudaSuccess) e = restore ? cp(a.ctl, s.ctl, sizeof(MsCtl)) : cp(s.ctl, a.ctl, sizeof(MsCtl));
    if (e != cudaSuccess) return fail(ALB_ERR_CUDA, "msbfs snapshot: %s", cudaGetErrorString(e));
    return ALB_OK;
}

alb_status msbfs_impl(alb_graph *g, const int32_t *roots, int32_t nroots, const alb_bfs_opts &o,
                      int32_t *d_levels, alb_stats *st, std::vector<alb_level_rec> *trace,
                      std::vector<alb_level_profile> *prof = nullptr) {
    MsScratch &m = ms_scratch(g);
    ALB_TRY(ms_alloc(g, m));
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
    const uint64_t unused = nroots >= 64 ? 0ull : ~((1ull << nroots) - 1);
    ALB_CK(cudaEventRecord(g->ev0, stream));
    k_ms_init<<<wide, 256, 0, stream>>>(a, unused);
    k_ms_roots<<<1, 64, 0, stream>>>(a, in);
    ALB_CK(cudaGetLastError());
    int64_t launches = 2;
    MsCtl *h = m.h_ctl;
    ALB_CK(cudaMemcpyAsync(h, a.ctl, sizeof(MsCtl), cudaMemcpyDeviceToHost, stream));
    ALB_CK(cudaStreamSynchronize(stream));
    // level 0's direction: same decision rule as later levels
    {
        BfsCtl fc;
        std::memset(&fc, 0, sizeof(fc));
        fc.n = h->n;
        fc.nwords = h->nwords;
        fc.nf = h->nf;
        fc.mf = h->mf;
        fc.nu = h->nu;
        fc.mu = h->mu;
        fc.prev_dir = -1;
        fc.policy = o.policy == ALB_POLICY_LEARNED ? ALB_POLICY_BEAMER : o.policy;
        fc.alpha = o.alpha;
        fc.beta = o.beta;
        h->dir = rule_dir(fc);
    }
    int base = 0;      // level held by slot 0
    bool first_flush = true;
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
        ALB_TRY(dmalloc((void **)&snap.ctl, sizeof(MsCtl), "msbfs snapshot"));
    }
    const int32_t level_cap = (int32_t)std::min<int64_t>(g->n + 1, INT32_MAX - 1);
    while (!h->done && h->level < level_cap) {
        const int L = h->level;
        int j = L - base;
        if (j + 1 >= m.K) {
            // snapshot store full: write out levels [base, base + K - 1) and
            // restart the store from the current frontier
            if (d_levels) {
                k_ms_expand<<<wide, 256, 0, stream>>>(a, m.K - 1, base, first_flush ? 1 : 0,
                                                      nroots, d_levels);
                launches++;
            }
            first_flush = false;
            ALB_CK(cudaMemcpyAsync(a.S, a.S + (int64_t)(m.K - 1) * a.npad,
                                   sizeof(uint64_t) * a.npad, cudaMemcpyDeviceToDevice, stream));
            base += m.K - 1;
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
        auto launch_step = [&](int d) -> alb_status {
            if (d == ALB_DIR_TOPDOWN) {
                if (!q_valid) {
                    k_ms_compact<<<wide, block, 0, stream>>>(a, j);
                    launches++;
                }
                ALB_CK(cudaMemsetAsync(a.S + (int64_t)(j + 1) * a.npad, 0,
                                       sizeof(uint64_t) * a.npad, stream));
                k_ms_td<<<wide, block, 0, stream>>>(a, j);
                k_ms_td_big<<<wide, block, 0, stream>>>(a, j);
                k_ms_td_finish<<<wide, block, 0, stream>>>(a, j);
                launches += 3;
            } else if (d == ALB_DIR_BOTTOMUP) {
                k_ms_bu<true, true><<<wide, block, 0, stream>>>(a, j);
                k_ms_bu_long<true><<<wide, block, 0, stream>>>(a, j);
                launches += 2;
            } else {
                k_ms_bu<false, false><<<wide, block, 0, stream>>>(a, j);
                k_ms_bu_long<false><<<wide, block, 0, stream>>>(a, j);
                launches += 2;
            }
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
        k_ms_end<<<1, 32, 0, stream>>>(a, dir);
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
                            : (int64_t)h->acc_bytes[k] + 8 * 3 * a.npad;
            trace->push_back(rec);
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (!h->done) return fail(ALB_ERR_DEVICE, "msbfs: level cap reached");
    if (d_levels) {
        const int nslots = h->level - base;  // slots 0 .. level-base-1 hold levels
        k_ms_expand<<<wide, 256, 0, stream>>>(a, std::min(nslots, m.K), base,
                                              first_flush ? 1 : 0, nroots, d_levels);
        launches++;
    }
    ALB_CK(cudaGetLastError());
    ALB_CK(cudaEventRecord(g->ev1, stream));
    ALB_CK(cudaStreamSynchronize(stream));
    float ms = 0;
    ALB_CK(cudaEventElapsedTime(&ms, g->ev0, g->ev1));
    if (st) {
        st->num_levels = h->level;
        st->levels_topdown = h->levels_td;
        st->levels_bottomup = h->levels_bu;
        st->pad_ = 0;
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
    MsScratch &m = ms_scratch(g);
    if (levels && !m.out) {
        ALB_TRY(dmalloc((void **)&m.out, sizeof(int32_t) * (size_t)g->n * 64, "msbfs levels"));
    }
    ALB_TRY(alb_msbfs64_device(g, roots, nroots, o, levels ? m.out : nullptr, st));
    if (levels) {
        ALB_CK(cudaMemcpyAsync(levels, m.out, sizeof(int32_t) * (size_t)g->n * 64,
                               cudaMemcpyDeviceToHost, g->stream));
        ALB_CK(cudaStreamSynchronize(g->stream));
    }
    return ALB_OK;
}

}  // extern "C"
