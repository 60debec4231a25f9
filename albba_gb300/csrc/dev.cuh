// Device-side types and helpers shared by the CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "albba.h"

namespace alb {

constexpr uint32_t kFull = 0xFFFFFFFFu;
// Top-down: rows longer than kBigRow are pushed in kBigChunk-edge chunks
// shared by every warp instead of by the one warp that dequeued them.
constexpr int64_t kBigRow = 256;
constexpr int64_t kBigChunk = 128;
// Bottom-up: a row kept out of the slices is pulled by one warp over its
// first kLongChunk sources; what remains is split into kLongChunk-source
// chunks spread over all warps (a hub would otherwise hold one warp).
constexpr int64_t kLongChunk = 1024;
// SELL build: rows with more raw entries than this are copied in chunks.
constexpr int64_t kFillChunk = 2048;

// ------------------------------------------------------- checked build
// Built with -DALB_CHECKED (libalbba_gb300_checked.so), every vertex id a
// traversal kernel loads from the matrix or a queue is checked against its
// array before it is used as an index: an id outside [0, limit) records
// ALB_ERR_DEVICE in the control block's error word (no trap) and is replaced
// by `safe`, a value the kernel treats as padding or "no entry". The normal
// build compiles the checks away.
#ifdef ALB_CHECKED
__device__ __forceinline__ int32_t checked_id(int32_t c, int64_t limit, int32_t safe,
                                              int32_t *err) {
    if (c >= 0 && (int64_t)c < limit) return c;
    atomicExch(err, ALB_ERR_DEVICE);
    return safe;
}
#define ALB_CHECK_ID(c, limit, safe, err) ((c) = ::alb::checked_id((c), (limit), (safe), (err)))
#define ALB_CHECK_ID4(c4, limit, safe, err)    \
    do {                                       \
        ALB_CHECK_ID((c4).x, limit, safe, err); \
        ALB_CHECK_ID((c4).y, limit, safe, err); \
        ALB_CHECK_ID((c4).z, limit, safe, err); \
        ALB_CHECK_ID((c4).w, limit, safe, err); \
    } while (0)
#define ALB_CHECK_POS(pos, limit, err) ((pos) >= 0 && (int64_t)(pos) < (int64_t)(limit) \
                                        ? true : (atomicExch((err), ALB_ERR_DEVICE), false))
#else
#define ALB_CHECK_ID(c, limit, safe, err) ((void)0)
#define ALB_CHECK_ID4(c4, limit, safe, err) ((void)0)
#define ALB_CHECK_POS(pos, limit, err) true
#endif

// ---------------------------------------------------------------- loads
// Column and structure arrays are read-only for a whole traversal: read them
// through the non-coherent path. Bitmaps and queues are rewritten between
// levels; inside the persistent kernel they must be read with ordinary
// (L1-coherent after the grid barrier's fence) loads, never .nc.
__device__ __forceinline__ int4 ld_nc(const int4 *p) {
    int4 r;
    asm volatile("ld.global.nc.L1::no_allocate.v4.s32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "l"(p));
    return r;
}
template <class T>
__device__ __forceinline__ T ld_ro(const T *p) { return __ldg(p); }

// L2 eviction policies (PTX createpolicy): the column stream of a level is
// read once and marked evict-first so that the bitmaps it is tested against
// keep their L2 lines.
__device__ __forceinline__ uint64_t l2_evict_first() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
// One 4-byte read-only load with an L2 policy (L1 allocation left as usual).
__device__ __forceinline__ int32_t ld_hint(const int32_t *ptr, uint64_t pol) {
    int32_t r;
    asm volatile("ld.global.nc.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(r) : "l"(ptr), "l"(pol));
    return r;
}
__device__ __forceinline__ int4 ld_stream(const int4 *ptr, uint64_t pol) {
    int4 r;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.s32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "l"(ptr), "l"(pol));
    return r;
}

// ------------------------------------------------- bulk copies (TMA engine)
// A 1-D bulk copy global -> shared completes on an mbarrier that counts the
// bytes delivered (expect_tx). Addresses 16-byte aligned, size a multiple of
// 16 bytes.
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Dynamic distribution of bitmap words to warps. Rows sorted by degree
// inside each sigma window make a word's cost depend on its offset in the
// window, so a fixed grid stride (a multiple of 32 warps) would hand one warp
// the heavy offset of every window; instead each warp takes kGrabWords
// consecutive words at a time from a counter shared by the launch, asking
// for its next run one run ahead. Call from all lanes of a warp.
constexpr int64_t kGrabWords = 8;

__device__ __forceinline__ int64_t grab_words(unsigned long long *ctr) {
    unsigned long long v = 0;
    if ((threadIdx.x & 31) == 0) v = atomicAdd(ctr, (unsigned long long)kGrabWords);
    return (int64_t)__shfl_sync(0xFFFFFFFFu, v, 0);
}

struct WordRuns {
    int64_t end, next;  // end of the current run; start of the one after it
    __device__ __forceinline__ int64_t first(unsigned long long *ctr, int64_t nwords) {
        const int64_t cur = grab_words(ctr);
        next = grab_words(ctr);
        end = min(cur + kGrabWords, nwords);
        return cur;
    }
    // the word after w (>= nwords when the launch's words are exhausted)
    __device__ __forceinline__ int64_t after(int64_t w, unsigned long long *ctr, int64_t nwords) {
        if (w + 1 < end) return w + 1;
        const int64_t cur = next;
        next = grab_words(ctr);
        end = min(cur + kGrabWords, nwords);
        return cur;
    }
};

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

template <class T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
    const unsigned lane = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T t = __shfl_up_sync(kFull, v, o);
        if (lane >= (unsigned)o) v += t;
    }
    return v;
}

// ----------------------------------------------------------- level control
// Counters produced while traversing level L (they describe level L+1) live
// in slot (L+1) % 3. All readers of slot k finish before slot k is zeroed
// again two levels later, so the persistent kernel needs no extra barrier
// for the rollover.
struct BfsCtl {
    int32_t level;    // depth of the current frontier
    int32_t dir;      // ALB_DIR_* chosen for the current level
    int32_t prev_dir; // direction of the previous level (-1 at level 0)
    int32_t q_valid;  // queue[level & 1] lists the current frontier
    int32_t n_dirty;  // bitmap[(level + 1) & 1] may hold stale bits
    int32_t done;
    int32_t err;      // ALB_ERR_* raised on the device (0 = none)
    int32_t policy;
    float alpha, beta;
    int32_t levels_td, levels_bu;
    int64_t n;               // vertices
    int64_t nwords;          // 32-bit words per bitmap
    int64_t nf, mf;          // current frontier: vertices, push-side entries
    int64_t prev_nf;
    int64_t nu, mu;          // unvisited vertices / pull-side entries
    int64_t active_words;    // bitmap words with an unvisited row
    int64_t reached, edges;  // running totals
    unsigned long long acc_n[3], acc_mo[3], acc_mi[3], acc_full[3], qn[3], acc_bytes[3];
    unsigned long long nbig[3];  // rows too long for one warp, per level slot
    unsigned long long work[3];  // bottom-up word counter (grab_words), per level slot
    unsigned long long acc_stat[3][5];  // bypass statistics per level slot (kSt*)
    int32_t trace_cap, trace_len;
    int32_t level_cap;       // safety bound on the number of levels
    int32_t branch;          // loop-graph switch branch taken this level
    int32_t lazy;            // persistent loop: visited / frontier bitmaps stale,
                             // level_pos authoritative (materialize before use)
    unsigned long long acc_active[3];  // words with an unvisited row, counted
                                       // when the bitmaps are rebuilt
    int64_t launches;        // kernel launches of the level loop
    float feat_mean_deg, feat_skew;  // static selector features
};

// Bypass statistics accumulated per level (alb_level_rec).
enum LevelStat : int {
    kStWordsBypassed = 0,
    kStRowsScanned = 1,
    kStGroupsRead = 2,
    kStGroupsTotal = 3,
    kStEdgesBypassed = 4,
    kStatN = 5,
};

// Per-traversal device arguments (passed by value to every kernel).
struct BfsArgs {
    int64_t n, nslices, nwords;
    int32_t C, log2C;
    const int32_t *perm;       // position -> original id
    const int32_t *inv;        // original id -> position
    const int32_t *ideg;       // pull-side row length by position
    const int32_t *odeg;       // push-side row length by position
    const int32_t *width;      // slice width (max row length)
    const int64_t *slice_off;  // slice start, int32 entries
    const int4 *col4;          // SELL columns, 4-interleaved
    const int64_t *prow;       // push CSR (position space)
    const int32_t *pcol;
    int64_t nlong;             // rows kept out of the slices
    const int32_t *lrow;
    const int64_t *lptr;
    const int32_t *lcol;
    const uint32_t *vinit;     // initial visited mask
    uint32_t *bm0, *bm1;       // frontier bitmaps (by level parity)
    uint32_t *vis;             // visited bitmap
    int32_t *q0, *q1;          // frontier queues (by level parity)
    int32_t *big;              // frontier rows split across all warps (top-down)
    int64_t *big_base;         // their first chunk index
    int32_t *level_pos;        // depth by position
    uint32_t *parent_pos;      // parent original id by position
    BfsCtl *ctl;
    unsigned long long *bar;   // persistent-kernel grid barrier: arrivals (bit 62: gave up),
                               // its own allocation, apart from the counters' cache lines
    alb_level_rec *trace;
    const float *mlp;          // selector parameters or null
    // bounded waits (DeviceWaits): limits and test hooks
    uint64_t barrier_ns, bulk_ns;
    int32_t withhold_level, withhold_block, short_bulk;
};

// Shared by host and device: pick the direction for the current level.
__host__ __device__ inline int beamer_dir(const BfsCtl &c) {
    if (c.prev_dir < 0 || c.prev_dir == ALB_DIR_TOPDOWN) {
        // top-down -> bottom-up when the frontier's edges exceed m_u / alpha
        return ((double)c.mf > (double)c.mu / (double)c.alpha) ? ALB_DIR_BOTTOMUP
                                                               : ALB_DIR_TOPDOWN;
    }
    // stay bottom-up while the frontier grows or is large
    bool stay = (c.nf >= c.prev_nf) || ((double)c.nf > (double)c.n / (double)c.beta);
    return stay ? ALB_DIR_BOTTOMUP : ALB_DIR_TOPDOWN;
}

__host__ __device__ inline int rule_dir(const BfsCtl &c) {
    switch (c.policy) {
        case ALB_POLICY_TOPDOWN:
            return ALB_DIR_TOPDOWN;
        case ALB_POLICY_BOTTOMUP:
            return c.level == 0 ? ALB_DIR_TOPDOWN : ALB_DIR_BOTTOMUP;
        case ALB_POLICY_BOTTOMUP_NOBYPASS:
            return c.level == 0 ? ALB_DIR_TOPDOWN : ALB_DIR_BOTTOMUP_NOBYPASS;
        case ALB_POLICY_REF004: {
            // SWITCH = (int)(nrows * 0.04); pull when nnzx > SWITCH
            int64_t thr = (int64_t)((double)c.n * 0.04);
            return c.nf > thr ? ALB_DIR_BOTTOMUP : ALB_DIR_TOPDOWN;
        }
        default:
            return beamer_dir(c);
    }
}

}  // namespace alb
