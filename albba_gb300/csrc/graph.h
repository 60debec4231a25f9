// The device-resident graph behind the opaque alb_graph handle.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "albba.h"
#include "dev.cuh"
#include "internal.h"

namespace alb {

// Device allocation with host fault injection; returns ALB_OK or ALB_ERR_OOM.
alb_status dmalloc(void **p, size_t bytes, const char *what);
void dfree(void *p);
// Blocks of `block` threads of func resident on one SM at once (cached per
// function and block size; 0 if the query fails).
int resident_blocks(const void *func, int block);

// Launches a grid-stride kernel with as many blocks as are resident at once
// (2048 / block per SM if the occupancy query fails).
template <class... P, class... A>
void launch_resident(void (*f)(P...), int block, int num_sms, cudaStream_t st, A &&...args) {
    const int per = resident_blocks((const void *)f, block);
    const int fallback = 2048 / block > 0 ? 2048 / block : 1;
    const unsigned grid = (unsigned)(num_sms * (per > 0 ? per : fallback));
    f<<<grid, block, 0, st>>>(static_cast<A &&>(args)...);
}

// CUDA error check that records the failing call and returns ALB_ERR_CUDA.
#define ALB_CK(call)                                                                 \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            cudaGetLastError();                                                      \
            return ::alb::fail(ALB_ERR_CUDA, "%s failed: %s (%s:%d)", #call,        \
                               cudaGetErrorString(e_), __FILE__, __LINE__);          \
        }                                                                            \
    } while (0)

#define ALB_TRY(expr)                        \
    do {                                     \
        alb_status s_ = (expr);              \
        if (s_ != ALB_OK) return s_;         \
    } while (0)

// Phase timer for the host-visible entry points: with ALB_TRACE_PHASES set
// in the environment, mark() waits for the stream and prints the wall time
// of the phase that just ended to stderr; otherwise it does nothing.
struct PhaseLog {
    bool on = false;
    const char *call = "";
    double t = 0;
    PhaseLog(const char *c);
    void mark(const char *phase, cudaStream_t st);
};

struct CachedLoop;  // CUDA graph for the device-driven level loop (bfs.cu)

struct Sell {
    bool built = false;
    int32_t C = 32, log2C = 5, sigma = 1024;
    int64_t nslices = 0, nwords = 0, ncol = 0;
    int32_t *perm = nullptr, *inv = nullptr, *ideg = nullptr, *odeg = nullptr;
    int32_t *width = nullptr;
    int64_t *slice_off = nullptr;
    int32_t *col = nullptr;
    int64_t *prow = nullptr;
    int32_t *pcol = nullptr;
    uint32_t *vinit = nullptr;
    // rows longer than long_row: empty in the SELL, pulled warp-cooperatively
    int32_t long_row = 0;
    int64_t nlong = 0;
    int32_t *lrow = nullptr;   // their positions, ascending
    int64_t *lptr = nullptr;   // nlong + 1 offsets into lcol
    int32_t *lcol = nullptr;   // their sources (positions), row order
    int64_t m_in = 0, m_out = 0;   // entries without self-loops
    int64_t active0 = 0;           // words of vinit that are not full
    int64_t zero_in = 0;           // rows without sources
    int32_t max_deg = 0;
};

struct BfsScratch {
    bool ready = false;
    uint32_t *bits = nullptr;  // one allocation: bm0 | bm1 | vis
    uint32_t *bm0 = nullptr, *bm1 = nullptr, *vis = nullptr;
    // L2 persisting-access window over `bits`, used when the frontier bitmap
    // is too large to stage in shared memory (num_bytes == 0: none)
    cudaAccessPolicyWindow win = {};
    int32_t *q0 = nullptr, *q1 = nullptr;
    int32_t *big = nullptr;
    int64_t *big_base = nullptr;
    int32_t *level_pos = nullptr;
    uint32_t *parent_pos = nullptr;
    int32_t *out_level = nullptr, *out_parent = nullptr;  // staging for host outputs
    BfsCtl *ctl = nullptr;
    BfsCtl *h_ctl = nullptr;  // pinned mirror
    unsigned long long *bar = nullptr;  // persistent-kernel grid barrier
    alb_level_rec *trace = nullptr;
    int32_t trace_cap = 0;
};

}  // namespace alb

struct alb_graph {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;      // stream in use
    cudaStream_t own_stream = nullptr;  // created with the graph
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int64_t n = 0;
    int64_t nnz_in = 0, nnz_out = 0;
    bool symmetric = false;
    // original-id CSRs on the device (pull side = sources, push side = targets)
    int64_t *rp_in = nullptr;
    int32_t *col_in = nullptr;
    int64_t *rp_out = nullptr;
    int32_t *col_out = nullptr;
    alb::Sell sell;
    alb::BfsScratch bfs;
    alb::CachedLoop *loop = nullptr;
    void *ms = nullptr;  // 64-root BFS scratch (msbfs.cu)
    std::vector<alb_level_rec> last_trace;
    bool last_trace_valid = false;
};

namespace alb {
alb_status bfs_scratch_alloc(alb_graph *g);
void bfs_scratch_free(alb_graph *g);
void ms_scratch_free(alb_graph *g);
float skew_of(const Sell &s, int64_t n);
void loop_cache_free(alb_graph *g);
// perm = positions -> rows, rows sorted by d_len descending (stable) inside
// windows of sigma rows (sigma <= 1: identity); the reference's
// get_order_by_row_size_radix (bfs/src/sorting_utils.c:232-253).
alb_status window_order(int64_t n, int32_t sigma, const int32_t *d_len, int32_t *d_perm,
                        cudaStream_t st);
BfsArgs make_args(alb_graph *g);
}  // namespace alb
