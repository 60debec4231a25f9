// alb_bfs_csr_noalloc: single-root BFS that allocates nothing.
//
// Some callers cannot call cudaMalloc: a plug-in living inside a host process
// whose device memory belongs to another allocator (a framework's caching
// allocator that must account for every byte, a fixed-budget serving process
// that reserves all device memory up front). For them this entry point runs a
// BFS on a CSR the caller already holds on the device, writes levels and
// parents to caller buffers, and keeps every temporary in one file-scope
// device array (kNoAllocScratchBytes = 8,782,080 bytes) that each GPU loading
// the library holds until the process exits.
//
// The array is shared by all calls on a device and keeps the last call's
// contents; each call clears what must start at zero. Calls that overlap on
// the GPU (two streams, two threads) race on the array: serialise them.
// In host code the array's name is not a device address: the first call on a
// device (and the first call after that device's context was destroyed and
// recreated, e.g. by cudaDeviceReset) looks up its address with
// cudaGetSymbolAddress, with that device current, and caches it keyed on the
// context's unique id; make that first call before any stream capture.
// Each call waits for the given stream once, to read the traversal's status.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "albba.h"
#include "dev.cuh"
#include "graph.h"

namespace alb {
namespace {

constexpr int64_t kNoAllocMaxN = int64_t(1) << 20;   // vertices
constexpr int64_t kNoAllocWords = kNoAllocMaxN / 32;  // bitmap words
constexpr uint64_t kNoAllocTimeoutNs = 4ull * 1000 * 1000 * 1000;

// Layout of the static scratch (offsets in bytes, each 256-aligned):
//   control block | visited | frontier | next | queue0 | queue1
struct NaCtl {
    unsigned long long qn[2];       // queue lengths by level parity
    unsigned long long nn, mo, mi;  // next-level counters
    unsigned int bar_count, bar_gen;
    int32_t err, level, done, pad;
};
constexpr size_t kCtlBytes = 256;
constexpr size_t kBitmapBytes = kNoAllocWords * 4;
constexpr size_t kQueueBytes = kNoAllocMaxN * 4;
constexpr size_t kOffVis = kCtlBytes;
constexpr size_t kOffF = kOffVis + kBitmapBytes;
constexpr size_t kOffN = kOffF + kBitmapBytes;
constexpr size_t kOffQ0 = kOffN + kBitmapBytes;
constexpr size_t kOffQ1 = kOffQ0 + kQueueBytes;
constexpr size_t kNoAllocScratchBytes = kOffQ1 + kQueueBytes;
static_assert(sizeof(NaCtl) <= kCtlBytes, "control block");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NaArgs {
    int64_t n;
    const int64_t *rp;
    const int32_t *col;
    int32_t root;
    int32_t symmetric;
    float alpha, beta;
    int32_t *level, *parent;
    unsigned char *scratch;  // device address of g_noalloc_scratch
    uint64_t barrier_ns;     // bound of every barrier wait
    int32_t withhold_level, withhold_block;  // test hook (DeviceWaits)
};

__device__ bool na_sync(NaCtl *c, unsigned nblocks, const NaArgs &a, int L) {
    // test hook: one block skips its arrival at level L's barriers and leaves
    if (a.withhold_level >= 0 && L == a.withhold_level && (int)blockIdx.x == a.withhold_block)
        return false;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = &c->bar_gen;
        const unsigned g0 = *gen;
        __threadfence();
        if (atomicAdd(&c->bar_count, 1u) == nblocks - 1) {
            atomicExch(&c->bar_count, 0u);
            __threadfence();
            atomicAdd(&c->bar_gen, 1u);
        } else {
            const uint64_t t0 = globaltimer_ns();
            while (*gen == g0) {
                if (globaltimer_ns() - t0 > a.barrier_ns) {
                    atomicExch(&c->err, ALB_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int32_t *)&c->err == 0;
}

// One cooperative kernel for the whole traversal: clear, seed, then per level
// a top-down push (queue, atomicMin parents, atomicOr claims) or, for a
// symmetric graph, a bottom-up pull (first frontier source in the row, which
// is the smallest when the row is ascending); Beamer alpha/beta picks the
// direction.
__global__ void k_bfs_noalloc(NaArgs a) {
    NaCtl *c = (NaCtl *)a.scratch;
    uint32_t *V = (uint32_t *)(a.scratch + kOffVis);
    uint32_t *F = (uint32_t *)(a.scratch + kOffF);
    uint32_t *N = (uint32_t *)(a.scratch + kOffN);
    int32_t *Q[2] = {(int32_t *)(a.scratch + kOffQ0), (int32_t *)(a.scratch + kOffQ1)};
    const unsigned nb = gridDim.x;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int64_t gw = tid >> 5, nwarps = nth >> 5;
    const int64_t nwords = (a.n + 31) / 32;
    const int64_t m = a.rp[a.n];
    for (int64_t w = tid; w < nwords; w += nth) {
        V[w] = 0;
        F[w] = 0;
        N[w] = 0;
    }
    for (int64_t v = tid; v < a.n; v += nth) {
        a.level[v] = -1;
        a.parent[v] = -1;
    }
    if (tid == 0) {
        c->qn[0] = 1;
        c->qn[1] = 0;
        c->nn = c->mo = c->mi = 0;
        c->err = 0;
    }
    if (!na_sync(c, nb, a, -1)) return;
    if (tid == 0) {
        const int32_t r = a.root;
        V[r >> 5] |= 1u << (r & 31);
        F[r >> 5] |= 1u << (r & 31);
        Q[0][0] = r;
        a.level[r] = 0;
        a.parent[r] = r;
    }
    if (!na_sync(c, nb, a, -1)) return;
    int64_t nf = 1, prev_nf = 0;
    int64_t mf = a.rp[a.root + 1] - a.rp[a.root];
    int64_t mu = m - mf;
    int prev_dir = 0;
    bool dense = false;  // F holds the frontier (true) or only Q does (false)
    for (int L = 0; nf > 0 && L <= a.n; L++) {
        int dir = 0;
        if (a.symmetric) {
            if (prev_dir == 0)
                dir = ((double)mf > (double)mu / a.alpha) ? 1 : 0;
            else
                dir = (nf >= prev_nf || (double)nf > (double)a.n / a.beta) ? 1 : 0;
        }
        int32_t *Qc = Q[L & 1], *Qn = Q[(L + 1) & 1];
        const int64_t qlen = (int64_t)*(volatile unsigned long long *)&c->qn[L & 1];
        if (dir == 0) {
            if (dense) {  // frontier only in F: rebuild the queue from it
                if (tid == 0) c->qn[L & 1] = 0;
                if (!na_sync(c, nb, a, L)) return;
                for (int64_t w = tid; w < nwords; w += nth) {
                    uint32_t word = __ldcg(F + w);
                    while (word) {
                        const int b = __ffs(word) - 1;
                        word &= word - 1;
                        Qc[atomicAdd(&c->qn[L & 1], 1ull)] = (int32_t)(w * 32 + b);
                    }
                }
                if (!na_sync(c, nb, a, L)) return;
            }
            const int64_t ql = (int64_t)*(volatile unsigned long long *)&c->qn[L & 1];
            unsigned long long cn = 0, cmo = 0;
            for (int64_t i = gw; i < ql; i += nwarps) {
                const int32_t u = *(volatile int32_t *)(Qc + i);
                for (int64_t e = a.rp[u] + lane; e < a.rp[u + 1]; e += 32) {
                    const int32_t v = a.col[e];
                    const uint32_t bit = 1u << (v & 31);
                    if (__ldcg(V + (v >> 5)) & bit) continue;
                    // parent starts at -1, i.e. UINT_MAX as unsigned: min over sources
                    atomicMin((unsigned int *)(a.parent + v), (unsigned int)u);
                    if (!(atomicOr(N + (v >> 5), bit) & bit)) {
                        Qn[atomicAdd(&c->qn[(L + 1) & 1], 1ull)] = v;
                        a.level[v] = L + 1;
                        cn++;
                        cmo += a.rp[v + 1] - a.rp[v];
                    }
                }
            }
            if (cn) {
                atomicAdd(&c->nn, cn);
                atomicAdd(&c->mo, cmo);
            }
            if (!na_sync(c, nb, a, L)) return;
            // V |= N; F <- N; N <- 0 (dense over the bitmap words)
            for (int64_t w = tid; w < nwords; w += nth) {
                const uint32_t x = __ldcg(N + w);
                V[w] |= x;
                F[w] = x;
                N[w] = 0;
            }
            dense = false;
        } else {
            unsigned long long cn = 0, cmo = 0;
            for (int64_t v = tid; v < a.n; v += nth) {
                const uint32_t bit = 1u << (v & 31);
                if (__ldcg(V + (v >> 5)) & bit) continue;
                for (int64_t e = a.rp[v]; e < a.rp[v + 1]; e++) {
                    const int32_t u = a.col[e];
                    if ((__ldcg(F + (u >> 5)) >> (u & 31)) & 1u) {
                        a.parent[v] = u;
                        a.level[v] = L + 1;
                        atomicOr(N + (v >> 5), bit);
                        cn++;
                        cmo += a.rp[v + 1] - a.rp[v];
                        break;
                    }
                }
            }
            if (cn) {
                atomicAdd(&c->nn, cn);
                atomicAdd(&c->mo, cmo);
            }
            if (!na_sync(c, nb, a, L)) return;
            for (int64_t w = tid; w < nwords; w += nth) {
                const uint32_t x = __ldcg(N + w);
                V[w] |= x;
                F[w] = x;
                N[w] = 0;
            }
            dense = true;
        }
        (void)qlen;
        if (tid == 0) c->qn[L & 1] = 0;
        if (!na_sync(c, nb, a, L)) return;
        prev_nf = nf;
        nf = (int64_t)*(volatile unsigned long long *)&c->nn;
        mf = (int64_t)*(volatile unsigned long long *)&c->mo;
        mu -= mf;
        prev_dir = dir;
        if (!na_sync(c, nb, a, L)) return;  // everyone has read the counters
        if (tid == 0) {
            c->nn = 0;
            c->mo = 0;
            c->level = L + 1;
        }
        if (!na_sync(c, nb, a, L)) return;
    }
    if (tid == 0) c->done = 1;
}

// Device address of g_noalloc_scratch per device ordinal, valid for the
// context whose unique id is stored beside it: a context destroyed and
// recreated (cudaDeviceReset) may load the module at another address.
struct NaCache {
    unsigned long long ctx_id;
    unsigned char *ptr;
};
std::mutex g_na_mu;
NaCache g_na_cache[64] = {};

typedef int (*PfnCtxGetCurrent)(void **);
typedef int (*PfnCtxGetId)(void *, unsigned long long *);

// Unique id of the calling thread's current context (driver API through the
// runtime's entry-point query, so the library does not link libcuda).
cudaError_t current_ctx_id(unsigned long long *id) {
    static PfnCtxGetCurrent get_cur = nullptr;
    static PfnCtxGetId get_id = nullptr;
    if (!get_cur || !get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                                         cudaEnableDefault, &q1);
        if (e == cudaSuccess)
            e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess) return e;
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return cudaErrorNotSupported;
        get_cur = (PfnCtxGetCurrent)f1;
        get_id = (PfnCtxGetId)f2;
    }
    void *ctx = nullptr;
    if (get_cur(&ctx) != 0) return cudaErrorInitializationError;
    if (!ctx) return cudaErrorDeviceUninitialized;
    if (get_id(ctx, id) != 0) return cudaErrorInitializationError;
    return cudaSuccess;
}

}  // namespace
}  // namespace alb

using namespace alb;

extern "C" alb_status alb_bfs_csr_noalloc(int64_t n, const int64_t *d_rowptr, const int32_t *d_col,
                                          int32_t symmetric, int32_t root, int32_t *d_level,
                                          int32_t *d_parent, void *stream) {
    if (n <= 0 || !d_rowptr || !d_col || !d_level || !d_parent || root < 0 || root >= n)
        return fail(ALB_ERR_INVALID, "alb_bfs_csr_noalloc: bad arguments");
    if (n > kNoAllocMaxN)
        return fail(ALB_ERR_UNSUPPORTED,
                    "alb_bfs_csr_noalloc: n = %lld exceeds the fixed scratch limit of %lld vertices",
                    (long long)n, (long long)kNoAllocMaxN);
    int dev = 0;
    ALB_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(ALB_ERR_UNSUPPORTED, "alb_bfs_csr_noalloc: device id %d", dev);
    unsigned long long ctx_id = 0;
    {
        cudaError_t e = current_ctx_id(&ctx_id);
        if (e == cudaErrorDeviceUninitialized) {
            // no context yet on this thread: make the device's primary context
            // current (initialising it if needed), then ask again
            ALB_CK(cudaSetDevice(dev));
            e = current_ctx_id(&ctx_id);
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(ALB_ERR_CUDA, "alb_bfs_csr_noalloc: current context: %s",
                        cudaGetErrorString(e));
        }
    }
    unsigned char *scratch;
    {
        std::lock_guard<std::mutex> lk(g_na_mu);
        NaCache &c = g_na_cache[dev];
        if (!c.ptr || c.ctx_id != ctx_id) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return fail(ALB_ERR_CUDA, "alb_bfs_csr_noalloc: cudaGetSymbolAddress: %s",
                            cudaGetErrorString(e));
            }
            c.ptr = (unsigned char *)p;
            c.ctx_id = ctx_id;
        }
        scratch = c.ptr;
    }
    cudaStream_t st = (cudaStream_t)stream;
    // the barrier counter must start at zero (the previous call leaves it so,
    // unless it was interrupted)
    ALB_CK(cudaMemsetAsync(scratch, 0, kCtlBytes, st));
    NaArgs a;
    a.n = n;
    a.rp = d_rowptr;
    a.col = d_col;
    a.root = root;
    a.symmetric = symmetric ? 1 : 0;
    a.alpha = 14.0f;
    a.beta = 24.0f;
    a.level = d_level;
    a.parent = d_parent;
    a.scratch = scratch;
    const DeviceWaits dw = device_waits(kNoAllocTimeoutNs, kNoAllocTimeoutNs);
    a.barrier_ns = dw.barrier_ns;
    a.withhold_level = dw.withhold_level;
    a.withhold_block = dw.withhold_block;
    int per_sm = 0, sms = 0;
    ALB_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bfs_noalloc, 256, 0));
    ALB_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (per_sm < 1) return fail(ALB_ERR_CUDA, "alb_bfs_csr_noalloc: kernel does not fit");
    void *kargs[] = {&a};
    ALB_CK(cudaLaunchCooperativeKernel((void *)k_bfs_noalloc, dim3(per_sm * sms), dim3(256), kargs,
                                       0, st));
    NaCtl hc;
    ALB_CK(cudaMemcpyAsync(&hc, scratch, sizeof(hc), cudaMemcpyDeviceToHost, st));
    ALB_CK(cudaStreamSynchronize(st));
    if (hc.err) return fail(hc.err, "alb_bfs_csr_noalloc: device-side wait gave up");
    if (!hc.done) return fail(ALB_ERR_DEVICE, "alb_bfs_csr_noalloc: traversal did not finish");
    return ALB_OK;
}
