// Persistent work-list BFS: many (graph, root) traversals of small and
// uneven graphs in one launch. No counterpart in the reference, which runs
// one graph per process (bfs/src/main.c).
//
// One CTA runs one traversal at a time and pops the next (graph, root) item
// from a global counter; items are ordered longest first (stored entries),
// so the tail of the launch holds the short ones. The three bitmaps of the
// traversal (frontier, next frontier, visited; one bit per sorted position)
// live in shared memory, so bottom-up frontier tests and top-down visited
// probes never leave the SM; the SELL-C-sigma and push-CSR arrays of each
// graph stay in HBM, built by alb_sell_build with that graph's own C, sigma
// and long-row threshold. Direction: Beamer alpha/beta per graph.
// Output: level arrays (original ids), one per item, concatenated in the
// order items were added. Graphs whose three bitmaps do not fit in one CTA's
// shared memory are not refused: their items run one by one on the
// device-driven single-root path (alb_bfs_device, CUDA-graph level loop,
// the entry's alpha and beta) into the same output, before the launch.
#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "graph.h"

namespace alb {
namespace {

struct WlGraph {
    int64_t n, nwords;
    int32_t C, log2C;
    const int32_t *perm, *inv, *ideg, *odeg, *width;
    const int64_t *slice_off;
    const int4 *col4;
    const int64_t *prow;
    const int32_t *pcol;
    int64_t nlong;
    const int32_t *lrow;
    const int64_t *lptr;
    const int32_t *lcol;
    const uint32_t *vinit;
    int64_t m_in;
    float alpha, beta;
};

struct WlItem {
    int32_t graph, root;
    int64_t out;  // offset of this item's level array
};

struct WlCounters {
    unsigned long long n, mo, mi;
};

__global__ void k_worklist(const WlGraph *graphs, const WlItem *items, int32_t nitems,
                           unsigned int *next_item, int32_t *out) {
    extern __shared__ uint32_t sm[];
    __shared__ int s_item;
    __shared__ WlCounters s_acc;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    while (true) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(next_item, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= nitems) break;
        const WlItem item = items[it];
        const WlGraph g = graphs[item.graph];
        uint32_t *F = sm, *N = sm + g.nwords, *V = sm + 2 * g.nwords;
        int32_t *lv = out + item.out;
        for (int64_t w = threadIdx.x; w < g.nwords; w += blockDim.x) {
            V[w] = g.vinit[w];
            F[w] = 0;
            N[w] = 0;
        }
        for (int64_t v = threadIdx.x; v < g.n; v += blockDim.x) lv[v] = -1;
        __syncthreads();
        int64_t nf = 1, mf, prev_nf = 0, mu;
        int prev_dir = -1;
        if (threadIdx.x == 0) {
            const int32_t rp = g.inv[item.root];
            V[rp >> 5] |= 1u << (rp & 31);
            F[rp >> 5] |= 1u << (rp & 31);
            lv[item.root] = 0;
        }
        {
            const int32_t rp = g.inv[item.root];
            mf = g.odeg[rp];
            mu = g.m_in - g.ideg[rp];
        }
        __syncthreads();
        for (int L = 0; nf > 0 && L <= g.n; L++) {
            // Beamer decision (identical in every thread)
            int dir;
            if (prev_dir < 0 || prev_dir == ALB_DIR_TOPDOWN)
                dir = ((double)mf > (double)mu / g.alpha) ? ALB_DIR_BOTTOMUP : ALB_DIR_TOPDOWN;
            else
                dir = (nf >= prev_nf || (double)nf > (double)g.n / g.beta) ? ALB_DIR_BOTTOMUP
                                                                           : ALB_DIR_TOPDOWN;
            if (threadIdx.x == 0) s_acc.n = s_acc.mo = s_acc.mi = 0;
            __syncthreads();
            unsigned long long cn = 0, cmo = 0, cmi = 0;
            if (dir == ALB_DIR_BOTTOMUP) {
                for (int64_t w = wib; w < g.nwords; w += nw) {
                    const uint32_t vis = V[w];
                    if (vis == kFull) {
                        if (lane == 0) N[w] = 0;
                        continue;
                    }
                    const int32_t p = (int32_t)(w * 32 + lane);
                    bool active = !((vis >> lane) & 1u);
                    int32_t ng = 0;
                    const int4 *cp = nullptr;
                    if (active) {
                        const int64_t s = (int64_t)p >> g.log2C;
                        ng = (__ldg(g.width + s) + 3) >> 2;
                        cp = g.col4 + (__ldg(g.slice_off + s) >> 2) + (p & (g.C - 1));
                    }
                    bool found = false;
                    for (int32_t j = 0;; j++) {
                        active = active && j < ng;
                        if (!__any_sync(kFull, active)) break;
                        if (!active) continue;
                        const int4 c = ld_nc(cp + (int64_t)j * g.C);
                        const int32_t cc[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            if (!active) break;
                            if (cc[k] == p) {
                                active = false;
                            } else if ((F[cc[k] >> 5] >> (cc[k] & 31)) & 1u) {
                                found = true;
                                active = false;
                            }
                        }
                    }
                    const unsigned nm = __ballot_sync(kFull, found);
                    if (lane == 0) {
                        N[w] = nm;
                        V[w] = vis | nm;
                    }
                    if (found) {
                        lv[__ldg(g.perm + p)] = L + 1;
                        cn++;
                        cmo += __ldg(g.odeg + p);
                        cmi += __ldg(g.ideg + p);
                    }
                }
                __syncthreads();
                // long rows: one warp each, frontier tests in shared memory
                for (int64_t i = wib; i < g.nlong; i += nw) {
                    const int32_t p = __ldg(g.lrow + i);
                    const uint32_t bit = 1u << (p & 31);
                    if (V[p >> 5] & bit) continue;
                    const int64_t st = __ldg(g.lptr + i), en = __ldg(g.lptr + i + 1);
                    bool found = false;
                    for (int64_t e0 = st; e0 < en && !found; e0 += 32) {
                        const int64_t e = e0 + lane;
                        const int32_t c = e < en ? __ldg(g.lcol + e) : p;
                        found = __any_sync(kFull, (F[c >> 5] >> (c & 31)) & 1u);
                    }
                    if (found && lane == 0) {
                        atomicOr(&N[p >> 5], bit);
                        atomicOr(&V[p >> 5], bit);
                        lv[__ldg(g.perm + p)] = L + 1;
                        cn++;
                        cmo += __ldg(g.odeg + p);
                        cmi += __ldg(g.ideg + p);
                    }
                }
            } else {
                // top-down: walk the set bits of F, one warp per frontier row
                for (int64_t w = wib; w < g.nwords; w += nw) {
                    uint32_t word = F[w];
                    while (word) {
                        const int b = __ffs(word) - 1;
                        word &= word - 1;
                        const int32_t u = (int32_t)(w * 32 + b);
                        const int64_t st = __ldg(g.prow + u), en = __ldg(g.prow + u + 1);
                        for (int64_t e = st + lane; e < en; e += 32) {
                            const int32_t v = __ldg(g.pcol + e);
                            const uint32_t bit = 1u << (v & 31);
                            if (V[v >> 5] & bit) continue;
                            if (!(atomicOr(&N[v >> 5], bit) & bit)) {
                                lv[__ldg(g.perm + v)] = L + 1;
                                cn++;
                                cmo += __ldg(g.odeg + v);
                                cmi += __ldg(g.ideg + v);
                            }
                        }
                    }
                }
                __syncthreads();
                for (int64_t w = threadIdx.x; w < g.nwords; w += blockDim.x) V[w] |= N[w];
            }
            cn = warp_sum(cn);
            cmo = warp_sum(cmo);
            cmi = warp_sum(cmi);
            if (lane == 0 && cn) {
                atomicAdd(&s_acc.n, cn);
                atomicAdd(&s_acc.mo, cmo);
                atomicAdd(&s_acc.mi, cmi);
            }
            __syncthreads();
            // N becomes the frontier; the old frontier is cleared for reuse
            uint32_t *t = F;
            F = N;
            N = t;
            for (int64_t w = threadIdx.x; w < g.nwords; w += blockDim.x) N[w] = 0;
            prev_nf = nf;
            nf = (int64_t)s_acc.n;
            mf = (int64_t)s_acc.mo;
            mu -= (int64_t)s_acc.mi;
            prev_dir = dir;
            __syncthreads();
        }
        __syncthreads();
    }
}

}  // namespace
}  // namespace alb

struct alb_worklist {
    struct Entry {
        alb_graph *g;
        std::vector<int32_t> roots;
        float alpha, beta;
    };
    std::vector<Entry> entries;
    int64_t total_out = 0;
};

using namespace alb;

extern "C" {

alb_status alb_worklist_create(alb_worklist **out) {
    if (!out) return fail(ALB_ERR_INVALID, "alb_worklist_create: out is NULL");
    try {
        *out = new alb_worklist();
    } catch (const std::bad_alloc &) {
        return fail(ALB_ERR_OOM, "alb_worklist_create: host allocation failed");
    }
    return ALB_OK;
}

void alb_worklist_destroy(alb_worklist *w) { delete w; }

alb_status alb_worklist_add(alb_worklist *w, alb_graph *g, const int32_t *roots, int32_t nroots,
                            float alpha, float beta) {
    if (!w || !g || !roots || nroots < 1) return fail(ALB_ERR_INVALID, "alb_worklist_add: bad arguments");
    if (!g->sell.built) return fail(ALB_ERR_STATE, "alb_worklist_add: call alb_sell_build first");
    if (!(alpha > 0) || !(beta > 0)) return fail(ALB_ERR_INVALID, "alb_worklist_add: alpha, beta > 0");
    for (int i = 0; i < nroots; i++)
        if (roots[i] < 0 || roots[i] >= g->n)
            return fail(ALB_ERR_INVALID, "alb_worklist_add: root %d outside the graph", roots[i]);
    try {
        w->entries.push_back({g, std::vector<int32_t>(roots, roots + nroots), alpha, beta});
    } catch (const std::bad_alloc &) {
        return fail(ALB_ERR_OOM, "alb_worklist_add: host allocation failed");
    }
    w->total_out += g->n * (int64_t)nroots;
    return ALB_OK;
}

alb_status alb_worklist_size(const alb_worklist *w, int64_t *level_entries, int32_t *items) {
    if (!w) return fail(ALB_ERR_INVALID, "alb_worklist_size: worklist is NULL");
    int32_t k = 0;
    for (auto &e : w->entries) k += (int32_t)e.roots.size();
    if (level_entries) *level_entries = w->total_out;
    if (items) *items = k;
    return ALB_OK;
}

alb_status alb_worklist_run_device(alb_worklist *w, int32_t block, int32_t *d_levels,
                                   alb_stats *st) {
    if (!w || w->entries.empty() || !d_levels)
        return fail(ALB_ERR_INVALID, "alb_worklist_run: empty worklist or no output");
    if (!(block == 128 || block == 256 || block == 512 || block == 1024))
        return fail(ALB_ERR_UNSUPPORTED, "alb_worklist_run: block must be 128, 256, 512 or 1024");
    alb_graph *g0 = w->entries[0].g;
    ALB_CK(cudaSetDevice(g0->device));
    int max_smem = 0;
    ALB_CK(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, g0->device));
    // a graph fits the kernel when its three bitmaps and 1 KB of other
    // shared state fit in one CTA
    auto fits = [&](const Sell &s) {
        return sizeof(uint32_t) * 3 * (size_t)s.nwords + 1024 <= (size_t)max_smem;
    };
    std::vector<WlGraph> hg;
    std::vector<WlItem> hi;
    std::vector<int64_t> cost;
    int64_t nwords_max = 0, off = 0;
    float big_ms = 0.f;
    int64_t big_kernels = 0;
    for (size_t gi = 0; gi < w->entries.size(); gi++) {
        const auto &e = w->entries[gi];
        const Sell &s = e.g->sell;
        if (!s.built) return fail(ALB_ERR_STATE, "alb_worklist_run: a graph lost its SELL build");
        if (!fits(s)) {
            // too large for one CTA's shared memory: the single-root path
            alb_bfs_opts o;
            alb_bfs_opts_default(&o);
            o.policy = ALB_POLICY_BEAMER;
            o.loop = ALB_LOOP_GRAPH;
            o.alpha = e.alpha;
            o.beta = e.beta;
            for (int32_t r : e.roots) {
                alb_stats bs;
                ALB_TRY(alb_bfs_device(e.g, r, &o, d_levels + off, nullptr, &bs));
                big_ms += bs.ms;
                big_kernels += bs.kernels;
                off += e.g->n;
            }
            continue;
        }
        WlGraph d;
        std::memset(&d, 0, sizeof(d));
        d.n = e.g->n;
        d.nwords = s.nwords;
        d.C = s.C;
        d.log2C = s.log2C;
        d.perm = s.perm;
        d.inv = s.inv;
        d.ideg = s.ideg;
        d.odeg = s.odeg;
        d.width = s.width;
        d.slice_off = s.slice_off;
        d.col4 = (const int4 *)s.col;
        d.prow = s.prow;
        d.pcol = s.pcol;
        d.nlong = s.nlong;
        d.lrow = s.lrow;
        d.lptr = s.lptr;
        d.lcol = s.lcol;
        d.vinit = s.vinit;
        d.m_in = s.m_in;
        d.alpha = e.alpha;
        d.beta = e.beta;
        hg.push_back(d);
        nwords_max = std::max(nwords_max, s.nwords);
        // the kernel's graph index is the position in hg
        for (int32_t r : e.roots) {
            hi.push_back({(int32_t)hg.size() - 1, r, off});
            cost.push_back(e.g->nnz_in);
            off += e.g->n;
        }
    }
    if (hi.empty()) {  // every graph took the single-root path
        if (st) {
            std::memset(st, 0, sizeof(*st));
            st->ms = big_ms;
            st->kernels = big_kernels;
        }
        return ALB_OK;
    }
    const size_t smem = sizeof(uint32_t) * 3 * (size_t)nwords_max;
    // longest items first
    std::vector<int32_t> order(hi.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return cost[a] > cost[b]; });
    std::vector<WlItem> sorted(hi.size());
    for (size_t i = 0; i < order.size(); i++) sorted[i] = hi[order[i]];
    WlGraph *dg = nullptr;
    WlItem *di = nullptr;
    unsigned int *dctr = nullptr;
    auto cleanup = [&]() {
        dfree(dg);
        dfree(di);
        dfree(dctr);
    };
    alb_status rc = [&]() -> alb_status {
        ALB_TRY(dmalloc((void **)&dg, sizeof(WlGraph) * hg.size(), "worklist graphs"));
        ALB_TRY(dmalloc((void **)&di, sizeof(WlItem) * sorted.size(), "worklist items"));
        ALB_TRY(dmalloc((void **)&dctr, sizeof(unsigned int), "worklist counter"));
        cudaStream_t stream = g0->stream;
        ALB_CK(cudaMemcpyAsync(dg, hg.data(), sizeof(WlGraph) * hg.size(), cudaMemcpyHostToDevice,
                               stream));
        ALB_CK(cudaMemcpyAsync(di, sorted.data(), sizeof(WlItem) * sorted.size(),
                               cudaMemcpyHostToDevice, stream));
        ALB_CK(cudaMemsetAsync(dctr, 0, sizeof(unsigned int), stream));
        ALB_CK(cudaFuncSetAttribute(k_worklist, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
        int per_sm = 0;
        ALB_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_worklist, block, smem));
        if (per_sm < 1) return fail(ALB_ERR_UNSUPPORTED, "alb_worklist_run: kernel does not fit");
        const unsigned grid = (unsigned)std::min<int64_t>((int64_t)per_sm * g0->num_sms,
                                                          (int64_t)sorted.size());
        ALB_CK(cudaEventRecord(g0->ev0, stream));
        k_worklist<<<grid, block, smem, stream>>>(dg, di, (int32_t)sorted.size(), dctr, d_levels);
        ALB_CK(cudaGetLastError());
        ALB_CK(cudaEventRecord(g0->ev1, stream));
        ALB_CK(cudaStreamSynchronize(stream));
        float ms = 0;
        ALB_CK(cudaEventElapsedTime(&ms, g0->ev0, g0->ev1));
        if (st) {
            std::memset(st, 0, sizeof(*st));
            st->ms = ms + big_ms;
            st->kernels = 1 + big_kernels;
        }
        return ALB_OK;
    }();
    cleanup();
    return rc;
}

alb_status alb_worklist_run(alb_worklist *w, int32_t block, int32_t *levels, alb_stats *st) {
    if (!w || w->entries.empty() || !levels)
        return fail(ALB_ERR_INVALID, "alb_worklist_run: empty worklist or no output");
    alb_graph *g0 = w->entries[0].g;
    ALB_CK(cudaSetDevice(g0->device));
    int32_t *d = nullptr;
    ALB_TRY(dmalloc((void **)&d, sizeof(int32_t) * (size_t)w->total_out, "worklist levels"));
    alb_status rc = alb_worklist_run_device(w, block, d, st);
    if (rc == ALB_OK) {
        cudaError_t e = cudaMemcpy(levels, d, sizeof(int32_t) * (size_t)w->total_out,
                                   cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = fail(ALB_ERR_CUDA, "alb_worklist_run: %s", cudaGetErrorString(e));
    }
    dfree(d);
    return rc;
}

}  // extern "C"
