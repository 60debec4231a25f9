/*
 * Timed CPU port of the reference's BFS level loop -- test infrastructure and
 * CPU baseline only (never part of the albba_gb300 product).
 *
 * Restated from scalbba/albba:
 *   SELL build      bfs/src/bfs_SELLCSv2.c:34-59 (C = 256, sigma window),
 *                   bfs/src/sorting_utils.c:232-253 (stable descending sort),
 *                   bfs/src/sparse_matrix.c:523-623 + bfs/src/utils.c:198-241
 *                   (active-lane column ops, per-op min/max column)
 *   task split      bfs/src/bfs_SELLCSv2.c:61-85 (nnz-balanced slice ranges)
 *   level loop      bfs/src/bfs_SELLCSv2.c:296-762
 *   pull kernel     bfs/src/bfs_par_kernels.c:128-198
 *   sparse-x kernel bfs/src/bfs_par_kernels.c:566-656
 *   converters      bfs/src/bfs_par_kernels.c:696-797
 *
 * Deliberate differences, each noted where it happens:
 *   - the root is any vertex (the reference always starts at row 0, which is
 *     the same as running it on a graph with 0 and root swapped);
 *   - the dense->sparse compaction scans the whole original-id range with
 *     its own offsets, so no frontier vertex is lost (the reference writes
 *     per-task id ranges at per-task counts taken in sorted-slice space,
 *     bfs/src/bfs_SELLCSv2.c:487-499, which can overwrite entries);
 *   - slice min columns start at n (the reference memsets bytes,
 *     bfs/src/bfs_SELLCSv2.c:173);
 *   - the task count is a parameter (the reference forces 8,
 *     bfs/src/bfs_SELLCSv2.c:214); the 50x warm-up SpMV is not run.
 */
#include "oracle.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RC 256 /* slice height of the reference (bfs_SELLCSv2.c:162) */

typedef struct {
    int64_t n;
    int64_t nslices;
    int32_t *row_order;    /* position -> original id */
    int32_t *width;        /* column ops per slice */
    int64_t *op_ptr;       /* first op of slice, nslices+1 */
    uint8_t *op_len;       /* active lanes - 1 per op */
    int64_t *slice_ptr;    /* first entry of slice, nslices+1 */
    int32_t *col;          /* entries, op-major inside a slice */
    int32_t *op_min, *op_max;
    int32_t *slice_min, *slice_max;
} rsell;

static double now_ms(void)
{
    struct timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec * 1000.0 + tv.tv_usec / 1000.0;
}

static void rsell_build(rsell *m, int64_t n, const int64_t *rowptr,
                        const int32_t *col, int32_t sigma)
{
    m->n = n;
    m->nslices = (n + RC - 1) / RC;
    int32_t *deg = (int32_t *)malloc(sizeof(int32_t) * n);
    for (int64_t i = 0; i < n; i++)
        deg[i] = (int32_t)(rowptr[i + 1] - rowptr[i]);
    m->row_order = (int32_t *)malloc(sizeof(int32_t) * n);
    orc_sell_order(n, deg, sigma, m->row_order);
    int32_t *sdeg = (int32_t *)malloc(sizeof(int32_t) * n);
    for (int64_t p = 0; p < n; p++)
        sdeg[p] = deg[m->row_order[p]];
    free(deg);
    int64_t S = m->nslices;
    m->width = (int32_t *)malloc(sizeof(int32_t) * S);
    m->op_ptr = (int64_t *)malloc(sizeof(int64_t) * (S + 1));
    m->slice_ptr = (int64_t *)malloc(sizeof(int64_t) * (S + 1));
    int64_t nops = 0;
    for (int64_t s = 0; s < S; s++) {
        m->width[s] = sdeg[s * RC]; /* first row is the longest (descending) */
        m->op_ptr[s] = nops;
        nops += m->width[s];
    }
    m->op_ptr[S] = nops;
    m->op_len = (uint8_t *)malloc(nops > 0 ? nops : 1);
    /* utils.c:198-241: op k of a slice is active on the rows longer than k */
    int64_t total = 0;
    for (int64_t s = 0; s < S; s++) {
        int64_t base = s * RC;
        int32_t rows = (int32_t)((base + RC <= n) ? RC : n - base);
        m->slice_ptr[s] = total;
        int32_t r = rows;
        for (int32_t k = 0; k < m->width[s]; k++) {
            while (r > 0 && sdeg[base + r - 1] <= k)
                r--;
            m->op_len[m->op_ptr[s] + k] = (uint8_t)(r - 1);
            total += r;
        }
    }
    m->slice_ptr[S] = total;
    m->col = (int32_t *)malloc(sizeof(int32_t) * (total > 0 ? total : 1));
    m->op_min = (int32_t *)malloc(sizeof(int32_t) * (nops > 0 ? nops : 1));
    m->op_max = (int32_t *)malloc(sizeof(int32_t) * (nops > 0 ? nops : 1));
    m->slice_min = (int32_t *)malloc(sizeof(int32_t) * S);
    m->slice_max = (int32_t *)malloc(sizeof(int32_t) * S);
#pragma omp parallel for schedule(dynamic, 32)
    for (int64_t s = 0; s < S; s++) {
        int64_t at = m->slice_ptr[s];
        int32_t smin = (int32_t)n, smax = 0;
        for (int32_t k = 0; k < m->width[s]; k++) {
            int64_t op = m->op_ptr[s] + k;
            int32_t lanes = m->op_len[op] + 1;
            int32_t mn = (int32_t)n, mx = 0;
            for (int32_t r = 0; r < lanes; r++) {
                int32_t c = col[rowptr[m->row_order[s * RC + r]] + k];
                m->col[at++] = c;
                if (c < mn)
                    mn = c;
                if (c > mx)
                    mx = c;
            }
            m->op_min[op] = mn;
            m->op_max[op] = mx;
            if (mn < smin)
                smin = mn;
            if (mx > smax)
                smax = mx;
        }
        m->slice_min[s] = smin;
        m->slice_max[s] = smax;
    }
    free(sdeg);
}

static void rsell_free(rsell *m)
{
    free(m->row_order);
    free(m->width);
    free(m->op_ptr);
    free(m->op_len);
    free(m->slice_ptr);
    free(m->col);
    free(m->op_min);
    free(m->op_max);
    free(m->slice_min);
    free(m->slice_max);
}

static inline int vis_get(const uint64_t *mask, int64_t pos)
{
    return (int)((mask[pos >> 6] >> (63 - (pos & 63))) & 1);
}
static inline void vis_set(uint64_t *mask, int64_t pos)
{
    mask[pos >> 6] |= 1ULL << (63 - (pos & 63));
}

static int32_t slice_visited(const uint64_t *mask, int64_t s, int32_t lanes)
{
    int32_t c = 0;
    for (int32_t r = 0; r < lanes; r++)
        c += vis_get(mask, s * RC + r);
    return c;
}

/* bfs_par_kernels.c:128-198 restated lane by lane */
static int64_t pull_kernel(const rsell *m, const int32_t *mask_x, int32_t *mask_y,
                           int64_t s0, int64_t s1, uint64_t *mask)
{
    int64_t cnt = 0;
    int32_t tmp[RC];
    for (int64_t s = s0; s < s1; s++) {
        int64_t base = s * RC;
        int32_t lanes = (int32_t)((base + RC > m->n) ? m->n - base : RC);
        if (slice_visited(mask, s, lanes) == lanes)
            continue; /* slice bypass */
        memset(tmp, 0, sizeof(tmp));
        int64_t at = m->slice_ptr[s];
        for (int32_t k = 0; k < m->width[s]; k++) {
            int32_t act = m->op_len[m->op_ptr[s] + k] + 1;
            for (int32_t r = 0; r < act; r++)
                tmp[r] |= mask_x[m->col[at + r]];
            at += act;
        }
        for (int32_t r = 0; r < lanes; r++) {
            if (tmp[r] > 0 && !vis_get(mask, base + r)) {
                vis_set(mask, base + r);
                mask_y[m->row_order[base + r]] = tmp[r];
                cnt++;
            }
        }
    }
    return cnt;
}

/* bfs_par_kernels.c:566-656 restated lane by lane */
static int64_t sparse_kernel(const rsell *m, const int32_t *bucket,
                             const int32_t *colidx_x, int32_t x_max, int32_t x_min,
                             int32_t *colidx_y, int64_t s0, int64_t s1,
                             uint64_t *mask)
{
    int64_t cnt = 0;
    uint8_t hit[RC];
    for (int64_t s = s0; s < s1; s++) {
        if (m->slice_max[s] < x_min || m->slice_min[s] > x_max)
            continue; /* slice range bypass */
        int64_t base = s * RC;
        int32_t lanes = (int32_t)((base + RC > m->n) ? m->n - base : RC);
        if (slice_visited(mask, s, lanes) == lanes)
            continue;
        memset(hit, 0, sizeof(hit));
        int64_t at = m->slice_ptr[s];
        for (int32_t k = 0; k < m->width[s]; k++) {
            int64_t op = m->op_ptr[s] + k;
            int32_t act = m->op_len[op] + 1;
            if (!(m->op_max[op] < x_min || m->op_min[op] > x_max)) {
                for (int32_t r = 0; r < act; r++) {
                    int32_t c = m->col[at + r];
                    if (colidx_x[bucket[c]] == c)
                        hit[r] = 1;
                }
            }
            at += act;
        }
        for (int32_t r = 0; r < lanes; r++) {
            if (hit[r] && !vis_get(mask, base + r)) {
                vis_set(mask, base + r);
                colidx_y[(s0 << 8) + cnt] = m->row_order[base + r];
                cnt++;
            }
        }
    }
    return cnt;
}

typedef struct {
    rsell m;
    int32_t T;
    int64_t *task;
    int32_t *inv;
    double conv_ms;
} refalgo;

void *orc_refalgo_prepare(int64_t n, const int64_t *rowptr, const int32_t *col, int32_t sigma,
                          int32_t ntasks, double *conv_ms)
{
    refalgo *h = (refalgo *)calloc(1, sizeof(refalgo));
    double t0 = now_ms();
    rsell_build(&h->m, n, rowptr, col, sigma);
    h->conv_ms = now_ms() - t0;
    if (conv_ms)
        *conv_ms = h->conv_ms;
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = omp_get_max_threads();
#endif
    int32_t T = ntasks > 0 ? ntasks : nthreads;
    h->T = T;
    /* bfs_SELLCSv2.c:61-85: nnz-balanced slice ranges */
    h->task = (int64_t *)malloc(sizeof(int64_t) * (T + 1));
    int64_t total = h->m.slice_ptr[h->m.nslices];
    int64_t per = (total + T - 1) / T;
    int64_t acc = 0;
    int32_t ti = 0;
    h->task[ti++] = 0;
    for (int64_t s = 0; s < h->m.nslices; s++) {
        if (acc >= per && ti < T) {
            h->task[ti++] = s;
            acc = 0;
        }
        acc += h->m.slice_ptr[s + 1] - h->m.slice_ptr[s];
    }
    for (int32_t i = ti; i <= T; i++)
        h->task[i] = h->m.nslices;
    h->inv = (int32_t *)malloc(sizeof(int32_t) * n);
    for (int64_t p = 0; p < n; p++)
        h->inv[h->m.row_order[p]] = (int32_t)p;
    return h;
}

void orc_refalgo_free(void *handle)
{
    refalgo *h = (refalgo *)handle;
    if (!h)
        return;
    rsell_free(&h->m);
    free(h->task);
    free(h->inv);
    free(h);
}

int32_t orc_refalgo_run(void *handle, int32_t root, int64_t *counts, double *bfs_ms)
{
    refalgo *h = (refalgo *)handle;
    const rsell *mp = &h->m;
    const int64_t n = mp->n;
    const int32_t T = h->T;
    const int64_t *task = h->task;
    int32_t *mask_x = (int32_t *)calloc(n, sizeof(int32_t));
    int32_t *mask_y = (int32_t *)calloc(n, sizeof(int32_t));
    int32_t *colidx_x = (int32_t *)calloc(n, sizeof(int32_t));
    int32_t *colidx_y = (int32_t *)calloc((size_t)(mp->nslices * RC), sizeof(int32_t));
    int32_t *bucket = (int32_t *)calloc(n + 1, sizeof(int32_t));
    uint64_t *mask = (uint64_t *)calloc(n / 64 + 8, sizeof(uint64_t));
    int64_t *tcnt = (int64_t *)calloc(T + 1, sizeof(int64_t));

    mask_x[root] = 1;
    colidx_x[0] = root;
    vis_set(mask, h->inv[root]);
    int64_t nnzx = 1;
    const int64_t thr = (int64_t)(n * 0.04); /* bfs_SELLCSv2.c:283-284 */
    int32_t iters = 0;

    double ts = now_ms();
    do {
        int32_t x_max = 0, x_min = (int32_t)n;
        if (nnzx <= thr) {
            for (int64_t i = 0; i < nnzx; i++) {
                if (colidx_x[i] > x_max)
                    x_max = colidx_x[i];
                if (colidx_x[i] < x_min)
                    x_min = colidx_x[i];
            }
#pragma omp parallel for
            for (int64_t i = 0; i < nnzx; i++)
                bucket[colidx_x[i]] = (int32_t)i;
        }
        const int dense = nnzx > thr;
#pragma omp parallel for schedule(dynamic, 1)
        for (int32_t t = 0; t < T; t++) {
            if (task[t] >= mp->nslices) {
                tcnt[t] = 0;
                continue;
            }
            if (dense)
                tcnt[t] = pull_kernel(mp, mask_x, mask_y, task[t], task[t + 1], mask);
            else
                tcnt[t] = sparse_kernel(mp, bucket, colidx_x, x_max, x_min, colidx_y,
                                        task[t], task[t + 1], mask);
        }
        counts[iters] = nnzx;
        int64_t nnzy = 0;
        for (int32_t t = 0; t < T; t++)
            nnzy += tcnt[t];
        if (dense) {
            if (nnzy > thr) {
#pragma omp parallel for
                for (int64_t i = 0; i < n; i++)
                    mask_x[i] = mask_y[i];
            } else {
                /* dense -> sparse: one pass over the whole id range */
                int64_t k = 0;
                for (int64_t i = 0; i < n; i++)
                    if (mask_y[i] > 0)
                        colidx_x[k++] = (int32_t)i;
            }
        } else {
            if (nnzy > thr) {
                for (int32_t t = 0; t < T; t++) {
                    int64_t b = task[t] << 8;
                    for (int64_t i = 0; i < tcnt[t]; i++)
                        mask_x[colidx_y[b + i]] = 1;
                }
            } else {
                int64_t k = 0;
                for (int32_t t = 0; t < T; t++) {
                    int64_t b = task[t] << 8;
                    for (int64_t i = 0; i < tcnt[t]; i++)
                        colidx_x[k++] = colidx_y[b + i];
                }
            }
        }
        nnzx = nnzy;
        if (nnzx > thr) {
#pragma omp parallel for
            for (int64_t i = 0; i < n; i++)
                mask_y[i] = 0;
        }
        iters++;
    } while (nnzx != 0);
    *bfs_ms = now_ms() - ts;

    free(mask_x);
    free(mask_y);
    free(colidx_x);
    free(colidx_y);
    free(bucket);
    free(mask);
    free(tcnt);
    return iters;
}

int32_t orc_refalgo_bfs(int64_t n, const int64_t *rowptr, const int32_t *col,
                        int32_t root, int32_t sigma, int32_t ntasks,
                        int64_t *counts, double *bfs_ms, double *conv_ms)
{
    void *h = orc_refalgo_prepare(n, rowptr, col, sigma, ntasks, conv_ms);
    int32_t nl = orc_refalgo_run(h, root, counts, bfs_ms);
    orc_refalgo_free(h);
    return nl;
}
