/*
 * CPU oracle for the ALBBA BFS hot path -- test infrastructure only.
 * See oracle.h for what each function restates and where in the reference.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* BFS levels + min-index parents                                            */
/* ------------------------------------------------------------------------ */

/* Level sets follow bfs/src/bfs_ref.h:50-62 + bfs/src/utils.c:313-330: a
 * vertex enters level L+1 exactly when it is unvisited and one of its sources
 * is in level L. A FIFO queue visits the same sets level by level. */
int32_t orc_bfs(int64_t n, const int64_t *out_rowptr, const int32_t *out_col,
                const int64_t *in_rowptr, const int32_t *in_col, int32_t root,
                int32_t *level, int32_t *parent)
{
    for (int64_t v = 0; v < n; v++) {
        level[v] = -1;
        parent[v] = -1;
    }
    if (n <= 0 || root < 0 || root >= n)
        return 0;
    int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int64_t head = 0, tail = 0;
    level[root] = 0;
    queue[tail++] = root;
    int32_t max_level = 0;
    while (head < tail) {
        int32_t u = queue[head++];
        int32_t lu = level[u];
        for (int64_t e = out_rowptr[u]; e < out_rowptr[u + 1]; e++) {
            int32_t v = out_col[e];
            if (level[v] < 0) {
                level[v] = lu + 1;
                if (lu + 1 > max_level)
                    max_level = lu + 1;
                queue[tail++] = v;
            }
        }
    }
    free(queue);
    /* parent[v] = min source at level[v]-1 (unique by construction). */
    for (int64_t v = 0; v < n; v++) {
        if (level[v] <= 0)
            continue;
        int32_t best = -1;
        for (int64_t e = in_rowptr[v]; e < in_rowptr[v + 1]; e++) {
            int32_t u = in_col[e];
            if (level[u] == level[v] - 1 && (best < 0 || u < best))
                best = u;
        }
        parent[v] = best;
    }
    parent[root] = root;
    return max_level + 1;
}

void orc_level_counts(int64_t n, const int32_t *level, int32_t num_levels,
                      int64_t *counts)
{
    for (int32_t l = 0; l < num_levels; l++)
        counts[l] = 0;
    for (int64_t v = 0; v < n; v++)
        if (level[v] >= 0 && level[v] < num_levels)
            counts[level[v]]++;
}

/* Return codes:
 *  1 root level/parent wrong      2 reached vertex with bad parent id
 *  3 parent not one level up      4 parent is not a source of v
 *  5 parent is not the min source 6 edge spans more than one level
 *  7 edge from reached to unreached 8 unreached vertex with level/parent set */
int32_t orc_validate(int64_t n, const int64_t *out_rowptr, const int32_t *out_col,
                     const int64_t *in_rowptr, const int32_t *in_col,
                     int32_t root, const int32_t *level, const int32_t *parent)
{
    if (level[root] != 0 || parent[root] != root)
        return 1;
    for (int64_t v = 0; v < n; v++) {
        if (level[v] < 0) {
            if (level[v] != -1 || parent[v] != -1)
                return 8;
            continue;
        }
        if (v == root)
            continue;
        int32_t p = parent[v];
        if (p < 0 || p >= n || level[p] < 0)
            return 2;
        if (level[p] != level[v] - 1)
            return 3;
        int found = 0;
        int32_t best = -1;
        for (int64_t e = in_rowptr[v]; e < in_rowptr[v + 1]; e++) {
            int32_t u = in_col[e];
            if (u == p)
                found = 1;
            if (level[u] == level[v] - 1 && (best < 0 || u < best))
                best = u;
        }
        if (!found)
            return 4;
        if (best != p)
            return 5;
    }
    for (int64_t u = 0; u < n; u++) {
        if (level[u] < 0)
            continue;
        for (int64_t e = out_rowptr[u]; e < out_rowptr[u + 1]; e++) {
            int32_t v = out_col[e];
            if (level[v] < 0)
                return 7;
            if (level[v] > level[u] + 1)
                return 6;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* SELL-C-sigma                                                              */
/* ------------------------------------------------------------------------ */

typedef struct {
    int32_t deg;
    int32_t id;
} deg_id;

static int cmp_deg_desc_id_asc(const void *a, const void *b)
{
    const deg_id *x = (const deg_id *)a, *y = (const deg_id *)b;
    if (x->deg != y->deg)
        return x->deg > y->deg ? -1 : 1;
    return x->id < y->id ? -1 : (x->id > y->id);
}

/* sorting_utils.c:232-253 sorts rows_size paired with identity ids inside
 * each sigma window by an LSD radix sort whose passes are stable
 * (sorting_utils.c:192-199 writes bin b at len - bins[b] and decrements, so
 * equal digits keep their input order) and descending. A stable descending
 * sort equals the total order (deg descending, id ascending). */
void orc_sell_order(int64_t n, const int32_t *deg, int32_t sigma, int32_t *order)
{
    if (sigma < 1)
        sigma = 1;
    deg_id *tmp = (deg_id *)malloc(sizeof(deg_id) * (size_t)(sigma));
    for (int64_t k = 0; k < n; k += sigma) {
        int64_t end = k + sigma < n ? k + sigma : n;
        int64_t len = end - k;
        for (int64_t i = 0; i < len; i++) {
            tmp[i].deg = deg[k + i];
            tmp[i].id = (int32_t)(k + i);
        }
        qsort(tmp, (size_t)len, sizeof(deg_id), cmp_deg_desc_id_asc);
        for (int64_t i = 0; i < len; i++)
            order[k + i] = tmp[i].id;
    }
    free(tmp);
}

static int32_t row_len(const int64_t *rowptr, int32_t r)
{
    return (int32_t)(rowptr[r + 1] - rowptr[r]);
}

static int32_t sell_len(const int64_t *rowptr, int32_t r, int32_t long_row)
{
    int32_t d = row_len(rowptr, r);
    return (long_row > 0 && d > long_row) ? 0 : d;
}

int64_t orc_sell_size(int64_t n, const int64_t *rowptr, const int32_t *order,
                      int32_t C, int32_t long_row)
{
    int64_t nslices = (n + C - 1) / C, total = 0;
    for (int64_t s = 0; s < nslices; s++) {
        int32_t w = 0;
        for (int64_t r = 0; r < C && s * C + r < n; r++) {
            int32_t d = sell_len(rowptr, order[s * C + r], long_row);
            if (d > w)
                w = d;
        }
        total += (int64_t)C * ((w + 3) & ~3);
    }
    return total;
}

void orc_sell_build(int64_t n, const int64_t *rowptr, const int32_t *adj,
                    const int32_t *order, int32_t C, int32_t long_row, int32_t *inv,
                    int32_t *width, int64_t *slice_off, int32_t *col)
{
    int64_t nslices = (n + C - 1) / C;
    for (int64_t p = 0; p < n; p++)
        inv[order[p]] = (int32_t)p;
    int64_t off = 0;
    for (int64_t s = 0; s < nslices; s++) {
        int32_t w = 0;
        for (int64_t r = 0; r < C && s * C + r < n; r++) {
            int32_t d = sell_len(rowptr, order[s * C + r], long_row);
            if (d > w)
                w = d;
        }
        int32_t w4 = (w + 3) & ~3;
        width[s] = w;
        slice_off[s] = off;
        for (int64_t r = 0; r < C; r++) {
            int64_t p = s * C + r;
            int32_t d = p < n ? sell_len(rowptr, order[p], long_row) : 0;
            const int32_t *row = p < n ? adj + rowptr[order[p]] : 0;
            for (int32_t k = 0; k < w4; k++) {
                int64_t at = off + (int64_t)(k / 4) * 4 * C + r * 4 + (k % 4);
                if (p >= n)
                    col[at] = 0;
                else if (k < d)
                    col[at] = inv[row[k]];
                else
                    col[at] = (int32_t)p;
            }
        }
        off += (int64_t)C * w4;
    }
    slice_off[nslices] = off;
}

int64_t orc_sell_long(int64_t n, const int64_t *rowptr, const int32_t *adj,
                      const int32_t *order, int32_t long_row, int32_t *lrow,
                      int64_t *lptr, int32_t *lcol)
{
    int32_t *inv = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t p = 0; p < n; p++)
        inv[order[p]] = (int32_t)p;
    int64_t k = 0, at = 0;
    for (int64_t p = 0; p < n; p++) {
        int32_t d = row_len(rowptr, order[p]);
        if (!(long_row > 0 && d > long_row))
            continue;
        if (lrow) {
            lrow[k] = (int32_t)p;
            lptr[k] = at;
            if (lcol)
                for (int32_t j = 0; j < d; j++)
                    lcol[at + j] = inv[adj[rowptr[order[p]] + j]];
        }
        at += d;
        k++;
    }
    if (lrow)
        lptr[k] = at;
    free(inv);
    return k;
}

/* ------------------------------------------------------------------------ */
/* MLP 8 -> 32 -> 32 -> 3 (ReLU) for checking the GPU selector kernels       */
/* ------------------------------------------------------------------------ */

#define IN 8
#define H 32
#define OUT 3
#define OFF_W1 0
#define OFF_B1 (OFF_W1 + H * IN)
#define OFF_W2 (OFF_B1 + H)
#define OFF_B2 (OFF_W2 + H * H)
#define OFF_W3 (OFF_B2 + H)
#define OFF_B3 (OFF_W3 + OUT * H)

static void mlp_one(const float *P, const float *x, float *h1, float *h2,
                    float *o)
{
    for (int j = 0; j < H; j++) {
        float a = P[OFF_B1 + j];
        for (int i = 0; i < IN; i++)
            a += P[OFF_W1 + j * IN + i] * x[i];
        h1[j] = a > 0.f ? a : 0.f;
    }
    for (int j = 0; j < H; j++) {
        float a = P[OFF_B2 + j];
        for (int i = 0; i < H; i++)
            a += P[OFF_W2 + j * H + i] * h1[i];
        h2[j] = a > 0.f ? a : 0.f;
    }
    for (int k = 0; k < OUT; k++) {
        float a = P[OFF_B3 + k];
        for (int i = 0; i < H; i++)
            a += P[OFF_W3 + k * H + i] * h2[i];
        o[k] = a;
    }
}

void orc_mlp_forward(const float *params, int32_t batch, const float *x,
                     float *out)
{
    float h1[H], h2[H];
    for (int32_t b = 0; b < batch; b++)
        mlp_one(params, x + b * IN, h1, h2, out + b * OUT);
}

float orc_mlp_loss_grad(const float *params, int32_t batch, const float *x,
                        const float *y, const float *mask, float *grad)
{
    memset(grad, 0, sizeof(float) * ORC_MLP_NPARAM);
    double loss = 0.0;
    float h1[H], h2[H], o[OUT], d3[OUT], d2[H], d1[H];
    const float *P = params;
    float inv_b = batch > 0 ? 1.0f / (float)batch : 0.f;
    for (int32_t b = 0; b < batch; b++) {
        const float *xb = x + b * IN;
        mlp_one(P, xb, h1, h2, o);
        for (int k = 0; k < OUT; k++) {
            float diff = o[k] - y[b * OUT + k];
            float m = mask[b * OUT + k];
            loss += (double)(m * diff * diff);
            d3[k] = 2.f * m * diff * inv_b;
        }
        for (int k = 0; k < OUT; k++) {
            grad[OFF_B3 + k] += d3[k];
            for (int i = 0; i < H; i++)
                grad[OFF_W3 + k * H + i] += d3[k] * h2[i];
        }
        for (int i = 0; i < H; i++) {
            float a = 0.f;
            for (int k = 0; k < OUT; k++)
                a += P[OFF_W3 + k * H + i] * d3[k];
            d2[i] = h2[i] > 0.f ? a : 0.f;
        }
        for (int j = 0; j < H; j++) {
            grad[OFF_B2 + j] += d2[j];
            for (int i = 0; i < H; i++)
                grad[OFF_W2 + j * H + i] += d2[j] * h1[i];
        }
        for (int i = 0; i < H; i++) {
            float a = 0.f;
            for (int j = 0; j < H; j++)
                a += P[OFF_W2 + j * H + i] * d2[j];
            d1[i] = h1[i] > 0.f ? a : 0.f;
        }
        for (int j = 0; j < H; j++) {
            grad[OFF_B1 + j] += d1[j];
            for (int i = 0; i < IN; i++)
                grad[OFF_W1 + j * IN + i] += d1[j] * xb[i];
        }
    }
    return (float)(loss * inv_b);
}

void orc_adam_step(float *params, const float *grad, float *m, float *v,
                   int32_t t, float lr, float beta1, float beta2, float eps)
{
    float c1 = 1.f - powf(beta1, (float)t);
    float c2 = 1.f - powf(beta2, (float)t);
    for (int i = 0; i < ORC_MLP_NPARAM; i++) {
        m[i] = beta1 * m[i] + (1.f - beta1) * grad[i];
        v[i] = beta2 * v[i] + (1.f - beta2) * grad[i] * grad[i];
        float mh = m[i] / c1, vh = v[i] / c2;
        params[i] -= lr * mh / (sqrtf(vh) + eps);
    }
}

/* kernel_SELLCS_DFC (bfs/src/bfs_par_kernels.c:8-53), row by row: entry k of
 * row r sits in column op k of r's slice lane, so the lane's accumulator sees
 * the row's entries in CSR order. */
void orc_spmv(int64_t n, const int64_t *rowptr, const int32_t *col, const double *val,
              const double *x, double *y)
{
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < n; r++) {
        double acc = 0.0;
        for (int64_t e = rowptr[r]; e < rowptr[r + 1]; e++)
            acc = fma(val[e], x[col[e]], acc);
        y[r] = acc;
    }
}
