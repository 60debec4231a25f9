/*
 * CPU oracle for the ALBBA linear-algebra BFS hot path.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the albba_gb300 product links, loads or
 * calls this code; only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py do, and only as the checker (or as the timed CPU baseline).
 *
 * What it restates (reference = scalbba/albba):
 *   - BFS level sets: bfs/src/bfs_ref.h:26-67 with the level-update rule of
 *     bfs/src/utils.c:305-334 (a vertex joins level L+1 when one of its row
 *     entries is in frontier L and it is not yet visited). Restated as a queue
 *     BFS, which produces the same level sets in O(n + nnz).
 *   - Parents: the reference has no parent output. Here parent[v] is the
 *     smallest original id among v's row entries at level[v]-1 (root is its own
 *     parent); that rule makes parents unique, so the GPU path must match it
 *     bit for bit.
 *   - SELL-C-sigma row order: bfs/src/sorting_utils.c:173-253 (stable,
 *     descending sort of row lengths inside windows of sigma rows).
 *   - Slice widths / offsets: bfs/src/sparse_matrix.c:435-521 (padded SELL);
 *     the column layout here is this project's 4-interleaved slice-major form,
 *     defined in orc_sell_build below.
 *   - The reference's level loop (bfs/src/bfs_SELLCSv2.c:296-762 with the
 *     kernels of bfs/src/bfs_par_kernels.c:128-198, 566-656, 696-797), as a
 *     scalar OpenMP port, for the timed CPU baseline (refalgo.c).
 *
 * Parity pin: tests/golden/ holds per-level frontier counts produced by the
 * reference's own run_bfs_ref and SELL orders/widths produced by the
 * reference's own get_order_by_row_size_radix / convert_csr_to_sellcs,
 * compiled from the reference sources (oracle/Makefile.ref). The oracle is
 * checked against them in tests/test_oracle.py.
 */
#ifndef ALBBA_ORACLE_H
#define ALBBA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Queue BFS from root. out_* = row u lists the targets of u's edges (push
 * side); in_* = row v lists the sources of v's edges (pull side; pass the
 * same arrays for a symmetric graph). level[v] = BFS depth or -1;
 * parent[v] = min source id at depth level[v]-1, root -> root, else -1.
 * Returns the number of non-empty levels. */
int32_t orc_bfs(int64_t n, const int64_t *out_rowptr, const int32_t *out_col,
                const int64_t *in_rowptr, const int32_t *in_col, int32_t root,
                int32_t *level, int32_t *parent);

/* Per-level sizes of a level array (counts[L] for L < num_levels). */
void orc_level_counts(int64_t n, const int32_t *level, int32_t num_levels,
                      int64_t *counts);

/* Graph500-style validation plus the min-index parent rule.
 * Returns 0 when valid, otherwise a positive code naming the first failed
 * rule (see oracle.c). */
int32_t orc_validate(int64_t n, const int64_t *out_rowptr, const int32_t *out_col,
                     const int64_t *in_rowptr, const int32_t *in_col,
                     int32_t root, const int32_t *level, const int32_t *parent);

/* Stable descending sort of deg inside windows of sigma rows:
 * order[p] = original row id placed at position p. */
void orc_sell_order(int64_t n, const int32_t *deg, int32_t sigma, int32_t *order);

/* Size of the 4-interleaved SELL column array (int32 entries) for slice
 * height C, given the row order. Rows longer than long_row (when > 0) are
 * stored empty in the SELL and kept in a separate long-row list. */
int64_t orc_sell_size(int64_t n, const int64_t *rowptr, const int32_t *order,
                      int32_t C, int32_t long_row);

/* Build the SELL-C-sigma layout used by the GPU path (position space):
 *   perm[p]  = order[p], inv[perm[p]] = p
 *   a row is long when long_row > 0 and its length exceeds long_row; long
 *   rows have no SELL entries (length 0 below)
 *   width[s] = max (non-long) row length in slice s, w4 = width rounded up to 4
 *   slice_off[s] = sum over t < s of C * w4[t]          (int64, nslices+1)
 *   col[slice_off[s] + (k/4)*4*C + r*4 + k%4] = inv[adj(perm[s*C+r])[k]]
 *       for k < deg; k in [deg, w4) holds the row's own position s*C+r;
 *       rows past n hold 0.
 * col must hold orc_sell_size(...) entries. */
void orc_sell_build(int64_t n, const int64_t *rowptr, const int32_t *adj,
                    const int32_t *order, int32_t C, int32_t long_row, int32_t *inv,
                    int32_t *width, int64_t *slice_off, int32_t *col);

/* Long-row list of the same layout: lrow[i] = positions of long rows in
 * ascending order, lptr (nlong+1) offsets, lcol = their entries relabelled to
 * positions, in row order. Returns nlong; call with lrow == NULL for the
 * count and lcol == NULL to skip the entries. */
int64_t orc_sell_long(int64_t n, const int64_t *rowptr, const int32_t *adj,
                      const int32_t *order, int32_t long_row, int32_t *lrow,
                      int64_t *lptr, int32_t *lcol);

/* y = A x in fp64 as the reference's SELL-C-sigma SpMV computes it
 * (kernel_SELLCS_DFC, bfs/src/bfs_par_kernels.c:8-53): row r accumulates
 * values * x[col] over its entries in CSR order with one fused multiply-add
 * each (_vel_vfmadd_vvvvl), starting from 0; the SELL layout only changes
 * which lane does the row, not the order of its operations. */
void orc_spmv(int64_t n, const int64_t *rowptr, const int32_t *col, const double *val,
              const double *x, double *y);

/* Timed CPU port of the reference's level loop (C = 256 SELL with active-lane
 * ("DFC") layout, pull kernel above 4% of n frontier, sparse-x kernel below),
 * for a symmetric graph. Root is relabelled by the caller-independent rule of
 * the reference (it always starts at row 0) by running on the graph with
 * vertex 0 and root swapped. Writes per-level frontier sizes into counts
 * (capacity n) and returns the number of levels; *bfs_ms = level-loop time,
 * *conv_ms = SELL build time. ntasks <= 0 selects one task per thread. */
int32_t orc_refalgo_bfs(int64_t n, const int64_t *rowptr, const int32_t *col,
                        int32_t root, int32_t sigma, int32_t ntasks,
                        int64_t *counts, double *bfs_ms, double *conv_ms);

/* The same port split into build (once) and traversal (per root). */
void *orc_refalgo_prepare(int64_t n, const int64_t *rowptr, const int32_t *col,
                          int32_t sigma, int32_t ntasks, double *conv_ms);
int32_t orc_refalgo_run(void *h, int32_t root, int64_t *counts, double *bfs_ms);
void orc_refalgo_free(void *h);

/* CPU MLP (8 -> 32 -> 32 -> 3, ReLU) used to check the GPU selector kernels.
 * Parameter block layout (fp32, 1,443 values):
 *   W1[32][8], b1[32], W2[32][32], b2[32], W3[3][32], b3[3]. */
#define ORC_MLP_NPARAM 1443
void orc_mlp_forward(const float *params, int32_t batch, const float *x,
                     float *out);
/* Loss = mean over batch of sum_k mask[b][k] * (out[b][k] - y[b][k])^2.
 * grad receives d loss / d params. Returns the loss. */
float orc_mlp_loss_grad(const float *params, int32_t batch, const float *x,
                        const float *y, const float *mask, float *grad);
/* One Adam step (Kingma & Ba 2015) over the parameter block. */
void orc_adam_step(float *params, const float *grad, float *m, float *v,
                   int32_t t, float lr, float beta1, float beta2, float eps);

#ifdef __cplusplus
}
#endif
#endif
