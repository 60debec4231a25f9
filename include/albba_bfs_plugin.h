/*
 * Drop-in BFS variant for the reference's CLI driver (scalbba/albba).
 *
 * A BFS variant of the reference is one C file linked with its driver
 * bfs/src/main.c (bfs/Makefile:35-38). This library (libbfs_gb300.so) exports
 * the same symbols as bfs/src/bfs_SELLCSv2.c, so main.c links against it
 * unchanged and runs the whole hot path on the GPU through the albba C ABI.
 *
 * The types below restate the reference's interface and must keep its
 * layout: SparseMatrixCSR is bfs/src/sparse_matrix.h:18-28, MatrixFormat is
 * bfs/src/sparse_matrix.h:8-16, elem_t is double (bfs/src/sparse_matrix.h:6).
 * When the reference headers are already included (its main.c includes
 * sparse_matrix.h before bfs.h), define ALBBA_PLUGIN_USE_REFERENCE_TYPES to
 * skip these definitions.
 */
#ifndef ALBBA_BFS_PLUGIN_H
#define ALBBA_BFS_PLUGIN_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef ALBBA_PLUGIN_USE_REFERENCE_TYPES
typedef double elem_t;

enum MatrixFormat { COO, CSR, CSC, CSRSIMD, ELLPACK, VBSF };

typedef struct SparseMatrixCSR_STRUCT {
    char *name;
    elem_t *values;
    int *column_indices;
    int *row_pointers;
    int nrows;
    int ncolumns;
    int nnz;
    int isSymmetric;
} SparseMatrixCSR;
#endif

/* Exported by the variant (bfs/src/bfs_SELLCSv2.c:26-31). sigma_window is the
 * SELL sort window (-w on the CLI); the slice height is 32. */
extern enum MatrixFormat required_matrix_format;
extern char algorithm_version[30];
extern int sigma_window;
extern int num_blocks;
extern int chunk_size;

/* Defined by the driver (bfs/src/main.c:14-22); this library carries weak
 * defaults so it also loads without the driver. */
extern size_t align_size;
extern int perf_analysis;
extern int verify;
extern int bypass_record;

/* bfs/src/bfs.h:13-24. The matrix is the driver's working matrix (row v lists
 * the sources of v's edges, bfs/src/main.c:117-126); the root is colidx_x[0]
 * (vertex 0 as set by init_bfs, bfs/src/utils.c:381-399). On return:
 * frontier[L] = size of level L (when verify is set), *num_iter = non-empty
 * levels, *num_vex = vertices reached, *bfs_time = traversal ms (device
 * events), *conv_time = SELL-C-sigma build ms, iter_times[L] = per-level ms
 * (when perf_analysis is set), *nnzx = 0. bit_flag and sort_flag are accepted
 * and ignored (the reference forces bit_flag = 1, main.c:189). On failure the
 * message goes to stderr, *num_iter = 0 and *bfs_time = -1 (the reference
 * itself exits on allocation failure, bfs/src/utils.c:102-109). */
void run_custom_bfs_test(const SparseMatrixCSR *csr_matrix, elem_t *bfs_x, int *colidx_x,
                         int *nnzx, int *frontier, int *num_vex, double *conv_time,
                         double *iter_times, double *bfs_time, int *num_iter, bool bit_flag,
                         bool sort_flag);

/* bfs/src/bfs.h:26 */
void print_additional_custom_report(char *text_padding, double *elapsed_times);

/* Levels and parents of the last run_custom_bfs_test call (n entries each,
 * original ids), NULL before the first successful call. No counterpart in the
 * reference, which returns only per-level sizes. */
const int *bfs_gb300_last_levels(void);
const int *bfs_gb300_last_parents(void);

#ifdef __cplusplus
}
#endif
#endif
