/*
 * Harness around the reference's own C sources (compiled from the reference
 * tree by oracle/Makefile.ref into oracle/_ref/libalbba_ref.so). Test
 * infrastructure only: tests/golden/make_golden.py calls it to produce the
 * golden vectors that pin the oracle.
 *
 * It supplies the globals that the reference's main.c normally defines
 * (bfs/src/main.c:14-22) and wraps:
 *   run_bfs_ref                  bfs/src/bfs_ref.h:26-67   (root is row 0)
 *   get_rows_size                bfs/src/utils.c:111-124
 *   get_order_by_row_size_radix  bfs/src/sorting_utils.c:232-253
 *   convert_csr_to_sellcs        bfs/src/sparse_matrix.c:435-521
 *   convert_csr_to_sellcs_dfc    bfs/src/sparse_matrix.c:523-623
 *   kernel_SELLCS_DFC            bfs/src/bfs_par_kernels.c:8-53 (fp64 SpMV, through
 *                                the scalar restatement in ve_scalar.c)
 *   run_custom_bfs_test          bfs/src/bfs_SELLCSv2.c:126-820 (root row 0)
 *   mmio_info, mmio_data         bfs/src/mmio_highlevel.h:11-263 (.mtx -> CSR)
 *   the undirected conversion    bfs/src/main.c:127-163 (CSR merged with its
 *                                CSC by MergeArr, utils.c:351-380), restated
 *                                here as a call sequence of the reference's
 *                                convert_csr_to_csc and MergeArr
 */
#include "common.h"
#include "sparse_matrix.h"
#include "sorting_utils.h"
#include "utils.h"
#include "bfs.h"

size_t align_size = 64;
int perf_analysis = 0;
int verify = 0;
int bypass_record = 0;

#include "bfs_ref.h"
#include "mmio_highlevel.h"

extern int sigma_window;
extern int ve_scalar_dead_calls;

static void make_csr(SparseMatrixCSR *m, int n, const int *rowptr, const int *col)
{
    int nnz = rowptr[n];
    m->name = "/golden/graph";
    m->nrows = n;
    m->ncolumns = n;
    m->nnz = nnz;
    m->isSymmetric = 1;
    m->row_pointers = (int *)malloc(sizeof(int) * (n + 1));
    memcpy(m->row_pointers, rowptr, sizeof(int) * (n + 1));
    m->column_indices = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    memcpy(m->column_indices, col, sizeof(int) * nnz);
    m->values = (elem_t *)malloc(sizeof(elem_t) * (nnz > 0 ? nnz : 1));
    for (int i = 0; i < nnz; i++)
        m->values[i] = 1.0; /* main.c:106-109 */
}

static void free_csr(SparseMatrixCSR *m)
{
    free(m->row_pointers);
    free(m->column_indices);
    free(m->values);
}

/* Per-level frontier sizes of the reference BFS from row 0. */
int refh_bfs_counts(int n, const int *rowptr, const int *col, int *counts)
{
    SparseMatrixCSR m;
    make_csr(&m, n, rowptr, col);
    elem_t *x = (elem_t *)calloc(n, sizeof(elem_t));
    int *colidx_x = (int *)calloc(n, sizeof(int));
    int *num_vex_ref = (int *)calloc(n + 1, sizeof(int));
    int nnzx = 1, iter_ref = 0, sum_vex_ref = 1;
    x[0] = 1; /* main.c:200-204 */
    colidx_x[0] = 0;
    run_bfs_ref(&m, x, colidx_x, &nnzx, &iter_ref, &sum_vex_ref, num_vex_ref);
    for (int i = 0; i < iter_ref; i++)
        counts[i] = num_vex_ref[i];
    free(x);
    free(colidx_x);
    free(num_vex_ref);
    free_csr(&m);
    return iter_ref;
}

/* Padded SELL-C-sigma. Call with padded_col == NULL to get the entry count. */
int refh_sell(int n, const int *rowptr, const int *col, int C, int sigma,
              int *order_out, int *widths_out, int *slice_ptr_out, int *padded_col)
{
    SparseMatrixCSR m;
    make_csr(&m, n, rowptr, col);
    int padded = 0;
    int *rows_size = get_rows_size(m.row_pointers, n, &padded);
    int *row_order = get_order_by_row_size_radix(rows_size, n, sigma);
    SparseMatrixSELLCS s;
    memset(&s, 0, sizeof(s));
    s.C = C;
    s.sigma = sigma;
    convert_csr_to_sellcs(&m, &s, rows_size, row_order, 0);
    int total = s.slice_pointers[s.nslices];
    if (padded_col) {
        for (int i = 0; i < n; i++)
            order_out[i] = row_order[i];
        for (int i = 0; i < s.nslices; i++)
            widths_out[i] = s.slice_widths[i];
        for (int i = 0; i <= s.nslices; i++)
            slice_ptr_out[i] = s.slice_pointers[i];
        for (int i = 0; i < total; i++)
            padded_col[i] = s.column_indices[i];
    }
    free(s.slice_widths);
    free(s.slice_widths_pointers);
    free(s.slice_pointers);
    free(s.column_indices);
    free(s.values);
    free(row_order);
    free(rows_size);
    free_csr(&m);
    return total;
}

/* Active-lane ("DFC") SELL with C = 256 as the reference's BFS builds it.
 * Call with vop_lengths_out == NULL to get the column-op count. */
int refh_sell_dfc(int n, const int *rowptr, const int *col, int sigma,
                  int *vop_lengths_out, int *slice_ptr_out)
{
    SparseMatrixCSR m;
    make_csr(&m, n, rowptr, col);
    int padded = 0;
    int *rows_size = get_rows_size(m.row_pointers, n, &padded);
    int *row_order = get_order_by_row_size_radix(rows_size, n, sigma);
    SparseMatrixSELLCS s;
    memset(&s, 0, sizeof(s));
    s.C = 256;
    s.sigma = sigma;
    convert_csr_to_sellcs_dfc(&m, &s, rows_size, row_order, 0);
    int nops = s.vop_pointers[s.nslices];
    if (vop_lengths_out) {
        for (int i = 0; i < nops; i++)
            vop_lengths_out[i] = s.vop_lengths[i];
        for (int i = 0; i <= s.nslices; i++)
            slice_ptr_out[i] = s.slice_pointers[i];
    }
    free(s.slice_widths);
    free(s.vop_pointers);
    free(s.vop_lengths);
    free(s.slice_pointers);
    free(s.max_index);
    free(s.min_index);
    free(s.column_indices);
    free(s.values);
    free(row_order);
    free(rows_size);
    free_csr(&m);
    return nops;
}

/* y = A x through the reference's fp64 SELL-C-sigma SpMV: the DFC matrix
 * (C = 256) built by convert_csr_to_sellcs_dfc from a CSR with the given
 * values, then kernel_SELLCS_DFC over all slices. */
void refh_spmv_dfc(int n, const int *rowptr, const int *col, const double *values, int sigma,
                   const double *x, double *y)
{
    SparseMatrixCSR m;
    make_csr(&m, n, rowptr, col);
    for (int i = 0; i < rowptr[n]; i++)
        m.values[i] = values[i];
    int padded = 0;
    int *rows_size = get_rows_size(m.row_pointers, n, &padded);
    int *row_order = get_order_by_row_size_radix(rows_size, n, sigma);
    SparseMatrixSELLCS s;
    memset(&s, 0, sizeof(s));
    s.C = 256;
    s.sigma = sigma;
    convert_csr_to_sellcs_dfc(&m, &s, rows_size, row_order, 0);
    s.row_order = row_order;
    kernel_SELLCS_DFC(&s, x, y, 0, s.nslices);
    free(s.slice_widths);
    free(s.vop_pointers);
    free(s.vop_lengths);
    free(s.slice_pointers);
    free(s.max_index);
    free(s.min_index);
    free(s.column_indices);
    free(s.values);
    free(row_order);
    free(rows_size);
    free_csr(&m);
}

/* The reference's own level loop from row 0 (verify on, so frontier sizes
 * are recorded). Returns num_iter; *num_vex = vertices reached. */
int refh_custom_bfs(int n, const int *rowptr, const int *col, int sigma,
                    int *frontier, int *num_vex, int *dead_calls)
{
    SparseMatrixCSR m;
    make_csr(&m, n, rowptr, col);
    elem_t *bfs_x = (elem_t *)calloc(n, sizeof(elem_t));
    int *colidx_x = (int *)calloc(n, sizeof(int));
    int *fr = (int *)calloc(n + 1, sizeof(int));
    double *iter_times = (double *)calloc(n + 1, sizeof(double));
    int nnzx = 0, num_iter = 0, nv = 0;
    double bfs_time = 0, conv_time = 0;
    /* init_bfs (utils.c:381-399) */
    nnzx = 1;
    bfs_x[0] = 1;
    colidx_x[0] = 0;
    nv = 1;
    verify = 1;
    sigma_window = sigma;
    ve_scalar_dead_calls = 0;
    run_custom_bfs_test(&m, bfs_x, colidx_x, &nnzx, fr, &nv, &conv_time, iter_times,
                        &bfs_time, &num_iter, 1, 0);
    verify = 0;
    for (int i = 0; i < num_iter; i++)
        frontier[i] = fr[i];
    *num_vex = nv;
    *dead_calls = ve_scalar_dead_calls;
    free(bfs_x);
    free(colidx_x);
    free(fr);
    free(iter_times);
    free_csr(&m);
    return num_iter;
}


/* .mtx header through the reference reader: rows, columns, CSR entry count
 * (after the symmetric mirroring), symmetric flag; nonzero on failure. */
int refh_mtx_info(const char *path, int *m, int *n, int *nnz, int *sym)
{
    return mmio_info(m, n, nnz, sym, (char *)path);
}

/* The CSR the reference reader builds (values dropped). */
int refh_mtx_data(const char *path, int m, int nnz, int *rowptr, int *col)
{
    double *val = (double *)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    int rc = mmio_data(rowptr, col, val, (char *)path);
    free(val);
    (void)m;
    return rc;
}

/* The reference driver's conversion of a non-symmetric CSR to an undirected
 * graph: row i of the result is MergeArr(row i of the CSC, row i of the
 * CSR). out_col needs 2 * nnz entries; returns the result's entry count. */
int refh_undirected(int n, const int *rowptr, const int *col, int *out_rowptr, int *out_col)
{
    SparseMatrixCSR m;
    make_csr(&m, n, rowptr, col);
    SparseMatrixCSC t;
    convert_csr_to_csc(&m, &t);
    int len = 0;
    for (int i = 0; i < n; i++) {
        const int l1 = t.column_pointers[i + 1] - t.column_pointers[i];
        const int l2 = m.row_pointers[i + 1] - m.row_pointers[i];
        out_rowptr[i] = MergeArr(t.row_indices + t.column_pointers[i], l1,
                                 m.column_indices + m.row_pointers[i], l2, out_col + len);
        len += out_rowptr[i];
    }
    out_rowptr[n] = 0;
    exclusive_scan(out_rowptr, n + 1);
    free(t.column_pointers);
    free(t.row_indices);
    free(t.values);
    free_csr(&m);
    return len;
}
