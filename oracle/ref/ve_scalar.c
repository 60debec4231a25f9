/*
 * Scalar C restatement of the NEC-VE kernel functions that the reference's
 * level loop (bfs/src/bfs_SELLCSv2.c) calls, so that the reference's own
 * level loop links and runs on a CPU without velintrin.h. Test
 * infrastructure only: it is compiled together with the reference sources
 * by oracle/Makefile.ref into oracle/_ref/ and used to produce golden
 * vectors.
 *
 * Each function restates the vector code lane by lane (slice height 256,
 * visited bit of lane l = bit 63-(l%64) of mask word 4*slice + l/64):
 *   kernel_SELLCS_DFC                     bfs/src/bfs_par_kernels.c:8-53
 *   bfs_kernel_SELLCS_DFC_bitmap          bfs/src/bfs_par_kernels.c:128-198
 *   bfs_kernel_spmspv_SELLCS_DFC_bitmap   bfs/src/bfs_par_kernels.c:566-656
 *   spmv_merge_res                        bfs/src/bfs_par_kernels.c:696-713
 *   merge_res                             bfs/src/bfs_par_kernels.c:715-729
 *   sparse2dense                          bfs/src/bfs_par_kernels.c:731-753
 *   dense2sparse                          bfs/src/bfs_par_kernels.c:754-787
 *   reset                                 bfs/src/bfs_par_kernels.c:789-797
 * The float-path and merge-path kernels are never reached with bit_flag = 1
 * and equal switch thresholds (bfs_SELLCSv2.c:283-284, main.c:189); they
 * only record that they were called.
 */
#include <math.h>

#include "bfs_par_kernels.h"

int ve_scalar_dead_calls = 0;

#define VL 256

static int lane_vis(const size_t *mask, int s, int l)
{
    return (int)((mask[s * 4 + l / 64] >> (63 - (l % 64))) & 1UL);
}

static void lane_set(size_t *mask, int s, int l)
{
    mask[s * 4 + l / 64] |= (1UL << (63 - (l % 64)));
}

static int max_lanes_of(const SparseMatrixSELLCS *m, int s)
{
    int row = s << 8;
    return (row + VL > m->nrows) ? (m->nrows - row) : VL;
}

void kernel_SELLCS_DFC(const SparseMatrixSELLCS *restrict m, const elem_t *restrict x,
                       elem_t *restrict y, const int start_slice, const int end_slice)
{
    for (int s = start_slice; s < end_slice; s++) {
        int lanes = max_lanes_of(m, s);
        elem_t acc[VL];
        for (int l = 0; l < VL; l++)
            acc[l] = 0;
        int at = m->slice_pointers[s];
        int op = m->vop_pointers[s];
        for (int i = 0; i < m->slice_widths[s]; i++) {
            int act = (int)m->vop_lengths[op++] + 1;
            for (int l = 0; l < act; l++) /* _vel_vfmadd_vvvvl: one rounding */
                acc[l] = fma(x[m->column_indices[at + l]], m->values[at + l], acc[l]);
            at += act;
        }
        for (int l = 0; l < lanes; l++)
            y[m->row_order[(s << 8) + l]] = acc[l];
    }
}

void bfs_kernel_SELLCS_DFC_bitmap(const SparseMatrixSELLCS *restrict m, const int *mask_x,
                                  int *mask_y, int *nnzy, const int start_slice,
                                  const int end_slice, size_t *mask, int *bypass_slice)
{
    int cnt = 0;
    for (int s = start_slice; s < end_slice; s++) {
        int lanes = max_lanes_of(m, s);
        int vis = 0;
        for (int l = 0; l < lanes; l++)
            vis += lane_vis(mask, s, l);
        if (vis < lanes) {
            long acc[VL];
            for (int l = 0; l < VL; l++)
                acc[l] = 0;
            int at = m->slice_pointers[s];
            int op = m->vop_pointers[s];
            for (int i = 0; i < m->slice_widths[s]; i++) {
                int act = (int)m->vop_lengths[op++] + 1;
                for (int l = 0; l < act; l++)
                    acc[l] |= (long)(unsigned)mask_x[m->column_indices[at + l]];
                at += act;
            }
            for (int l = 0; l < lanes; l++) {
                if (acc[l] > 0 && !lane_vis(mask, s, l)) {
                    lane_set(mask, s, l);
                    mask_y[m->row_order[(s << 8) + l]] = (int)acc[l];
                    cnt++;
                }
            }
        } else {
            (*bypass_slice)++;
        }
    }
    (*nnzy) = cnt;
}

void bfs_kernel_spmspv_SELLCS_DFC_bitmap(const SparseMatrixSELLCS *restrict m,
                                         const int *slice_idx_max, const int *slice_idx_min,
                                         const int *bucket, const int *colidx_x,
                                         const int *nnzx, const int x_max, const int x_min,
                                         int *colidx_y, int *nnzy, const int start_slice,
                                         const int end_slice, size_t *mask,
                                         int *bypass_slice, int *bypass_width)
{
    int cnt = 0;
    (void)nnzx;
    for (int s = start_slice; s < end_slice; s++) {
        if (slice_idx_max[s] < x_min || slice_idx_min[s] > x_max) {
            (*bypass_slice)++;
            continue;
        }
        int lanes = max_lanes_of(m, s);
        int vis = 0;
        for (int l = 0; l < lanes; l++)
            vis += lane_vis(mask, s, l);
        if (vis >= lanes)
            continue;
        unsigned char hit[VL];
        for (int l = 0; l < VL; l++)
            hit[l] = 0;
        int at = m->slice_pointers[s];
        int op = m->vop_pointers[s];
        for (int i = 0; i < m->slice_widths[s]; i++) {
            int act = (int)m->vop_lengths[op + i] + 1;
            if (!(m->max_index[op + i] < x_min || m->min_index[op + i] > x_max)) {
                for (int l = 0; l < act; l++) {
                    int c = m->column_indices[at + l];
                    if (colidx_x[bucket[c]] == c)
                        hit[l] = 1;
                }
            } else {
                (*bypass_width)++;
            }
            at += act;
        }
        int base = (start_slice << 8) + cnt;
        int k = 0;
        for (int l = 0; l < lanes; l++) {
            if (hit[l] && !lane_vis(mask, s, l)) {
                lane_set(mask, s, l);
                colidx_y[base + k++] = m->row_order[(s << 8) + l];
            }
        }
        cnt += k;
    }
    (*nnzy) = cnt;
}

void spmv_merge_res(elem_t *x, int *mask_x, int start_pos, int end_pos, elem_t *y,
                    int *mask_y, int MVL, bool bit_flag)
{
    (void)MVL;
    for (int i = start_pos; i < end_pos; i++) {
        if (!bit_flag)
            x[i] = y[i];
        else
            mask_x[i] = mask_y[i];
    }
}

void merge_res(elem_t *bfs_y, int *colidx_y, int start_pos, int nnz, elem_t *bfs_y_tmp,
               int *colidx_y_tmp, const int max_lanes, bool bit_flag)
{
    (void)max_lanes;
    for (int i = 0; i < nnz; i++) {
        if (!bit_flag)
            bfs_y[start_pos + i] = bfs_y_tmp[i];
        colidx_y[start_pos + i] = colidx_y_tmp[i];
    }
}

void sparse2dense(elem_t *bfs_y, int *colidx_y, int nnz, elem_t *bfs_x, int *mask_x,
                  int MVL, bool bit_flag, int nrows)
{
    (void)MVL;
    (void)nrows;
    for (int i = 0; i < nnz; i++) {
        if (!bit_flag)
            bfs_x[colidx_y[i]] = bfs_y[i];
        else
            mask_x[colidx_y[i]] = 1;
    }
}

void dense2sparse(elem_t *bfs_y, int *mask_y, int start_pos, int end_pos, int nnz_start,
                  elem_t *bfs_x, int *mask_x, int *colidx_x, int MVL, bool bit_flag,
                  int nrows)
{
    (void)MVL;
    (void)nrows;
    (void)mask_x;
    int k = 0;
    for (int i = start_pos; i < end_pos; i++) {
        if (!bit_flag) {
            if (bfs_y[i] > 0) {
                bfs_x[nnz_start + k] = bfs_y[i];
                colidx_x[nnz_start + k] = i;
                k++;
            }
        } else if (mask_y[i] > 0) {
            colidx_x[nnz_start + k] = i;
            k++;
        }
    }
}

void reset(int *arr, int start, int end, int MVL)
{
    (void)MVL;
    for (int i = start; i < end; i++)
        arr[i] = 0;
}

/* Unreached with bit_flag = 1 and equal thresholds: record the call only. */
void bfs_kernel_spmv_SELLCS_NC_DFC(const SparseMatrixSELLCS *restrict m, const elem_t *x,
                                   elem_t *y, int *nnzy, const int start_slice,
                                   const int end_slice, size_t *mask)
{
    (void)m; (void)x; (void)y; (void)start_slice; (void)end_slice; (void)mask;
    *nnzy = 0;
    ve_scalar_dead_calls++;
}

void bfs_kernel_spmspv_SELLCS_DFC(const SparseMatrixSELLCS *restrict m,
                                  const int *slice_idx_max, const int *slice_idx_min,
                                  const int *bucket, const elem_t *restrict x,
                                  const int *colidx_x, const int *nnzx, const int x_max,
                                  const int x_min, elem_t *restrict y, int *colidx_y,
                                  int *nnzy, const int start_slice, const int end_slice,
                                  size_t *mask, int *bypass_slice, int *bypass_width)
{
    (void)m; (void)slice_idx_max; (void)slice_idx_min; (void)bucket; (void)x;
    (void)colidx_x; (void)nnzx; (void)x_max; (void)x_min; (void)y; (void)colidx_y;
    (void)start_slice; (void)end_slice; (void)mask; (void)bypass_slice; (void)bypass_width;
    *nnzy = 0;
    ve_scalar_dead_calls++;
}

void csc_spmspv_merge(const SparseMatrixCSC *csc_matrix, const SparseMatrixSELLCS *restrict m,
                      const int *vop_length_ptr, const int *colidx_x, const int *nnzx,
                      elem_t *restrict y, int *colidx_y, int col_y_pos, int *mask_y,
                      int *nnzy, int *merge_row_order, int start_pos, int end_pos,
                      size_t *mask)
{
    (void)csc_matrix; (void)m; (void)vop_length_ptr; (void)colidx_x; (void)nnzx; (void)y;
    (void)colidx_y; (void)col_y_pos; (void)mask_y; (void)merge_row_order; (void)start_pos;
    (void)end_pos; (void)mask;
    *nnzy = 0;
    ve_scalar_dead_calls++;
}
