// Device-side CSR ingest (ingest.cu): every O(nnz) step of getting a caller's
// CSR into the shape the traversal needs runs on the device.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "albba.h"

namespace alb {

// Offsets start at 0, never decrease and end at nnz; columns in [0, n)
// (ALB_ERR_INVALID otherwise). *sorted: every row ascending (sorted == NULL:
// the order is not checked).
alb_status csr_check(int64_t n, const int64_t *d_rp, const int32_t *d_col, int64_t nnz,
                     cudaStream_t st, bool *sorted);
// Sorts every row ascending in place.
alb_status sort_rows(int64_t n, const int64_t *d_rp, int32_t *d_col, int64_t nnz, cudaStream_t st);
// Transpose with ascending rows (device buffers allocated with dmalloc).
alb_status transpose(int64_t n, const int64_t *d_rp, const int32_t *d_col, int64_t nnz,
                     int64_t **d_trp, int32_t **d_tcol, cudaStream_t st);
// Entry-for-entry equality of two CSRs with nnz entries each.
alb_status csr_equal(int64_t n, const int64_t *rp_a, const int32_t *col_a, const int64_t *rp_b,
                     const int32_t *col_b, int64_t nnz, cudaStream_t st, bool *equal);
// A u A^T as the reference's driver builds it (MergeArr of column i and row i).
alb_status merge_undirected(int64_t n, const int64_t *d_rp, const int32_t *d_col, int64_t nnz,
                            int64_t **d_urp, int32_t **d_ucol, int64_t *unnz, cudaStream_t st);

}  // namespace alb
