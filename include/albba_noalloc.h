/*
 * albba_gb300 -- BFS entry point that allocates no memory.
 *
 * No counterpart in the reference (scalbba/albba): it exists for callers that
 * cannot call cudaMalloc, such as a plug-in inside a process whose device
 * memory is owned by another allocator (a framework's caching allocator, a
 * fixed-budget serving process) or a latency-critical caller that cannot
 * accept cudaMalloc's implicit device synchronisation.
 */
#ifndef ALBBA_NOALLOC_H
#define ALBBA_NOALLOC_H

#include <stdint.h>

#include "albba.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Single-root BFS on a CSR the caller already holds on the current device:
 * d_rowptr[n+1] (int64), d_col (int32, rows ascending) in; d_level[n],
 * d_parent[n] (int32) out, with the same values as alb_bfs (parent = the
 * smallest source one level up, root -> root, unreached -> -1).
 * symmetric != 0: row u lists u's neighbours and both directions are used;
 * symmetric == 0: row u lists the targets of u's edges and every level is a
 * top-down push. stream: a cudaStream_t or NULL.
 *
 * Nothing is allocated: all temporaries live in one fixed device array of
 * 8,782,080 bytes (8.4 MiB) inside the library (held by every GPU that loads
 * it until the process exits), so n is limited to 2^20 vertices; larger graphs get
 * ALB_ERR_UNSUPPORTED. The first call on a device looks up that array's
 * address (cudaGetSymbolAddress, with the device current) and caches it:
 * make the first call before any stream capture. All calls share the array
 * and each call clears what must start at zero; calls that overlap on the
 * GPU race on it, so serialise them. */
alb_status alb_bfs_csr_noalloc(int64_t n, const int64_t *d_rowptr, const int32_t *d_col,
                               int32_t symmetric, int32_t root, int32_t *d_level,
                               int32_t *d_parent, void *stream);

#ifdef __cplusplus
}
#endif
#endif
