/*
 * albba_gb300 -- BFS entry point that allocates no memory.
 *
 * No counterpart in the reference (scalbba/albba): it exists for callers that
 * cannot call cudaMalloc, such as a plug-in inside a process whose device
 * memory is owned by another allocator (a framework's caching allocator that
 * must account for every byte, a fixed-budget serving process that reserves
 * all device memory up front), where an allocation of its own would fail or
 * break the owner's accounting.
 */
#ifndef ALBBA_NOALLOC_H
#define ALBBA_NOALLOC_H

#include <stdint.h>

#include "albba.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Single-root BFS on a CSR the caller already holds on the current device:
 * d_rowptr[n+1] (int64), d_col (int32) in; d_level[n], d_parent[n] (int32)
 * out, with the same values as alb_bfs (parent = the smallest source one
 * level up, root -> root, unreached -> -1).
 * symmetric != 0: row u lists u's neighbours and both directions are used.
 *   The rows must then be ascending: the bottom-up levels take the first
 *   frontier source of a row as the parent, which is the smallest only in an
 *   ascending row (with unsorted rows the levels are still exact, but a
 *   parent may be any source one level up).
 * symmetric == 0: row u lists the targets of u's edges and every level is a
 *   top-down push (parents are the smallest source in any row order).
 * stream: a cudaStream_t or NULL. The call waits for that stream once before
 * it returns (it reads the traversal's status back to the host).
 *
 * Nothing is allocated: all temporaries live in one fixed device array of
 * 8,782,080 bytes (8.4 MiB) inside the library (held by every GPU that loads
 * it until the process exits), so n is limited to 2^20 vertices; larger
 * graphs get ALB_ERR_UNSUPPORTED. The first call on a device looks up that
 * array's address (cudaGetSymbolAddress, with the device current) and caches
 * it for the device's current context; a call after the context was destroyed
 * and recreated (cudaDeviceReset) looks it up again. Make the first call on a
 * device before any stream capture. All calls share the array and each call
 * clears what must start at zero; calls that overlap on the GPU race on it,
 * so serialise them. */
alb_status alb_bfs_csr_noalloc(int64_t n, const int64_t *d_rowptr, const int32_t *d_col,
                               int32_t symmetric, int32_t root, int32_t *d_level,
                               int32_t *d_parent, void *stream);

#ifdef __cplusplus
}
#endif
#endif
