/*
 * albba_gb300 synthetic graph generators (host, C ABI).
 *
 * The reference benchmarks on SuiteSparse matrices read from .mtx/.cbd files
 * (bfs/src/biio.h:127-149); it ships no generator. These generators build the
 * synthetic inputs used in their place: RMAT/Kronecker, a 2D grid with
 * dropped edges and long-range shortcuts, and an Erdos-Renyi graph. Every
 * random draw is a SplitMix64 hash of (seed, counter), so a graph depends on
 * its parameters only, not on thread count or machine.
 *
 * Output: symmetric CSR, self-loops and duplicates removed, rows ascending,
 * int64 row offsets, int32 ids. Arrays are malloc'd by the library and
 * released by alb_host_csr_free.
 */
#ifndef ALBBA_GEN_H
#define ALBBA_GEN_H

#include <stdint.h>
#include "albba.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int64_t n;
    int64_t nnz;
    int64_t *rowptr; /* n + 1 */
    int32_t *col;    /* nnz */
} alb_host_csr;

/* RMAT: 2^scale vertices, edgefactor * 2^scale generated edges, quadrant
 * probabilities a, b, c (d = 1 - a - b - c), vertex ids permuted by a seeded
 * Fisher-Yates shuffle when permute != 0. */
alb_status alb_gen_rmat(int32_t scale, int32_t edgefactor, uint64_t seed, double a,
                        double b, double c, int32_t permute, alb_host_csr *out);

/* rows x cols 4-neighbour grid (vertex r*cols + c), each grid edge dropped
 * with probability drop, plus round(shortcut_frac * n) random vertex pairs. */
alb_status alb_gen_grid(int32_t rows, int32_t cols, double drop, double shortcut_frac,
                        uint64_t seed, alb_host_csr *out);

/* Erdos-Renyi G(n, m) with m = round(n * mean_degree / 2) random pairs. */
alb_status alb_gen_er(int64_t n, double mean_degree, uint64_t seed, alb_host_csr *out);

/* Build a symmetric CSR from an edge list (u[i], v[i]) over n vertices. */
alb_status alb_csr_from_edges(int64_t n, int64_t m, const int32_t *u, const int32_t *v,
                              alb_host_csr *out);

/* count distinct roots with degree >= 1, drawn from the seed. */
alb_status alb_pick_roots(const alb_host_csr *g, int32_t count, uint64_t seed,
                          int32_t *roots);

void alb_host_csr_free(alb_host_csr *g);

/* Reference binary CSR (.cbd) files, bfs/src/biio.h:21-96:
 * int rows, cols, nnz; int row_ptr[rows+1]; int col_idx[nnz]; double val[nnz]. */
alb_status alb_cbd_write(const char *path, const alb_host_csr *g);
alb_status alb_cbd_read(const char *path, alb_host_csr *out);

/* Coordinate Matrix Market (.mtx) file -> CSR, as the reference's reader
 * builds it (replaces mmio_info + mmio_data, bfs/src/mmio_highlevel.h:11-263):
 * values dropped; symmetric and hermitian files have every off-diagonal entry
 * placed in both rows; entries in file order within a row (the mirrored copy
 * at its source entry's turn); skew-symmetric read as general. Refuses dense
 * files and non-square matrices (ALB_ERR_UNSUPPORTED), malformed files and
 * indices out of range (ALB_ERR_IO). *is_symmetric (may be NULL) = 1 for
 * symmetric or hermitian files. */
alb_status alb_mtx_read(const char *path, alb_host_csr *out, int32_t *is_symmetric);

/* The reference driver's undirected conversion of a non-symmetric graph
 * (bfs/src/main.c:127-163): row i = the two-pointer merge of row i of the
 * transpose and row i of the input (bfs/src/utils.c:351-380). */
alb_status alb_csr_undirected(const alb_host_csr *in, alb_host_csr *out);

/* Graph load of the reference driver (bfs/src/main.c:86-163, biio.h:127-149):
 * path ending in .cbd -> alb_cbd_read; .mtx -> alb_mtx_read, then
 * alb_csr_undirected unless the file is symmetric. */
alb_status alb_graph_read(const char *path, alb_host_csr *out);

#ifdef __cplusplus
}
#endif
#endif
