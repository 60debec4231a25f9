/*
 * albba_gb300 -- GB300-native linear-algebra BFS (C ABI).
 *
 * One process, one GPU (the current CUDA device when a graph is created).
 * Every entry point returns an alb_status (0 = ALB_OK, negative = error) and
 * never exits the process; alb_last_error() gives a message for the calling
 * thread's last failure. A graph is not thread-safe; distinct graphs may be
 * used from distinct threads.
 *
 * The reference (scalbba/albba) exposes the hot path as one plugin function,
 * run_custom_bfs_test (bfs/src/bfs.h:13-24), fed by a CSR loaded in
 * bfs/src/main.c:86-126. This header splits that path into its stages so a
 * caller can hold a graph on the device and run many roots:
 *
 *   reference                                   this library
 *   read_Dmatrix -> SparseMatrixCSR             alb_graph_create / _create32
 *     (bfs/src/biio.h:127-149, main.c:91)
 *   sellcs_preprocess (bfs_SELLCSv2.c:34-59)    alb_sell_build
 *   level loop (bfs_SELLCSv2.c:296-762)         alb_bfs / alb_bfs_device
 *   frontier[] / num_iter / num_vex / bfs_time  alb_stats + alb_level_trace
 *   (no counterpart)                            alb_msbfs64, alb_worklist_*,
 *                                               alb_selector_*, alb_tune_*
 *
 * The drop-in with the reference's exact plugin signature is
 * include/albba_bfs_plugin.h.
 *
 * Index space: vertex ids are int32 (n < 2^31); row offsets are int64, so a
 * graph may hold more than 2^31 stored entries (the reference's int nnz,
 * bfs/src/sparse_matrix.h:26, cannot).
 */
#ifndef ALBBA_H
#define ALBBA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t alb_status;
#define ALB_OK 0
#define ALB_ERR_INVALID (-1)     /* bad argument (null pointer, root out of range, ...) */
#define ALB_ERR_OOM (-2)         /* device or host allocation failed */
#define ALB_ERR_CUDA (-3)        /* CUDA runtime error (includes "no GPU") */
#define ALB_ERR_TIMEOUT (-4)     /* a bounded device-side wait gave up */
#define ALB_ERR_STATE (-5)       /* call order (e.g. BFS before alb_sell_build) */
#define ALB_ERR_IO (-6)          /* file read/write failed or file malformed */
#define ALB_ERR_UNSUPPORTED (-7) /* option outside the supported range */
#define ALB_ERR_DEVICE (-8)      /* a kernel reported an internal bound violation */

/* Thread-local message for the last failing call on this thread. */
const char *alb_last_error(void);
/* Library version string. */
const char *alb_version(void);

/* ---------------------------------------------------------------- graphs */

typedef struct alb_graph alb_graph;

/* CSR orientation flags for alb_graph_create*. */
#define ALB_CSR_OUT 0u       /* row u lists the targets of u's edges */
#define ALB_CSR_IN 1u        /* row v lists the sources of v's edges: the
                                reference's working matrix after its
                                transpose (bfs/src/main.c:117-126) */
#define ALB_CSR_SYMMETRIC 2u /* A == A^T (both of the above) */
#define ALB_CSR_SORTED 4u    /* caller guarantees ascending rows (skips the
                                check; rows are sorted when the flag is absent) */

/* Copy a host CSR (int64 offsets) to the current device. Duplicate entries
 * are kept as given; self-loops are ignored by the traversal. */
alb_status alb_graph_create(int64_t n, const int64_t *rowptr, const int32_t *col,
                            uint32_t flags, alb_graph **out);
/* Same, from the reference's int32 CSR (bfs/src/sparse_matrix.h:18-28). */
alb_status alb_graph_create32(int32_t n, const int32_t *rowptr, const int32_t *col,
                              uint32_t flags, alb_graph **out);
/* Every O(nnz) step of graph creation runs on the device: the CSR is copied
 * as given, then checked there (offsets from 0 to nnz, never decreasing;
 * columns in [0, n): ALB_ERR_INVALID otherwise), rows sorted ascending when
 * they are not, and -- unless ALB_CSR_SYMMETRIC -- transposed (rows of the
 * transpose ascending, as the reference's counting transpose leaves them,
 * bfs/src/sparse_matrix.c:230-290); a transpose equal to the matrix is
 * dropped and the graph marked symmetric. */

/* The reference driver's undirected graph of a non-symmetric input
 * (bfs/src/main.c:127-163), built on the device: row i = MergeArr(column i of
 * A, row i of A as given) (bfs/src/utils.c:351-379). Host CSR in (rows in
 * any order, duplicates kept); the graph is symmetric, rows sorted. */
alb_status alb_graph_create_undirected(int64_t n, const int64_t *rowptr, const int32_t *col,
                                       alb_graph **out);
/* Graph load of the reference driver (bfs/src/main.c:86-163) onto the
 * device: .cbd files (bfs/src/biio.h:21-149) as is (ALB_CSR_IN: the
 * reference's working matrix), .mtx files parsed on the host, then on the
 * device either taken as symmetric or made undirected as above. */
alb_status alb_graph_load(const char *path, alb_graph **out);
void alb_graph_destroy(alb_graph *g);

alb_status alb_graph_info(const alb_graph *g, int64_t *n, int64_t *nnz);
/* Copy the device CSR to host buffers: side 0 = pull side (row v lists v's
 * sources), 1 = push side (row u lists u's targets); rowptr[n+1], col[nnz]
 * (either may be NULL). Rows are ascending. */
alb_status alb_graph_export_csr(const alb_graph *g, int32_t side, int64_t *rowptr, int32_t *col);
/* *symmetric = 1 when one CSR serves both sides (declared or detected). */
alb_status alb_graph_is_symmetric(const alb_graph *g, int32_t *symmetric);

/* Run the graph's work on a caller-provided cudaStream_t (NULL restores the
 * graph's own stream). Entry points still synchronise that stream before
 * returning host-visible results. */
alb_status alb_graph_set_stream(alb_graph *g, void *cuda_stream);

/* ------------------------------------------------------------ SELL-C-sigma */

typedef struct {
    int32_t C;        /* slice height: 8, 16, 32 (default) or 64 */
    int32_t sigma;    /* sort window in rows: 1 .. 16384 (default 1024) */
    int32_t long_row; /* rows longer than this are kept out of the slices and
                         pulled by a whole warp each (default 1024; <= 0: none) */
} alb_sell_opts;

void alb_sell_opts_default(alb_sell_opts *o);

/* Build the device SELL-C-sigma matrix (degree sort inside sigma windows by
 * a device segmented radix sort, slice-major 4-interleaved int32 columns in
 * sorted-position space) and the position-space push CSR. Replaces
 * sellcs_preprocess (bfs/src/bfs_SELLCSv2.c:34-59). *ms (optional) receives
 * the build time in milliseconds. Rebuilding with new options is allowed. */
alb_status alb_sell_build(alb_graph *g, const alb_sell_opts *o, double *ms);

/* Copy the built SELL arrays to host buffers (any pointer may be NULL):
 * perm[n] (position -> original id), width[nslices], slice_off[nslices+1]
 * (int64, in int32 entries), col[slice_off[nslices]]. */
alb_status alb_sell_export(const alb_graph *g, int64_t *nslices, int32_t *perm,
                           int32_t *width, int64_t *slice_off, int32_t *col);
/* The long-row list: lrow[nlong] positions (ascending), lptr[nlong+1],
 * lcol[lptr[nlong]] sources as positions in row order (NULL to skip). */
alb_status alb_sell_long_export(const alb_graph *g, int64_t *nlong, int32_t *lrow,
                                int64_t *lptr, int32_t *lcol);

/* -------------------------------------------------------------------- BFS */

/* Direction policy. Policies change speed only, never the BFS result. */
#define ALB_POLICY_BEAMER 0    /* Beamer alpha/beta direction optimisation */
#define ALB_POLICY_REF004 1    /* the reference's rule: pull when the frontier
                                  holds more than 4% of n
                                  (bfs/src/bfs_SELLCSv2.c:283-284, 344-356) */
#define ALB_POLICY_LEARNED 2   /* device MLP selector (falls back to BEAMER
                                  when no weights are loaded) */
#define ALB_POLICY_TOPDOWN 3   /* every level top-down push */
#define ALB_POLICY_BOTTOMUP 4  /* every level bottom-up pull with bypass
                                  (level 0 runs top-down) */
#define ALB_POLICY_BOTTOMUP_NOBYPASS 5 /* bottom-up pull, no slice bypass */

/* Level-loop driver. */
#define ALB_LOOP_HOST 0       /* one set of launches per level, host decides */
#define ALB_LOOP_GRAPH 1      /* CUDA graph with a device-driven while node */
#define ALB_LOOP_PERSISTENT 2 /* one cooperative kernel for all levels */

/* Variant ids (per-level direction records, selector classes). */
#define ALB_DIR_TOPDOWN 0
#define ALB_DIR_BOTTOMUP 1
#define ALB_DIR_BOTTOMUP_NOBYPASS 2

typedef struct {
    int32_t policy;  /* ALB_POLICY_* (default BEAMER) */
    int32_t loop;    /* ALB_LOOP_* (default GRAPH) */
    float alpha;     /* top-down -> bottom-up when m_f > m_u / alpha (14) */
    float beta;      /* bottom-up -> top-down when n_f < n / beta (24) */
    int32_t block;   /* threads per block for the level kernels (256) */
    int32_t trace;   /* record per-level statistics (alb_level_trace) */
} alb_bfs_opts;

void alb_bfs_opts_default(alb_bfs_opts *o);

typedef struct {
    int32_t num_levels;   /* non-empty levels (the reference's num_iter) */
    int32_t levels_topdown;
    int32_t levels_bottomup;
    int32_t pushed_roots; /* 64-root batched BFS: roots pushed instead of pulled
                             at a bottom-up level (0 for the other forms) */
    int64_t reached;      /* vertices reached (the reference's num_vex) */
    int64_t edges;        /* stored push-side entries of reached vertices */
    double ms;            /* device time of the traversal, SELL build excluded */
    int64_t kernels;      /* kernel launches made by this call */
} alb_stats;

/* Single-root BFS. level[v] = depth or -1; parent[v] = smallest original id
 * among v's sources one level up (root -> root, unreached -> -1). Host
 * output buffers of n int32 each; either may be NULL. */
alb_status alb_bfs(alb_graph *g, int32_t root, const alb_bfs_opts *o,
                   int32_t *level, int32_t *parent, alb_stats *st);
/* Same with device output buffers (n int32 each, either may be NULL). */
alb_status alb_bfs_device(alb_graph *g, int32_t root, const alb_bfs_opts *o,
                          int32_t *d_level, int32_t *d_parent, alb_stats *st);

typedef struct {
    int32_t dir;           /* ALB_DIR_* used for this level */
    int32_t level;         /* frontier depth */
    int64_t nf;            /* frontier vertices */
    int64_t mf;            /* push-side entries of the frontier */
    int64_t nu;            /* unvisited vertices before this level */
    int64_t mu;            /* pull-side entries of unvisited vertices */
    int64_t active_slices; /* bitmap words (32 rows) with an unvisited row */
    int64_t t_ns;          /* device timestamp at level start (ns) */
    int64_t bytes;         /* algorithmic bytes of the level's step (see below) */
    float step_us;         /* CUDA-event time of the step kernels (host loop
                              only; -1 otherwise) */
    int32_t pad_;
    /* Bypass statistics of the single-root BFS, counted by the kernels (the
     * reference records slice and column bypass per level,
     * bfs/src/bfs_SELLCSv2.c:773-818, counted at bfs/src/bfs_par_kernels.c:
     * 192 and 630; 0 for the 64-root batched BFS). Bottom-up levels: */
    int64_t words_bypassed;  /* 32-row bitmap words skipped because every row
                                in them was visited (slice bypass) */
    int64_t rows_scanned;    /* unvisited rows whose SELL columns were read */
    int64_t groups_read;     /* 4-column groups those rows read */
    int64_t groups_bypassed; /* groups of those rows (up to the slice width)
                                left unread because the row stopped at its
                                first frontier source or its end (column
                                bypass) */
    /* Top-down levels: */
    int64_t edges_bypassed;  /* pushed entries whose target was already
                                visited (no parent/claim update issued) */
} alb_level_rec;
/* Algorithmic bytes (the elements the step reads or writes, counted by the
 * kernels themselves): bottom-up = 12*nwords (visited read and write, next
 * frontier write) + 32 per row per 4-column group scanned (four int32
 * columns, the four frontier words they select) + 20 per row reached (level,
 * parent, the parent's id, two degrees) + 8 per long-row source scanned;
 * top-down = 20*|F| + 8*sum(deg F) + 12*|F_next| (queue + offsets, adjacency
 * + visited probes, level/parent/queue writes). The 64-root batched BFS
 * counts the same way with 8-byte frontier and visited words: 8 per row
 * pulled, 48 per 4-column group (32 + 8 per frontier word fetched when the
 * nonzero bitmap is consulted), 12 per row reached, 8*npad + 8*nwords for the
 * next-frontier, done and nonzero-bitmap words; a bottom-up level's push of
 * its pushed roots adds 4 per bitmap word + 8 per frontier row + 4 per queued
 * row (queue build), 20 per queued row, 16 per edge, 16 per new claim, and
 * the per-root frontier sampling that precedes it 4 per sampled word + 16 per
 * sampled row + 12 to 16 per long row. */

/* Per-level records of the last traversal on g (requires opts.trace). */
alb_status alb_level_trace(const alb_graph *g, int32_t cap, alb_level_rec *out,
                           int32_t *count);

/* ------------------------------------------------------ 64-root batched BFS */

/* Bit-parallel BFS from up to 64 roots at once (one uint64 frontier/visited
 * word per vertex, one traversal of the matrix per level for all roots).
 * levels (host, n * 64 int32) is vertex-major: levels[v * 64 + i] = depth of
 * v from roots[i], -1 if unreached (and for i >= nroots); page-locked host
 * memory is written by the device directly, other host memory through a
 * device buffer and one copy. The level loop is a CUDA graph that decides
 * and launches every level on the device (ALB_LOOP_GRAPH, the default; the
 * host steps in only when the 32-level snapshot store fills) or host-driven
 * (ALB_LOOP_HOST: one small device-to-host read per level); the direction of
 * each level is decided on the device (policy as for alb_bfs; the learned
 * policy uses selector 1). stats: reached = (vertex, root) pairs reached,
 * edges = sum over roots of push-side entries in the root's component. */
alb_status alb_msbfs64(alb_graph *g, const int32_t *roots, int32_t nroots,
                       const alb_bfs_opts *o, int32_t *levels, alb_stats *st);
/* Same with a device output buffer of n * 64 int32 (may be NULL). */
alb_status alb_msbfs64_device(alb_graph *g, const int32_t *roots, int32_t nroots,
                              const alb_bfs_opts *o, int32_t *d_levels, alb_stats *st);

/* ---------------------------------------------------------------- work list */

/* Many (graph, root) traversals of small graphs in one persistent launch:
 * each CTA runs one traversal at a time with its frontier, next-frontier and
 * visited bitmaps in shared memory, popping the next item from a global
 * counter (longest graphs first). Graphs keep their own SELL build (C, sigma,
 * long rows) and Beamer thresholds. Levels only (no parents). A graph added
 * to a work list must outlive the list's runs. A graph whose bitmaps exceed
 * one CTA's shared memory (3 bits per vertex: above about 600K vertices)
 * runs its items one by one on the single-root path (alb_bfs_device,
 * CUDA-graph loop, the entry's alpha and beta) into the same output. */
typedef struct alb_worklist alb_worklist;
alb_status alb_worklist_create(alb_worklist **out);
void alb_worklist_destroy(alb_worklist *w);
alb_status alb_worklist_add(alb_worklist *w, alb_graph *g, const int32_t *roots, int32_t nroots,
                            float alpha, float beta);
/* Total int32 level entries (sum over items of n) and item count. */
alb_status alb_worklist_size(const alb_worklist *w, int64_t *level_entries, int32_t *items);
/* levels: host buffer of alb_worklist_size entries; item k (in the order
 * added, roots in order) occupies n_g consecutive entries, original ids.
 * block: threads per CTA (128, 256, 512 or 1024). stats.ms = kernel time
 * plus the single-root runs of graphs too large for the kernel; stats.kernels
 * counts the kernel and those runs' launches. */
alb_status alb_worklist_run(alb_worklist *w, int32_t block, int32_t *levels, alb_stats *st);
alb_status alb_worklist_run_device(alb_worklist *w, int32_t block, int32_t *d_levels,
                                   alb_stats *st);

/* --------------------------------------------------------------- selector */

/* Load the 1,443 fp32 parameters of a direction-selector MLP
 * (8 -> 32 -> 32 -> 3, ReLU; layout W1[32][8], b1, W2[32][32], b2, W3[3][32],
 * b3). which = 0: single-root BFS, 1: 64-root batched BFS. The MLP's output k
 * is the predicted cost of variant k (ALB_DIR_*); the cheapest is taken. */
alb_status alb_selector_load(int32_t which, const float *params);
/* Forget loaded weights (ALB_POLICY_LEARNED falls back to Beamer). */
alb_status alb_selector_clear(int32_t which);

/* Per-level oracle timings. At every level each variant (ALB_DIR_*) runs
 * from the same state (restored between runs) and its step kernels are timed
 * with CUDA events; the traversal then continues with the fastest. Levels and
 * parents are those of alb_bfs; this is the selector's training data and the
 * judge of its regret. */
typedef struct {
    alb_level_rec rec; /* statistics at the start of the level */
    float feat[8];     /* the selector's eight features for this level */
    float us[3];       /* step time of each variant, microseconds */
    int32_t best;      /* fastest variant (the one the traversal took) */
} alb_level_profile;

alb_status alb_bfs_profile(alb_graph *g, int32_t root, const alb_bfs_opts *o, int32_t cap,
                           alb_level_profile *out, int32_t *count);
alb_status alb_msbfs64_profile(alb_graph *g, const int32_t *roots, int32_t nroots,
                               const alb_bfs_opts *o, int32_t cap, alb_level_profile *out,
                               int32_t *count);

/* The selector's hand-written CUDA kernels, callable on host arrays:
 * forward (batch x 8 -> batch x 3), loss + gradient (masked squared error,
 * mean over the batch), one Adam step, and full-batch Adam training
 * (He initialisation from seed when init != 0, else params is the start). */
alb_status alb_mlp_forward(const float *params, const float *x, int32_t batch, float *out);
alb_status alb_mlp_loss_grad(const float *params, const float *x, const float *y,
                             const float *mask, int32_t batch, float *grad, float *loss);
alb_status alb_adam_step(float *params, const float *grad, float *m, float *v, int32_t t,
                         float lr, float beta1, float beta2, float eps);
alb_status alb_selector_train(const float *x, const float *y, const float *mask, int32_t batch,
                              int32_t steps, float lr, uint64_t seed, int32_t init,
                              float *params, float *loss);

/* ------------------------------------------- sparse frontier expansion */

/* The reference's push-merge kernel csc_spmspv_merge
 * (bfs/src/bfs_par_kernels.c:350-416, with the task merge of
 * bfs/src/bfs_SELLCSv2.c:530-575): the next frontier of the frontier x[nx]
 * (original ids) as the ascending, duplicate-free list of the out-neighbours
 * of x whose bit in visited (host bitmap over original ids, n bits, bit
 * v & 31 of word v >> 5) is clear. *ny receives the list's length; y (host,
 * may be NULL) must hold up to n entries. Computed by marking a bitmap on
 * the device and compacting it in id order, which gives the reference's
 * sorted merge result without merging. */
alb_status alb_spmspv_merge(alb_graph *g, const int32_t *x, int64_t nx, const uint32_t *visited,
                            int32_t *y, int64_t *ny);

/* ----------------------------------------------- fp64 SELL-C-sigma SpMV */

/* y = A x in fp64 over a SELL-C-sigma matrix on the device. Replaces the
 * reference's kernel_SELLCS_DFC (bfs/src/bfs_par_kernels.c:8-53) and its
 * matrix build convert_csr_to_sellcs_dfc (bfs/src/sparse_matrix.c:523-623):
 * row r accumulates values[e] * x[col[e]] over its entries in CSR order with
 * one fused multiply-add each, starting from 0 -- the reference's per-lane
 * vfmadd chain -- so y is bit-identical to the reference's for the same CSR.
 * Rows are ordered by length inside sigma windows (1..16384) as in the
 * reference; slices hold 32 rows, entries 4-interleaved (int32 columns,
 * fp64 values), diagonal and repeated entries kept as given. Rows longer
 * than 512 entries are summed one lane each from a separate list (the eight
 * longest on SMs of their own): the in-order chain of fused multiply-adds
 * makes a launch last at least as long as its longest row's chain. */
typedef struct alb_sellmat alb_sellmat;
alb_status alb_sellmat_create(int64_t n, const int64_t *rowptr, const int32_t *col,
                              const double *values, int32_t sigma, alb_sellmat **out);
void alb_sellmat_destroy(alb_sellmat *m);
/* n, entries, and stored SELL slots (entries + padding). */
alb_status alb_sellmat_info(const alb_sellmat *m, int64_t *n, int64_t *nnz, int64_t *stored);
/* Device vectors x[n], y[n] (current device); kernel_us (may be NULL)
 * receives the kernel's CUDA-event time in microseconds. */
alb_status alb_sellmat_spmv(alb_sellmat *m, const double *d_x, double *d_y, float *kernel_us);
/* Host vectors, copied in and out. */
alb_status alb_sellmat_spmv_host(alb_sellmat *m, const double *x, double *y);

/* ---------------------------------------------------------------- testing */

/* Host-side fault injection: the k-th next device allocation made by the
 * library fails with ALB_ERR_OOM (k >= 1); k = 0 disarms. */
void alb_debug_fail_alloc_after(int32_t k);

/* Test hooks for the bounded device-side waits (the reference has no
 * failure handling: bfs/src/utils.c:102-109 exits). timeout_us > 0 makes
 * every such wait give up after timeout_us instead of seconds;
 * withhold_level >= 0 makes block withhold_block skip its arrival at the grid
 * barriers of that level (the persistent level loop and
 * alb_bfs_csr_noalloc), so the other blocks' waits run out; short_bulk != 0
 * makes the staged bottom-up pass expect 16 bytes more than its bulk copy
 * delivers, so its wait runs out. The call that hits one returns
 * ALB_ERR_TIMEOUT; nothing faults and the next call on the same graph runs
 * normally. (-1, 0, 0, 0) turns everything off. */
void alb_debug_device_waits(int32_t withhold_level, int32_t withhold_block, int32_t short_bulk,
                            int64_t timeout_us);

#ifdef __cplusplus
}
#endif
#endif
