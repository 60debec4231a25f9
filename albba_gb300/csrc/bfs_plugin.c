/*
 * libbfs_gb300.so: the reference's BFS-variant interface (bfs/src/bfs.h:13-26,
 * globals of bfs/src/bfs_SELLCSv2.c:26-31) implemented on the albba C ABI.
 * See include/albba_bfs_plugin.h for the contract.
 */
#include "albba_bfs_plugin.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "albba.h"

enum MatrixFormat required_matrix_format = CSR;
char algorithm_version[30] = "BFS_GB300";
int sigma_window = 16384;
int num_blocks = 1;
int chunk_size = 8;

/* driver-owned globals: weak defaults, overridden by bfs/src/main.c */
__attribute__((weak)) size_t align_size = 64;
__attribute__((weak)) int perf_analysis = 0;
__attribute__((weak)) int verify = 0;
__attribute__((weak)) int bypass_record = 0;

static int *g_levels = NULL;
static int *g_parents = NULL;

const int *bfs_gb300_last_levels(void) { return g_levels; }
const int *bfs_gb300_last_parents(void) { return g_parents; }

/* Directory of the bypass records: the reference writes them to
 * ../bfs/data/ (bfs/src/bfs_SELLCSv2.c:774); ALB_BYPASS_DIR overrides it. */
static const char *bypass_dir(void)
{
    const char *d = getenv("ALB_BYPASS_DIR");
    return (d && *d) ? d : "../bfs/data";
}

/* One CSV line per run in the reference's bypass record format
 * (bfs/src/bfs_SELLCSv2.c:773-818): name, rows, columns, entries, levels, the
 * unit count, then one count per level. The slice record counts 32-row words
 * skipped because every row was visited (the reference's slices); the column
 * record counts 4-column groups a row left unread because it stopped at its
 * first frontier source, against the total of such groups per lane. */
static void write_bypass(const SparseMatrixCSR *m, alb_graph *g, const alb_level_rec *tr, int cnt)
{
    const char *name = m->name ? m->name : "matrix";
    const char *slash = strrchr(name, '/');
    if (slash) name = slash + 1;
    int64_t nslices = 0, nwords = 0;
    alb_sell_export(g, &nslices, NULL, NULL, NULL, NULL);
    int64_t *off = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nslices + 1));
    int64_t ngroups = 0;
    if (off && alb_sell_export(g, NULL, NULL, NULL, off, NULL) == ALB_OK)
        ngroups = off[nslices] / (4 * 32);
    free(off);
    nwords = (m->nrows + 31) / 32;
    const char *files[2] = {bypass_record == 2 ? "spmv-slice-bypass.csv" : "bfs-slice-bypass.csv",
                            "bfs-column-bypass.csv"};
    for (int f = 0; f < (bypass_record == 2 ? 1 : 2); f++) {
        char path[4096];
        snprintf(path, sizeof(path), "%s/%s", bypass_dir(), files[f]);
        FILE *out = fopen(path, "a");
        if (!out) { /* the reference crashes here (unchecked fopen) */
            fprintf(stderr, "bfs_gb300: cannot append to %s\n", path);
            continue;
        }
        fprintf(out, "%s,%i,%i,%i,%i,%lld", name, m->nrows, m->ncolumns, m->nnz, cnt,
                (long long)(f == 0 ? nwords : ngroups));
        for (int l = 0; l < cnt; l++)
            fprintf(out, ",%lld", (long long)(f == 0 ? tr[l].words_bypassed : tr[l].groups_bypassed));
        fprintf(out, "\n");
        fclose(out);
    }
}

static void report_failure(const char *what, int *num_iter, double *bfs_time)
{
    fprintf(stderr, "bfs_gb300: %s failed: %s\n", what, alb_last_error());
    *num_iter = 0;
    *bfs_time = -1.0;
}

void run_custom_bfs_test(const SparseMatrixCSR *m, elem_t *bfs_x, int *colidx_x, int *nnzx,
                         int *frontier, int *num_vex, double *conv_time, double *iter_times,
                         double *bfs_time, int *num_iter, bool bit_flag, bool sort_flag)
{
    (void)bfs_x;
    (void)bit_flag;
    (void)sort_flag;
    *num_iter = 0;
    *bfs_time = -1.0;
    if (!m || m->nrows <= 0 || !m->row_pointers) {
        fprintf(stderr, "bfs_gb300: empty or missing matrix\n");
        return;
    }
    const int n = m->nrows;
    const int root = (nnzx && *nnzx > 0 && colidx_x) ? colidx_x[0] : 0;
    alb_graph *g = NULL;
    if (alb_graph_create32(n, m->row_pointers, m->column_indices, ALB_CSR_IN, &g) != ALB_OK) {
        report_failure("graph upload", num_iter, bfs_time);
        return;
    }
    alb_sell_opts so;
    alb_sell_opts_default(&so);
    so.sigma = sigma_window < 1 ? 1 : (sigma_window > 16384 ? 16384 : sigma_window);
    double cms = 0;
    if (alb_sell_build(g, &so, &cms) != ALB_OK) {
        report_failure("SELL-C-sigma build", num_iter, bfs_time);
        alb_graph_destroy(g);
        return;
    }
    if (conv_time) *conv_time = cms;
    alb_bfs_opts bo;
    alb_bfs_opts_default(&bo);
    bo.trace = 1;
    if (perf_analysis) bo.loop = ALB_LOOP_HOST; /* CUDA-event time per level */
    int *lv = (int *)realloc(g_levels, sizeof(int) * (size_t)n);
    int *pa = (int *)realloc(g_parents, sizeof(int) * (size_t)n);
    if (!lv || !pa) {
        g_levels = lv;
        g_parents = pa;
        fprintf(stderr, "bfs_gb300: host allocation failed\n");
        alb_graph_destroy(g);
        return;
    }
    g_levels = lv;
    g_parents = pa;
    alb_stats st;
    if (alb_bfs(g, root, &bo, lv, pa, &st) != ALB_OK) {
        report_failure("BFS", num_iter, bfs_time);
        alb_graph_destroy(g);
        return;
    }
    int32_t cnt = 0;
    alb_level_rec *tr = (alb_level_rec *)malloc(sizeof(alb_level_rec) * (size_t)(st.num_levels + 1));
    if (tr && alb_level_trace(g, st.num_levels, tr, &cnt) == ALB_OK) {
        for (int32_t l = 0; l < cnt && l < st.num_levels; l++) {
            if (verify && frontier) frontier[l] = (int)tr[l].nf; /* bfs_SELLCSv2.c:444-447 */
            if (perf_analysis && iter_times) iter_times[l] = tr[l].step_us / 1000.0;
        }
        if (bypass_record == 1 || bypass_record == 2) write_bypass(m, g, tr, cnt);
    }
    free(tr);
    *num_iter = st.num_levels;
    *num_vex = (int)st.reached;
    *bfs_time = st.ms;
    if (nnzx) *nnzx = 0;
    printf("iteration = %d, bfs runtime = %.3f ms\n", *num_iter, *bfs_time); /* bfs_SELLCSv2.c:771 */
    alb_graph_destroy(g);
}

void print_additional_custom_report(char *text_padding, double *elapsed_times)
{
    (void)elapsed_times;
    printf("%s\"Row order sigma window\": %d,\n", text_padding, sigma_window);
    printf("%s\"Slice height\": 32\n", text_padding);
}
