/*
 * CPU oracle for the persistent graph kernels and the non-persistent tasks.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls this
 * code; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
 * reference arms load it, and only as the checker or the timed CPU baseline.
 *
 * Every function restates one reference algorithm phase by phase and cites the
 * reference file:line it follows (paths relative to the reference project).
 * The restatement is pinned by tests against the reference's own OpenCL kernel
 * source compiled as C++ under a one-work-group shim (oracle/ref_shim), since
 * the reference ships no golden vectors.
 *
 * Graph layout everywhere: 0-based CSR, row_ptr[V+1], col[row_ptr[V]].
 * Callers that want the Lonestar loader's behaviour pass the CSR produced by
 * oracle_lonestar_csr_from_gr (the last edge of vertex V-1 is dropped).
 */
#ifndef WGM_ORACLE_H
#define WGM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_LONESTAR_INF 1000000000u /* lonestar/graph_apps/bfs/device/bfs.cl:33 */
#define ORACLE_PANNOTIA_BIG 99999999    /* pannotia/graph_apps/sssp/sssp.h:3 */

/* Lonestar `.gr` loader semantics (lonestar/graph_apps/bfs/bfs.h:40-46,137-161).
 * out_idx[i] is the Galois cumulative end index of vertex i; outs[] the
 * destinations.  Writes the 0-based CSR the device kernel actually walks:
 * row_ptr[i] = psrc[i]-1 for i<V and row_ptr[V] = nedges-1. */
void oracle_lonestar_csr_from_gr(int64_t V, int64_t E, const uint64_t *out_idx,
                                 const uint32_t *outs, int32_t *row_ptr,
                                 int32_t *col);

/* Lonestar BFS drelax2 (bfs.cl:104-302).  Returns the number of worklist
 * iterations the persistent loop ran (iteration 0 seeds the source). */
int oracle_lonestar_bfs(int32_t V, const int32_t *row_ptr, const int32_t *col,
                        int32_t source, uint32_t *dist);

/* Lonestar SSSP drelax2 (sssp.cl:104-318): worklist Bellman-Ford with
 * atomic_min relaxations.  Returns the iteration count. */
int oracle_lonestar_sssp(int32_t V, const int32_t *row_ptr, const int32_t *col,
                         const uint32_t *wt, int32_t source, uint32_t *dist);

/* Pannotia color_combined (pannotia/graph_apps/color/device/color.cl:3-97).
 * color[] is written in full (initialised to -1 as color.h:50 does).
 * Returns the number of rounds (the final graph_color). */
int oracle_pannotia_color(int32_t V, const int32_t *row_ptr,
                          const int32_t *col, const float *node_value,
                          int32_t *color);

/* Pannotia mis_combined (pannotia/graph_apps/mis/device/mis.cl:5-125).
 * s_array[] gets 2 for members and 0 otherwise (mis.h:60-63). Returns rounds. */
int oracle_pannotia_mis(int32_t V, const int32_t *row_ptr, const int32_t *col,
                        const float *node_value, int32_t *s_array);

/* Pannotia sssp_combined (pannotia/graph_apps/sssp/device/sssp.cl:10-88):
 * Jacobi min-plus iteration to a fixpoint. cost[] is the x vector the host
 * reads back (sssp.h:166-170). Returns rounds. */
int oracle_pannotia_sssp(int32_t V, const int32_t *row_ptr, const int32_t *col,
                         const int32_t *data, int32_t source, int32_t *cost);

/* PageRank has no reference implementation.  FP64 pull PageRank written from
 * the definition: pr0 = 1/V; pr' = (1-d)/V + d*(sum_{u->v} pr[u]/deg(u) +
 * dangling/V), dangling = sum of pr over zero-degree vertices. */
void oracle_pagerank_f64(int32_t V, const int32_t *row_ptr, const int32_t *col,
                         double damping, int iterations, double *pr);

/* Same recurrence in FP32 with OpenMP (the timed CPU baseline). */
void oracle_pagerank_f32_omp(int32_t V, const int32_t *row_ptr,
                             const int32_t *col, float damping, int iterations,
                             float *pr, float *scratch);

/* OpenMP level-synchronous variants (timed CPU baseline; same outputs). */
int oracle_lonestar_bfs_omp(int32_t V, const int32_t *row_ptr,
                            const int32_t *col, int32_t source, uint32_t *dist,
                            int32_t *scratch /* 2*V */);
int oracle_lonestar_sssp_omp(int32_t V, const int32_t *row_ptr,
                             const int32_t *col, const uint32_t *wt,
                             int32_t source, uint32_t *dist,
                             int32_t *scratch /* 3*V */);
int oracle_pannotia_color_omp(int32_t V, const int32_t *row_ptr,
                              const int32_t *col, const float *node_value,
                              int32_t *color, float *max_d);
/* oracle_pannotia_mis plus its work: work[0] = edges scanned by the
 * minimum phase summed over rounds, work[1] = active vertices summed over
 * rounds. */
int oracle_pannotia_mis_work(int32_t V, const int32_t *row_ptr, const int32_t *col,
                             const float *node_value, int32_t *s_array, int64_t *work);
int oracle_pannotia_mis_omp(int32_t V, const int32_t *row_ptr,
                            const int32_t *col, const float *node_value,
                            int32_t *s_array, int32_t *scratch /* 2*V */,
                            float *min_array);

/* Non-persistent tasks. */
/* matmult.h:107-119 middle-square fill; returns the updated seed. */
int32_t oracle_matmult_rand_fill(int32_t *M, int32_t rows, int32_t cols,
                                 int32_t seed);
/* matmult.cl:26-56 C = A*B with wrapping int32 arithmetic. */
void oracle_matmult_i32(const int32_t *A, int32_t A_row, int32_t A_col,
                        const int32_t *B, int32_t B_col, int32_t *C);
/* matmult.cl:9-22 djb2 hash of the diagonal (wrapping int32). */
int32_t oracle_hash_diag(const int32_t *M, int32_t rows, int32_t cols);
/* reduce.cl:3-39 min over the buffer. */
int32_t oracle_reduce_min_i32(const int32_t *buf, int64_t n);
/* FP32 variants of the tasks (no reference counterpart). */
void oracle_matmult_f32(const float *A, int32_t M, int32_t K, const float *B,
                        int32_t N, float *C);
float oracle_reduce_min_f32(const float *buf, int64_t n);

/* Batched CPU baseline: njobs Lonestar BFS (algo 0) / SSSP (algo 1) jobs,
 * spread over the OpenMP threads (dynamic schedule, in the order given),
 * each job the serial restatement above.  Job k reads graph rows at
 * rows + row_off[k] (V[k]+1 entries), cols/wts at col_off[k], writes
 * dist + dist_off[k]. */
void oracle_batch_lonestar(int32_t njobs, const int32_t *V, const int64_t *row_off,
                           const int64_t *col_off, const int64_t *dist_off,
                           const int32_t *algo, const int32_t *source, const int32_t *rows,
                           const int32_t *cols, const uint32_t *wts, uint32_t *dist);

int oracle_omp_threads(void);

/* connect four (test_suite/connect_four/device/connect_four.cl): the value
 * of each of the 7 first moves from a 42-cell board (0 empty, 1 human, 2
 * computer), maxlevel moves of look-ahead (1..7).  Returns 0, or -1. */
int oracle_connect_four(const uint8_t *board, int32_t maxlevel, int32_t *next_move_value);

/* Pannotia betweenness centrality (bc.cl) in double precision, sources
 * 0 .. num_sources-1.  Returns 0, or -1 when memory runs out. */
int oracle_pannotia_bc_f64(int32_t V, const int32_t *row, const int32_t *col,
                           int32_t num_sources, double *bc);

/* Seeded synthetic graphs (oracle_inputs.c): a rows x cols grid (row_ptr
 * V+1, col oracle_grid_edges(rows, cols)), and an RMAT graph whose arrays are
 * allocated here and released with oracle_free. */
int64_t oracle_grid_edges(int32_t rows, int32_t cols);
int oracle_gen_grid(int32_t rows, int32_t cols, int32_t *row_ptr, int32_t *col);
int oracle_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c,
                    uint64_t seed, int32_t permute, uint32_t wmin, uint32_t wmax,
                    int32_t **row_ptr_out, int32_t **col_out, uint32_t **w_out,
                    int64_t *num_edges);
void oracle_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
