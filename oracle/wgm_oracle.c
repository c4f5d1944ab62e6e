/*
 * CPU oracle: restatement of the reference's persistent graph kernels and
 * non-persistent tasks.  TEST INFRASTRUCTURE ONLY (see wgm_oracle.h).
 *
 * Each inter-barrier phase of a reference kernel becomes a sequential loop
 * over vertices.  The comment above each loop states why the phase's result
 * does not depend on the order in which the GPU's work-items ran it, which is
 * what makes a sequential restatement a valid oracle for a racy parallel
 * kernel.
 */
#include "wgm_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int oracle_omp_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Vertex degree as the Lonestar kernel computes it: psrc[nn+1]-psrc[nn]
 * (bfs.cl:165).  With the loader quirk an isolated last vertex yields -1; the
 * kernel's gather loop then runs zero times for that vertex, so it is 0 here. */
static inline int32_t lonestar_degree(const int32_t *row_ptr, int32_t v) {
  int32_t d = row_ptr[v + 1] - row_ptr[v];
  return d < 0 ? 0 : d;
}

void oracle_lonestar_csr_from_gr(int64_t V, int64_t E, const uint64_t *out_idx,
                                 const uint32_t *outs, int32_t *row_ptr,
                                 int32_t *col) {
  /* bfs.h:41-43: psrc[nnodes] = nedges; edgessrcdst is 1-based.
   * bfs.h:141-148: psrc[0] = 1, psrc[ii] = outIdx[ii-1] + 1.
   * bfs.h:149-157: edgessrcdst[psrc[ii]+jj] = outs[psrc[ii]+jj-1] for
   * jj < outIdx[ii]-outIdx[ii-1].  In 0-based form the kernel sees
   * row_ptr[ii] = psrc[ii]-1 and col[k] = outs[k]; row_ptr[V] = E-1. */
  for (int64_t i = 0; i < V; i++)
    row_ptr[i] = (i == 0) ? 0 : (int32_t)out_idx[i - 1];
  row_ptr[V] = (int32_t)(E - 1);
  for (int64_t k = 0; k < E; k++) col[k] = (int32_t)outs[k];
}

/* ------------------------------------------------------------------------ */
/* Lonestar BFS: lonestar/graph_apps/bfs/device/bfs.cl                       */
/* ------------------------------------------------------------------------ */

int oracle_lonestar_bfs(int32_t V, const int32_t *row_ptr, const int32_t *col,
                        int32_t source, uint32_t *dist) {
  /* bfs.h:250-262: dist = MYINFINITY everywhere, then dist[source] = 0. */
  for (int32_t i = 0; i < V; i++) dist[i] = ORACLE_LONESTAR_INF;
  if (V <= 0) return 0;
  dist[source] = 0;
  int32_t *in_wl = (int32_t *)malloc(sizeof(int32_t) * (size_t)(V + 1));
  int32_t *out_wl = (int32_t *)malloc(sizeof(int32_t) * (size_t)(V + 1));
  /* bfs.cl:235-241: iteration 0 pushes the source only. */
  int32_t in_n = 1;
  in_wl[0] = source;
  int iteration = 1;
  /* bfs.cl:278-300: while(1) { drelax; barrier; swap; iteration++; barrier;
   * if (*in_index <= 0) break; }.  Phase order independence: a vertex is
   * written only when its dist is MYINFINITY and always with the value
   * `iteration`, so every interleaving of the unsynchronised writes at
   * bfs.cl:121-123 stores the same value; duplicates in the worklist change
   * nothing but the worklist length. */
  while (in_n > 0) {
    int32_t out_n = 0;
    for (int32_t k = 0; k < in_n; k++) {
      int32_t nn = in_wl[k];
      int32_t start = row_ptr[nn], deg = lonestar_degree(row_ptr, nn);
      for (int32_t j = 0; j < deg; j++) {
        uint32_t dst = (uint32_t)col[start + j];
        if (dst >= (uint32_t)V) continue; /* bfs.cl:116 */
        if (dist[dst] == ORACLE_LONESTAR_INF) {
          dist[dst] = (uint32_t)iteration; /* bfs.cl:121-123 */
          out_wl[out_n++] = (int32_t)dst;
        }
      }
    }
    int32_t *t = in_wl;
    in_wl = out_wl;
    out_wl = t;
    in_n = out_n;
    iteration++;
  }
  free(in_wl);
  free(out_wl);
  return iteration;
}

/* ------------------------------------------------------------------------ */
/* Lonestar SSSP: lonestar/graph_apps/sssp/device/sssp.cl                    */
/* ------------------------------------------------------------------------ */

int oracle_lonestar_sssp(int32_t V, const int32_t *row_ptr, const int32_t *col,
                         const uint32_t *wt, int32_t source, uint32_t *dist) {
  for (int32_t i = 0; i < V; i++) dist[i] = ORACLE_LONESTAR_INF;
  if (V <= 0) return 0;
  dist[source] = 0;
  int32_t *in_wl = (int32_t *)malloc(sizeof(int32_t) * (size_t)(V + 1));
  int32_t *out_wl = (int32_t *)malloc(sizeof(int32_t) * (size_t)(V + 1));
  uint8_t *queued = (uint8_t *)calloc((size_t)V, 1);
  int32_t in_n = 1;
  in_wl[0] = source;
  int iteration = 1;
  /* sssp.cl:104-133: altdist = dist[src] + wt; if (altdist < dist[dst])
   * { atomic_min(&dist[dst], altdist); push dst }.  Every decrease of a
   * vertex's distance pushes it, so the loop ends at the fixpoint of the
   * relaxation, which is the unique shortest-path distance vector whatever
   * the order of relaxations.  A vertex queued twice in one round is
   * processed once here: its second visit would relax the same edges with
   * the same distance, a no-op. */
  while (in_n > 0) {
    int32_t out_n = 0;
    for (int32_t k = 0; k < in_n; k++) {
      int32_t nn = in_wl[k];
      int32_t start = row_ptr[nn], deg = lonestar_degree(row_ptr, nn);
      for (int32_t j = 0; j < deg; j++) {
        uint32_t dst = (uint32_t)col[start + j];
        if (dst >= (uint32_t)V) continue;           /* sssp.cl:117 */
        uint32_t w = wt[start + j];
        if (w >= ORACLE_LONESTAR_INF) continue;     /* sssp.cl:120 */
        uint32_t alt = dist[nn] + w;                /* sssp.cl:123 */
        if (alt < dist[dst]) {                      /* sssp.cl:126-129 */
          dist[dst] = alt;
          if (!queued[dst]) {
            queued[dst] = 1;
            out_wl[out_n++] = (int32_t)dst;
          }
        }
      }
    }
    for (int32_t k = 0; k < out_n; k++) queued[out_wl[k]] = 0;
    int32_t *t = in_wl;
    in_wl = out_wl;
    out_wl = t;
    in_n = out_n;
    iteration++;
  }
  free(in_wl);
  free(out_wl);
  free(queued);
  return iteration;
}

/* ------------------------------------------------------------------------ */
/* Pannotia colour: pannotia/graph_apps/color/device/color.cl:3-97           */
/* ------------------------------------------------------------------------ */

int oracle_pannotia_color(int32_t V, const int32_t *row_ptr,
                          const int32_t *col, const float *node_value,
                          int32_t *color) {
  int32_t num_edges = row_ptr[V];
  float *max_d = (float *)malloc(sizeof(float) * (size_t)(V > 0 ? V : 1));
  for (int32_t i = 0; i < V; i++) color[i] = -1; /* color.h:50 */
  int graph_color = 1;
  int stop[2] = {0, 0}; /* stop1, stop2 (color.h:73-76) */
  int w = 0;            /* write_stop = stop1, read_stop = stop2 */
  for (;;) {
    /* Phase color1 (color.cl:27-55).  Reads color[] (not written in this
     * phase) and writes max_d[i] for the vertex's own i: order independent.
     * `start != end - 1` (color.cl:46) skips every neighbour of a degree-1
     * vertex. */
    for (int32_t i = 0; i < V; i++) {
      if (color[i] != -1) continue;
      int32_t start = row_ptr[i];
      int32_t end = (i + 1 < V) ? row_ptr[i + 1] : num_edges;
      float maximum = -1;
      for (int32_t e = start; e < end; e++) {
        if (color[col[e]] == -1 && start != end - 1) {
          stop[w] = 1;
          if (node_value[col[e]] > maximum) maximum = node_value[col[e]];
        }
      }
      max_d[i] = maximum;
    }
    int r = w; /* swap: read_stop = the flag just written (color.cl:59-61) */
    w = 1 - w;
    /* Phase color2 (color.cl:74-83): each i writes only color[i]. */
    for (int32_t i = 0; i < V; i++)
      if (color[i] == -1 && node_value[i] > max_d[i]) color[i] = graph_color;
    if (stop[r] == 0) break; /* color.cl:85-87 */
    graph_color++;
    stop[w] = 0; /* color.cl:90 */
  }
  free(max_d);
  return graph_color;
}

/* ------------------------------------------------------------------------ */
/* Pannotia MIS: pannotia/graph_apps/mis/device/mis.cl:5-125                 */
/* ------------------------------------------------------------------------ */

#define MIS_BIGNUM 99999999 /* mis.cl:1 */

/* work[0] += edges scanned by mis1 (the active vertices' degrees, summed
 * over rounds), work[1] += active vertices summed over rounds: the work
 * units of the MIS bytes/s figure.  NULL: no counting. */
static int mis_impl(int32_t V, const int32_t *row_ptr, const int32_t *col,
                    const float *node_value, int32_t *s_array, int64_t *work) {
  int32_t num_edges = row_ptr[V];
  size_t n = (size_t)(V > 0 ? V : 1);
  int32_t *c = (int32_t *)malloc(sizeof(int32_t) * n);
  int32_t *cu = (int32_t *)malloc(sizeof(int32_t) * n);
  float *min_array = (float *)malloc(sizeof(float) * n);
  /* mis.h:58-92: s = 0, c = cu = -1, min_array = 6666666.0, stop = 0. */
  for (int32_t i = 0; i < V; i++) {
    s_array[i] = 0;
    c[i] = -1;
    cu[i] = -1;
    min_array[i] = 6666666.0f;
  }
  int stop = 0, rounds = 0;
  for (;;) {
    rounds++;
    /* mis1 (mis.cl:29-53): reads c[] (unchanged in this phase), writes
     * min_array[tid] only: order independent. */
    for (int32_t t = 0; t < V; t++) {
      if (c[t] != -1) continue;
      stop = 1;
      int32_t start = row_ptr[t];
      int32_t end = (t + 1 < V) ? row_ptr[t + 1] : num_edges;
      if (work) {
        work[0] += end - start;
        work[1] += 1;
      }
      float mn = (float)MIS_BIGNUM;
      for (int32_t e = start; e < end; e++)
        if (c[col[e]] == -1 && node_value[col[e]] < mn) mn = node_value[col[e]];
      min_array[t] = mn;
    }
    int local_stop = stop; /* mis.cl:59 */
    /* mis2 (mis.cl:66-96).  A vertex joins when its value is below the
     * minimum over its active neighbours; two adjacent active vertices can
     * never both satisfy that, so the c[] writes of joiners never change the
     * c[col] tests another joiner makes (the neighbours it tests are never
     * joiners).  cu[] is only written, with one value.  Order independent. */
    for (int32_t t = 0; t < V; t++) {
      if (node_value[t] < min_array[t] && c[t] == -1) {
        s_array[t] = 2;
        int32_t start = row_ptr[t];
        int32_t end = (t + 1 < V) ? row_ptr[t + 1] : num_edges;
        c[t] = -2;
        for (int32_t e = start; e < end; e++)
          if (c[col[e]] == -1) cu[col[e]] = -2;
      }
    }
    if (local_stop == 0) break; /* mis.cl:106-108 */
    stop = 0;                   /* mis.cl:109 */
    /* mis3 (mis.cl:114-118): own-index writes. */
    for (int32_t t = 0; t < V; t++)
      if (cu[t] == -2) c[t] = cu[t];
  }
  free(c);
  free(cu);
  free(min_array);
  return rounds;
}

int oracle_pannotia_mis(int32_t V, const int32_t *row_ptr, const int32_t *col,
                        const float *node_value, int32_t *s_array) {
  return mis_impl(V, row_ptr, col, node_value, s_array, NULL);
}

int oracle_pannotia_mis_work(int32_t V, const int32_t *row_ptr, const int32_t *col,
                             const float *node_value, int32_t *s_array, int64_t *work) {
  work[0] = work[1] = 0;
  return mis_impl(V, row_ptr, col, node_value, s_array, work);
}

/* ------------------------------------------------------------------------ */
/* Pannotia SSSP: pannotia/graph_apps/sssp/device/sssp.cl:10-88              */
/* ------------------------------------------------------------------------ */

int oracle_pannotia_sssp(int32_t V, const int32_t *row_ptr, const int32_t *col,
                         const int32_t *data, int32_t source, int32_t *cost) {
  size_t n = (size_t)(V > 0 ? V : 1);
  int32_t *y = (int32_t *)malloc(sizeof(int32_t) * n);
  /* sssp.h:58-66: x = y = BIG_NUM except the source. */
  for (int32_t i = 0; i < V; i++)
    cost[i] = y[i] = (i == source) ? 0 : ORACLE_PANNOTIA_BIG;
  int rounds = 0;
  for (;;) {
    rounds++;
    /* vector_assign (sssp.cl:31-33) */
    for (int32_t i = 0; i < V; i++) cost[i] = y[i];
    /* spmv_min_dot_plus (sssp.cl:51-64): reads x, writes y[own]: a Jacobi
     * step, order independent. */
    for (int32_t it = 0; it < V; it++) {
      int32_t mn = cost[it];
      for (int32_t j = row_ptr[it]; j < row_ptr[it + 1]; j++)
        if (data[j] + cost[col[j]] < mn) mn = data[j] + cost[col[j]];
      y[it] = mn;
    }
    /* vector_diff (sssp.cl:77-80) and the exit test (sssp.cl:88-90) */
    int stop = 0;
    for (int32_t i = 0; i < V; i++)
      if (y[i] != cost[i]) stop = 1;
    if (!stop) break;
  }
  free(y);
  return rounds;
}

/* ------------------------------------------------------------------------ */
/* PageRank (no reference implementation)                                    */
/* ------------------------------------------------------------------------ */

void oracle_pagerank_f64(int32_t V, const int32_t *row_ptr, const int32_t *col,
                         double damping, int iterations, double *pr) {
  size_t n = (size_t)(V > 0 ? V : 1);
  double *contrib = (double *)malloc(sizeof(double) * n);
  double *next = (double *)malloc(sizeof(double) * n);
  for (int32_t i = 0; i < V; i++) pr[i] = 1.0 / (double)V;
  for (int it = 0; it < iterations; it++) {
    double dangling = 0.0;
    for (int32_t u = 0; u < V; u++) {
      int32_t d = row_ptr[u + 1] - row_ptr[u];
      if (d > 0) {
        contrib[u] = pr[u] / (double)d;
      } else {
        contrib[u] = 0.0;
        dangling += pr[u];
      }
    }
    double base = (1.0 - damping) / (double)V + damping * dangling / (double)V;
    for (int32_t v = 0; v < V; v++) {
      double s = 0.0;
      for (int32_t j = row_ptr[v]; j < row_ptr[v + 1]; j++) s += contrib[col[j]];
      next[v] = base + damping * s;
    }
    memcpy(pr, next, sizeof(double) * (size_t)V);
  }
  free(contrib);
  free(next);
}

void oracle_pagerank_f32_omp(int32_t V, const int32_t *row_ptr,
                             const int32_t *col, float damping, int iterations,
                             float *pr, float *scratch) {
  float *contrib = scratch;
  float *next = scratch + V;
  for (int32_t i = 0; i < V; i++) pr[i] = 1.0f / (float)V;
  for (int it = 0; it < iterations; it++) {
    double dangling = 0.0;
#pragma omp parallel for reduction(+ : dangling) schedule(static)
    for (int32_t u = 0; u < V; u++) {
      int32_t d = row_ptr[u + 1] - row_ptr[u];
      if (d > 0) {
        contrib[u] = pr[u] / (float)d;
      } else {
        contrib[u] = 0.0f;
        dangling += pr[u];
      }
    }
    float base = (1.0f - damping) / (float)V + damping * (float)dangling / (float)V;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int32_t v = 0; v < V; v++) {
      float s = 0.0f;
      for (int32_t j = row_ptr[v]; j < row_ptr[v + 1]; j++) s += contrib[col[j]];
      next[v] = base + damping * s;
    }
    memcpy(pr, next, sizeof(float) * (size_t)V);
  }
}

/* ------------------------------------------------------------------------ */
/* OpenMP variants (timed CPU baseline); same phase structure                */
/* ------------------------------------------------------------------------ */

int oracle_lonestar_bfs_omp(int32_t V, const int32_t *row_ptr,
                            const int32_t *col, int32_t source, uint32_t *dist,
                            int32_t *scratch) {
#pragma omp parallel for schedule(static)
  for (int32_t i = 0; i < V; i++) dist[i] = ORACLE_LONESTAR_INF;
  if (V <= 0) return 0;
  dist[source] = 0;
  int32_t *in_wl = scratch, *out_wl = scratch + V;
  int32_t in_n = 1, out_n = 0;
  in_wl[0] = source;
  int iteration = 1;
  while (in_n > 0) {
    out_n = 0;
#pragma omp parallel for schedule(dynamic, 64)
    for (int32_t k = 0; k < in_n; k++) {
      int32_t nn = in_wl[k];
      int32_t start = row_ptr[nn], deg = lonestar_degree(row_ptr, nn);
      for (int32_t j = 0; j < deg; j++) {
        uint32_t dst = (uint32_t)col[start + j];
        if (dst >= (uint32_t)V) continue;
        uint32_t expect = ORACLE_LONESTAR_INF;
        if (__atomic_load_n(&dist[dst], __ATOMIC_RELAXED) == expect &&
            __atomic_compare_exchange_n(&dist[dst], &expect, (uint32_t)iteration,
                                        0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
          int32_t slot = __atomic_fetch_add(&out_n, 1, __ATOMIC_RELAXED);
          out_wl[slot] = (int32_t)dst;
        }
      }
    }
    int32_t *t = in_wl;
    in_wl = out_wl;
    out_wl = t;
    in_n = out_n;
    iteration++;
  }
  return iteration;
}

int oracle_lonestar_sssp_omp(int32_t V, const int32_t *row_ptr,
                             const int32_t *col, const uint32_t *wt,
                             int32_t source, uint32_t *dist, int32_t *scratch) {
  int32_t *in_wl = scratch, *out_wl = scratch + V, *stamp = scratch + 2 * (size_t)V;
#pragma omp parallel for schedule(static)
  for (int32_t i = 0; i < V; i++) {
    dist[i] = ORACLE_LONESTAR_INF;
    stamp[i] = 0;
  }
  if (V <= 0) return 0;
  dist[source] = 0;
  int32_t in_n = 1, out_n = 0;
  in_wl[0] = source;
  int iteration = 1;
  while (in_n > 0) {
    out_n = 0;
#pragma omp parallel for schedule(dynamic, 64)
    for (int32_t k = 0; k < in_n; k++) {
      int32_t nn = in_wl[k];
      int32_t start = row_ptr[nn], deg = lonestar_degree(row_ptr, nn);
      uint32_t dsrc = __atomic_load_n(&dist[nn], __ATOMIC_RELAXED);
      for (int32_t j = 0; j < deg; j++) {
        uint32_t dst = (uint32_t)col[start + j];
        if (dst >= (uint32_t)V) continue;
        uint32_t w = wt[start + j];
        if (w >= ORACLE_LONESTAR_INF) continue;
        uint32_t alt = dsrc + w;
        uint32_t cur = __atomic_load_n(&dist[dst], __ATOMIC_RELAXED);
        int lowered = 0;
        while (alt < cur) {
          if (__atomic_compare_exchange_n(&dist[dst], &cur, alt, 1,
                                          __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
            lowered = 1;
            break;
          }
        }
        if (lowered &&
            __atomic_exchange_n(&stamp[dst], iteration, __ATOMIC_RELAXED) != iteration) {
          int32_t slot = __atomic_fetch_add(&out_n, 1, __ATOMIC_RELAXED);
          out_wl[slot] = (int32_t)dst;
        }
      }
    }
    int32_t *t = in_wl;
    in_wl = out_wl;
    out_wl = t;
    in_n = out_n;
    iteration++;
  }
  return iteration;
}

int oracle_pannotia_color_omp(int32_t V, const int32_t *row_ptr,
                              const int32_t *col, const float *node_value,
                              int32_t *color, float *max_d) {
  int32_t num_edges = row_ptr[V];
#pragma omp parallel for schedule(static)
  for (int32_t i = 0; i < V; i++) color[i] = -1;
  int graph_color = 1;
  for (;;) {
    int stop = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : stop)
    for (int32_t i = 0; i < V; i++) {
      if (color[i] != -1) continue;
      int32_t start = row_ptr[i];
      int32_t end = (i + 1 < V) ? row_ptr[i + 1] : num_edges;
      float maximum = -1;
      for (int32_t e = start; e < end; e++) {
        if (color[col[e]] == -1 && start != end - 1) {
          stop = 1;
          if (node_value[col[e]] > maximum) maximum = node_value[col[e]];
        }
      }
      max_d[i] = maximum;
    }
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < V; i++)
      if (color[i] == -1 && node_value[i] > max_d[i]) color[i] = graph_color;
    if (!stop) break;
    graph_color++;
  }
  return graph_color;
}

int oracle_pannotia_mis_omp(int32_t V, const int32_t *row_ptr,
                            const int32_t *col, const float *node_value,
                            int32_t *s_array, int32_t *scratch,
                            float *min_array) {
  int32_t num_edges = row_ptr[V];
  int32_t *c = scratch, *cu = scratch + V;
#pragma omp parallel for schedule(static)
  for (int32_t i = 0; i < V; i++) {
    s_array[i] = 0;
    c[i] = -1;
    cu[i] = -1;
    min_array[i] = 6666666.0f;
  }
  int rounds = 0;
  for (;;) {
    rounds++;
    int stop = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : stop)
    for (int32_t t = 0; t < V; t++) {
      if (c[t] != -1) continue;
      stop = 1;
      int32_t start = row_ptr[t];
      int32_t end = (t + 1 < V) ? row_ptr[t + 1] : num_edges;
      float mn = (float)MIS_BIGNUM;
      for (int32_t e = start; e < end; e++)
        if (c[col[e]] == -1 && node_value[col[e]] < mn) mn = node_value[col[e]];
      min_array[t] = mn;
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (int32_t t = 0; t < V; t++) {
      if (node_value[t] < min_array[t] && c[t] == -1) {
        s_array[t] = 2;
        int32_t start = row_ptr[t];
        int32_t end = (t + 1 < V) ? row_ptr[t + 1] : num_edges;
        __atomic_store_n(&c[t], -2, __ATOMIC_RELAXED);
        for (int32_t e = start; e < end; e++)
          if (__atomic_load_n(&c[col[e]], __ATOMIC_RELAXED) == -1)
            __atomic_store_n(&cu[col[e]], -2, __ATOMIC_RELAXED);
      }
    }
    if (!stop) break;
#pragma omp parallel for schedule(static)
    for (int32_t t = 0; t < V; t++)
      if (cu[t] == -2) c[t] = cu[t];
  }
  return rounds;
}

/* ------------------------------------------------------------------------ */
/* Non-persistent tasks                                                      */
/* ------------------------------------------------------------------------ */

int32_t oracle_matmult_rand_fill(int32_t *M, int32_t rows, int32_t cols,
                                 int32_t seed) {
  /* matmult.h:107-119: middle-square; `seed * seed` wraps as 32-bit. */
  for (int32_t r = 0; r < rows; r++) {
    for (int32_t c = 0; c < cols; c++) {
      seed = (int32_t)((uint32_t)seed * (uint32_t)seed);
      seed = (seed / 1000) % 1000000;
      M[(int64_t)r * cols + c] = seed % 10;
    }
  }
  return seed;
}

void oracle_matmult_i32(const int32_t *A, int32_t A_row, int32_t A_col,
                        const int32_t *B, int32_t B_col, int32_t *C) {
  /* matmult.cl:48-56 (row-major, wrapping int32 accumulation). */
  for (int32_t r = 0; r < A_row; r++)
    for (int32_t c = 0; c < B_col; c++) {
      uint32_t acc = 0;
      for (int32_t j = 0; j < A_col; j++)
        acc += (uint32_t)A[(int64_t)r * A_col + j] * (uint32_t)B[(int64_t)j * B_col + c];
      C[(int64_t)r * B_col + c] = (int32_t)acc;
    }
}

int32_t oracle_hash_diag(const int32_t *M, int32_t rows, int32_t cols) {
  /* matmult.cl:9-22: djb2 over the diagonal, wrapping int32. */
  uint32_t h = 5381;
  for (int32_t i = 0; i < rows && i < cols; i++)
    h = h * 33u + (uint32_t)M[(int64_t)i * cols + i];
  return (int32_t)h;
}

int32_t oracle_reduce_min_i32(const int32_t *buf, int64_t n) {
  int32_t m = INT_MAX; /* reduce.cl:291: INT_MAX is the identity */
  for (int64_t i = 0; i < n; i++)
    if (buf[i] < m) m = buf[i];
  return m;
}

void oracle_matmult_f32(const float *A, int32_t M, int32_t K, const float *B,
                        int32_t N, float *C) {
  for (int32_t r = 0; r < M; r++)
    for (int32_t c = 0; c < N; c++) {
      double acc = 0.0;
      for (int32_t j = 0; j < K; j++)
        acc += (double)A[(int64_t)r * K + j] * (double)B[(int64_t)j * N + c];
      C[(int64_t)r * N + c] = (float)acc;
    }
}

float oracle_reduce_min_f32(const float *buf, int64_t n) {
  float m = FLT_MAX;
  for (int64_t i = 0; i < n; i++)
    if (buf[i] < m) m = buf[i];
  return m;
}

void oracle_batch_lonestar(int32_t njobs, const int32_t *V, const int64_t *row_off,
                           const int64_t *col_off, const int64_t *dist_off,
                           const int32_t *algo, const int32_t *source, const int32_t *rows,
                           const int32_t *cols, const uint32_t *wts, uint32_t *dist) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int32_t k = 0; k < njobs; k++) {
    const int32_t *rp = rows + row_off[k];
    const int32_t *cl = cols + col_off[k];
    uint32_t *d = dist + dist_off[k];
    if (algo[k] == 0)
      oracle_lonestar_bfs(V[k], rp, cl, source[k], d);
    else
      oracle_lonestar_sssp(V[k], rp, cl, wts + col_off[k], source[k], d);
  }
}

/* ---- connect four (src/test_suite/connect_four/device/connect_four.cl) ---- */

/* chain_value (connect_four.cl:70-80): 2 = computer, 1 = human, 0 empty. */
static void c4_chain(int *v, int player, int chain) {
  if (player != 0) {
    if (chain >= 4)
      *v = player == 2 ? 666 : -666;
    else if (chain >= 2)
      *v += player == 2 ? 1 : -1;
  }
}

/* scan_board (connect_four.cl:84-130). */
static int c4_scan(const uint8_t *b, int row, int col, int dr, int dc) {
  int res = 0, player = 0, chain = 0;
  do {
    int cell = b[row * 7 + col];
    if (cell == player) {
      chain++;
    } else {
      c4_chain(&res, player, chain);
      if (res == 666 || res == -666) return res;
      player = cell;
      chain = 1;
    }
    row += dr;
    col += dc;
  } while (0 <= row && row < 6 && 0 <= col && col < 7);
  c4_chain(&res, player, chain);
  return res;
}

/* board_value with one work-item per line (work-groups of 25 or more
 * items, connect_four.cl:135-176) and the master's reduction in item order
 * (connect_four.cl:433-441): the first +-666 wins, else the sum. */
static int c4_board_value(const uint8_t *b) {
  int value = 0;
  for (int i = 0; i < 25; i++) {
    int t;
    if (i < 6)
      t = c4_scan(b, i, 0, 0, 1);
    else if (i < 13)
      t = c4_scan(b, 0, i - 6, 1, 0);
    else if (i < 19)
      t = (i - 13) < 3 ? c4_scan(b, i - 13, 0, 1, 1) : c4_scan(b, 0, i - 13 - 2, 1, 1);
    else
      t = (i - 19) < 3 ? c4_scan(b, i - 19, 6, 1, -1) : c4_scan(b, 0, i - 19, 1, -1);
    if (t == 666 || t == -666) return t;
    value += t;
  }
  return value;
}

/* update_board (connect_four.cl:180-220): the computer moves first; a move
 * into a full column is skipped and does not change the player. */
static void c4_replay(const uint8_t *base, const uint8_t *moves, int level, uint8_t *b) {
  memcpy(b, base, 42);
  int player = 2;
  for (int i = 0; i < level; i++) {
    int col = moves[i];
    if (b[col] != 0) continue;
    int row = 0;
    while (row < 6 && b[row * 7 + col] == 0) row++;
    b[(row - 1) * 7 + col] = (uint8_t)player;
    player = player == 2 ? 1 : 2;
  }
}

/* A node's final value (connect_four.cl:443-485 with wgm_update_parent,
 * :305-340): its own board value, then, unless it is a leaf (maxlevel or a
 * +-666 score), combined with its 7 children's - min at an even level, max
 * at an odd one. */
static int c4_node(const uint8_t *base, uint8_t *moves, int level, int maxlevel) {
  uint8_t b[42];
  c4_replay(base, moves, level, b);
  int v = c4_board_value(b);
  if (level >= maxlevel || v == 666 || v == -666) return v;
  int acc = v;
  for (int i = 0; i < 7; i++) {
    moves[level] = (uint8_t)i;
    int c = c4_node(base, moves, level + 1, maxlevel);
    if (level % 2 == 0)
      acc = c < acc ? c : acc;
    else
      acc = c > acc ? c : acc;
  }
  return acc;
}

/* next_move_value[7] of the look-ahead from `board` (connect_four.h:336-351). */
int oracle_connect_four(const uint8_t *board, int32_t maxlevel, int32_t *next_move_value) {
  if (maxlevel < 1 || maxlevel > 7) return -1;
#pragma omp parallel for schedule(dynamic, 1)
  for (int r = 0; r < 7; r++) {
    uint8_t moves[8] = {0};
    moves[0] = (uint8_t)r;
    next_move_value[r] = c4_node(board, moves, 1, maxlevel);
  }
  return 0;
}

/* ---- Pannotia betweenness centrality (pannotia/graph_apps/bc/device/bc.cl) ---- */

/* bc_combined in double precision: for every source s < num_sources a BFS
 * over out-edges counting shortest paths (rho), then levels in reverse:
 * every vertex i at level L adds rho[w]/rho[i] * (1 + sigma[i]) to sigma[w]
 * of each in-neighbour w at level L-1 (bc.cl:122-124) and, unless it is s,
 * sigma[i] to bc[i] (bc.cl:131).  The reference's factor 10000 on rho and
 * sigma cancels.  The GPU computes in float; tests compare within a
 * stated tolerance. */
int oracle_pannotia_bc_f64(int32_t V, const int32_t *row, const int32_t *col,
                           int32_t num_sources, double *bc) {
  const int64_t E = row[V];
  int32_t *trow = calloc((size_t)V + 1, sizeof(int32_t));
  int32_t *tcol = malloc(sizeof(int32_t) * (size_t)(E > 0 ? E : 1));
  int32_t *fill = malloc(sizeof(int32_t) * (size_t)V + 4);
  int32_t *dist = malloc(sizeof(int32_t) * (size_t)V + 4);
  int32_t *order = malloc(sizeof(int32_t) * (size_t)V + 4);
  double *rho = malloc(sizeof(double) * (size_t)V + 8);
  double *sigma = malloc(sizeof(double) * (size_t)V + 8);
  if (!trow || !tcol || !fill || !dist || !order || !rho || !sigma) return -1;
  for (int64_t e = 0; e < E; e++) trow[col[e] + 1]++;
  for (int32_t v = 0; v < V; v++) trow[v + 1] += trow[v];
  for (int32_t v = 0; v < V; v++) fill[v] = trow[v];
  for (int32_t v = 0; v < V; v++)
    for (int32_t e = row[v]; e < row[v + 1]; e++) tcol[fill[col[e]]++] = v;
  for (int32_t v = 0; v < V; v++) bc[v] = 0.0;
  for (int32_t s = 0; s < num_sources && s < V; s++) {
    for (int32_t v = 0; v < V; v++) {
      dist[v] = -1;
      rho[v] = 0.0;
      sigma[v] = 0.0;
    }
    dist[s] = 0;
    rho[s] = 1.0;
    int32_t head = 0, tail = 0;
    order[tail++] = s;
    while (head < tail) {
      const int32_t i = order[head++];
      for (int32_t e = row[i]; e < row[i + 1]; e++) {
        const int32_t w = col[e];
        if (dist[w] < 0) {
          dist[w] = dist[i] + 1;
          order[tail++] = w;
        }
        if (dist[w] == dist[i] + 1) rho[w] += rho[i];
      }
    }
    for (int32_t k = tail - 1; k >= 0; k--) {
      const int32_t i = order[k];
      for (int32_t e = trow[i]; e < trow[i + 1]; e++) {
        const int32_t w = tcol[e];
        if (dist[w] == dist[i] - 1) sigma[w] += rho[w] / rho[i] * (1.0 + sigma[i]);
      }
      if (i != s) bc[i] += sigma[i];
    }
  }
  free(trow);
  free(tcol);
  free(fill);
  free(dist);
  free(order);
  free(rho);
  free(sigma);
  return 0;
}
