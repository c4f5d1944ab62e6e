/*
 * Seeded synthetic graphs for the CPU arms.  TEST INFRASTRUCTURE ONLY (see
 * wgm_oracle.h): the CPU baseline and bench.py's reference arm build their
 * inputs with these functions, so they never load the product library.
 *
 * The graphs are defined by their seeds, not by a file (the reference reads
 * Galois .gr / Metis / DIMACS files that are not distributed with it):
 *
 *  - grid: rows x cols, node r*cols+c, neighbours in (up, left, right, down)
 *    order, which is ascending id order;
 *  - RMAT(scale, edge_factor, a, b, c, seed): sample i of V*edge_factor
 *    starts a SplitMix64 stream at splitmix(seed * 0x9e3779b97f4a7c15 + i);
 *    each of `scale` levels draws r = next() >> 11 scaled to [0, 1) and picks
 *    the quadrant (r < a: none, < a+b: column bit, < a+b+c: row bit, else
 *    both), most significant bit first.  An optional seeded relabelling is a
 *    Fisher-Yates shuffle from splitmix(seed ^ 0xa0761d6478bd642f), i from
 *    V-1 down to 1 swapping with next() % (i+1).  Both directions of every
 *    non-loop sample are kept, each row sorted, duplicates dropped;
 *  - edge weight of {u, v}: wmin + splitmix(seed ^ 0x5bd1e9955bd1e995 ^
 *    (min << 32 | max)) % (wmax - wmin + 1), the same for both directions.
 *
 * The product's generators implement the same definitions; a CPU test
 * checks that both give identical arrays.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline uint64_t oi_mix(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

/* Edge count of a rows x cols grid. */
int64_t oracle_grid_edges(int32_t rows, int32_t cols) {
  if (rows < 1 || cols < 1) return -1;
  return 4 * (int64_t)rows * cols - 2 * (int64_t)rows - 2 * (int64_t)cols;
}

int oracle_gen_grid(int32_t rows, int32_t cols, int32_t *row_ptr, int32_t *col) {
  if (rows < 1 || cols < 1 || !row_ptr || !col) return -1;
  const int64_t V = (int64_t)rows * cols;
  if (V >= INT32_MAX) return -1;
  /* Degrees first, then every row in ascending id order. */
  row_ptr[0] = 0;
  for (int64_t v = 0; v < V; v++) {
    const int32_t r = (int32_t)(v / cols), c = (int32_t)(v % cols);
    const int32_t d = (r > 0) + (c > 0) + (c + 1 < cols) + (r + 1 < rows);
    row_ptr[v + 1] = row_ptr[v] + d;
  }
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < V; v++) {
    const int32_t r = (int32_t)(v / cols), c = (int32_t)(v % cols);
    int32_t *o = col + row_ptr[v];
    if (r > 0) *o++ = (int32_t)(v - cols);
    if (c > 0) *o++ = (int32_t)(v - 1);
    if (c + 1 < cols) *o++ = (int32_t)(v + 1);
    if (r + 1 < rows) *o++ = (int32_t)(v + cols);
  }
  return 0;
}

static int oi_cmp_i32(const void *x, const void *y) {
  const int32_t a = *(const int32_t *)x, b = *(const int32_t *)y;
  return (a > b) - (a < b);
}

/* An RMAT graph as above.  *row_ptr_out (V+1), *col_out (E) and, when wmax
 * > 0, *w_out (E) are malloc'ed here and freed with oracle_free. */
int oracle_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c,
                    uint64_t seed, int32_t permute, uint32_t wmin, uint32_t wmax,
                    int32_t **row_ptr_out, int32_t **col_out, uint32_t **w_out,
                    int64_t *num_edges) {
  if (scale < 1 || scale > 26 || edge_factor < 1 || !row_ptr_out || !col_out || !num_edges)
    return -1;
  const int64_t V = (int64_t)1 << scale, M = V * edge_factor;
  int32_t *eu = (int32_t *)malloc((size_t)M * 4), *ev = (int32_t *)malloc((size_t)M * 4);
  int64_t *beg = (int64_t *)calloc((size_t)V + 1, 8);
  int32_t *perm = permute ? (int32_t *)malloc((size_t)V * 4) : NULL;
  int rc = -1;
  int32_t *adj = NULL, *rp = NULL, *cl = NULL;
  uint32_t *wt = NULL;
  int64_t *fill = NULL, *kept = NULL;
  if (!eu || !ev || !beg || (permute && !perm)) goto out;
  const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < M; i++) {
    uint64_t s = oi_mix(seed * 0x9e3779b97f4a7c15ull + (uint64_t)i);
    uint32_t u = 0, v = 0;
    for (int l = 0; l < scale; l++) {
      s = oi_mix(s);
      const double r = (double)(s >> 11) * 0x1.0p-53;
      const uint32_t ru = r >= ab, rv = (r >= a && r < ab) || r >= abc;
      u = u << 1 | ru;
      v = v << 1 | rv;
    }
    eu[i] = (int32_t)u;
    ev[i] = (int32_t)v;
  }
  if (permute) {
    for (int64_t i = 0; i < V; i++) perm[i] = (int32_t)i;
    uint64_t s = oi_mix(seed ^ 0xa0761d6478bd642full);
    for (int64_t i = V - 1; i > 0; i--) {
      s = oi_mix(s);
      const int64_t j = (int64_t)(s % (uint64_t)(i + 1));
      const int32_t t = perm[i];
      perm[i] = perm[j];
      perm[j] = t;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; i++) {
      eu[i] = perm[eu[i]];
      ev[i] = perm[ev[i]];
    }
  }
  /* Both directions of every non-loop sample, bucketed by source. */
  for (int64_t i = 0; i < M; i++)
    if (eu[i] != ev[i]) {
      beg[eu[i] + 1]++;
      beg[ev[i] + 1]++;
    }
  for (int64_t v = 0; v < V; v++) beg[v + 1] += beg[v];
  adj = (int32_t *)malloc((size_t)(beg[V] > 0 ? beg[V] : 1) * 4);
  fill = (int64_t *)malloc((size_t)V * 8);
  kept = (int64_t *)malloc((size_t)V * 8);
  rp = (int32_t *)malloc((size_t)(V + 1) * 4);
  if (!adj || !fill || !kept || !rp) goto out;
  memcpy(fill, beg, (size_t)V * 8);
  for (int64_t i = 0; i < M; i++)
    if (eu[i] != ev[i]) {
      adj[fill[eu[i]]++] = ev[i];
      adj[fill[ev[i]]++] = eu[i];
    }
  free(eu);
  free(ev);
  eu = ev = NULL;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t v = 0; v < V; v++) {
    int32_t *row = adj + beg[v];
    const int64_t n = beg[v + 1] - beg[v];
    qsort(row, (size_t)n, 4, oi_cmp_i32);
    int64_t k = 0;
    for (int64_t j = 0; j < n; j++)
      if (k == 0 || row[j] != row[k - 1]) row[k++] = row[j];
    kept[v] = k;
  }
  int64_t E = 0;
  for (int64_t v = 0; v < V; v++) {
    rp[v] = (int32_t)E;
    E += kept[v];
  }
  if (E >= INT32_MAX) goto out;
  rp[V] = (int32_t)E;
  cl = (int32_t *)malloc((size_t)(E > 0 ? E : 1) * 4);
  if (!cl) goto out;
  if (wmax > 0) {
    wt = (uint32_t *)malloc((size_t)(E > 0 ? E : 1) * 4);
    if (!wt) goto out;
  }
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t v = 0; v < V; v++) {
    memcpy(cl + rp[v], adj + beg[v], (size_t)kept[v] * 4);
    if (wt)
      for (int64_t k = rp[v]; k < rp[v + 1]; k++) {
        const uint64_t lo = (uint64_t)(v < cl[k] ? v : cl[k]);
        const uint64_t hi = (uint64_t)(v < cl[k] ? cl[k] : v);
        wt[k] = wmin + (uint32_t)(oi_mix(seed ^ 0x5bd1e9955bd1e995ull ^ (lo << 32 | hi)) %
                                  (uint64_t)(wmax - wmin + 1));
      }
  }
  *row_ptr_out = rp;
  *col_out = cl;
  if (w_out) *w_out = wt;
  else free(wt);
  *num_edges = E;
  rp = NULL;
  cl = NULL;
  wt = NULL;
  rc = 0;
out:
  free(eu);
  free(ev);
  free(beg);
  free(perm);
  free(adj);
  free(fill);
  free(kept);
  free(rp);
  free(cl);
  free(wt);
  return rc;
}

void oracle_free(void *p) { free(p); }
