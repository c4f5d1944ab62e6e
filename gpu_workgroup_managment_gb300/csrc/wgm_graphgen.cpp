/*
 * Seeded synthetic graphs (include/wgm.h "synthetic inputs").
 *
 * The reference reads its graphs from files (Galois .gr, Metis, DIMACS) that
 * are not distributed with it; these generators produce the graph families
 * its benchmarks name, deterministically from a seed and independent of the
 * number of host threads (every random draw is a SplitMix64 function of
 * (seed, sample index)).
 */
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/wgm.h"

struct wgm_host_graph {
  int32_t V = 0;
  int64_t E = 0;
  std::vector<int32_t> row_ptr, col;
  std::vector<uint32_t> weights;
};

static inline uint64_t wgm_splitmix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

extern "C" int wgm_gen_grid(int32_t rows, int32_t cols, int32_t *row_ptr, int32_t *col,
                            int64_t *num_edges) {
  if (rows < 1 || cols < 1 || !row_ptr || (int64_t)rows * cols > INT32_MAX) return WGM_ERR_INVALID;
  int64_t k = 0;
  for (int32_t r = 0; r < rows; r++) {
    for (int32_t c = 0; c < cols; c++) {
      int32_t v = r * cols + c;
      row_ptr[v] = (int32_t)k;
      /* neighbours in (up, left, right, down) order: ascending ids */
      if (r > 0) {
        if (col) col[k] = v - cols;
        k++;
      }
      if (c > 0) {
        if (col) col[k] = v - 1;
        k++;
      }
      if (c + 1 < cols) {
        if (col) col[k] = v + 1;
        k++;
      }
      if (r + 1 < rows) {
        if (col) col[k] = v + cols;
        k++;
      }
    }
  }
  row_ptr[(int64_t)rows * cols] = (int32_t)k;
  if (num_edges) *num_edges = k;
  return WGM_OK;
}

static inline uint32_t wgm_edge_weight(uint32_t u, uint32_t v, uint64_t seed, uint32_t wmin,
                                       uint32_t wmax) {
  uint32_t lo = u < v ? u : v, hi = u < v ? v : u;
  uint64_t h = wgm_splitmix64(seed ^ 0x5bd1e9955bd1e995ull ^ (((uint64_t)lo << 32) | hi));
  return wmin + (uint32_t)(h % (uint64_t)(wmax - wmin + 1));
}

extern "C" int wgm_gen_rmat(int scale, int edge_factor, double a, double b, double c,
                            uint64_t seed, int permute, uint32_t wmin, uint32_t wmax,
                            wgm_host_graph **out) {
  if (!out || scale < 1 || scale > 26 || edge_factor < 1 || a < 0 || b < 0 || c < 0 ||
      a + b + c > 1.0 || (wmax > 0 && wmin > wmax))
    return WGM_ERR_INVALID;
  *out = nullptr;
  const int64_t V = (int64_t)1 << scale;
  const int64_t M = V * edge_factor;
  wgm_host_graph *g = new (std::nothrow) wgm_host_graph();
  if (!g) return WGM_ERR_OOM;
  try {
    std::vector<int32_t> src(M), dst(M);
    const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; i++) {
      uint64_t st = wgm_splitmix64(seed * 0x9e3779b97f4a7c15ull + (uint64_t)i);
      uint32_t u = 0, v = 0;
      for (int l = 0; l < scale; l++) {
        st = wgm_splitmix64(st);
        double r = (double)(st >> 11) * (1.0 / 9007199254740992.0);
        uint32_t bu = 0, bv = 0;
        if (r < a) {
        } else if (r < ab) {
          bv = 1;
        } else if (r < abc) {
          bu = 1;
        } else {
          bu = 1;
          bv = 1;
        }
        u = (u << 1) | bu;
        v = (v << 1) | bv;
      }
      src[i] = (int32_t)u;
      dst[i] = (int32_t)v;
    }
    if (permute) {
      /* Seeded relabelling (Fisher-Yates), so hubs are not clustered at low ids. */
      std::vector<int32_t> perm(V);
      for (int64_t i = 0; i < V; i++) perm[i] = (int32_t)i;
      uint64_t st = wgm_splitmix64(seed ^ 0xa0761d6478bd642full);
      for (int64_t i = V - 1; i > 0; i--) {
        st = wgm_splitmix64(st);
        int64_t j = (int64_t)(st % (uint64_t)(i + 1));
        std::swap(perm[i], perm[j]);
      }
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < M; i++) {
        src[i] = perm[src[i]];
        dst[i] = perm[dst[i]];
      }
    }
    /* Symmetrise (both directions), drop self loops. */
    std::vector<int64_t> deg(V + 1, 0);
    for (int64_t i = 0; i < M; i++) {
      if (src[i] == dst[i]) continue;
      deg[src[i]]++;
      deg[dst[i]]++;
    }
    std::vector<int64_t> start(V + 1, 0);
    for (int64_t v = 0; v < V; v++) start[v + 1] = start[v] + deg[v];
    std::vector<int32_t> tmp(start[V]);
    std::vector<int64_t> cur(start.begin(), start.end() - 1);
    for (int64_t i = 0; i < M; i++) {
      int32_t u = src[i], v = dst[i];
      if (u == v) continue;
      tmp[cur[u]++] = v;
      tmp[cur[v]++] = u;
    }
    src.clear();
    src.shrink_to_fit();
    dst.clear();
    dst.shrink_to_fit();
    /* Sort each row and drop duplicates. */
    std::vector<int64_t> ucount(V, 0);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < V; v++) {
      int32_t *b0 = tmp.data() + start[v], *e0 = tmp.data() + start[v + 1];
      std::sort(b0, e0);
      ucount[v] = std::unique(b0, e0) - b0;
    }
    g->V = (int32_t)V;
    g->row_ptr.assign(V + 1, 0);
    int64_t acc = 0;
    for (int64_t v = 0; v < V; v++) {
      g->row_ptr[v] = (int32_t)acc;
      acc += ucount[v];
    }
    if (acc >= INT32_MAX) {
      delete g;
      return WGM_ERR_INVALID;
    }
    g->row_ptr[V] = (int32_t)acc;
    g->E = acc;
    g->col.resize(acc);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t v = 0; v < V; v++)
      std::memcpy(g->col.data() + g->row_ptr[v], tmp.data() + start[v], ucount[v] * 4);
    if (wmax > 0) {
      g->weights.resize(acc);
#pragma omp parallel for schedule(dynamic, 1024)
      for (int64_t v = 0; v < V; v++)
        for (int64_t k = g->row_ptr[v]; k < g->row_ptr[v + 1]; k++)
          g->weights[k] = wgm_edge_weight((uint32_t)v, (uint32_t)g->col[k], seed, wmin, wmax);
    }
  } catch (const std::bad_alloc &) {
    delete g;
    return WGM_ERR_OOM;
  }
  *out = g;
  return WGM_OK;
}

extern "C" int wgm_host_graph_info(const wgm_host_graph *g, int32_t *num_nodes,
                                   int64_t *num_edges) {
  if (!g) return WGM_ERR_INVALID;
  if (num_nodes) *num_nodes = g->V;
  if (num_edges) *num_edges = g->E;
  return WGM_OK;
}

extern "C" int wgm_host_graph_arrays(const wgm_host_graph *g, const int32_t **row_ptr,
                                     const int32_t **col, const uint32_t **weights) {
  if (!g) return WGM_ERR_INVALID;
  if (row_ptr) *row_ptr = g->row_ptr.data();
  if (col) *col = g->col.data();
  if (weights) *weights = g->weights.empty() ? nullptr : g->weights.data();
  return WGM_OK;
}

extern "C" void wgm_host_graph_free(wgm_host_graph *g) { delete g; }
