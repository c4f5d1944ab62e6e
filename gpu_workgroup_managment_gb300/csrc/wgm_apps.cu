/*
 * Persistent app plugins of libwgm (include/wgm.h "persistent app plugins").
 *
 * One wgm_app owns the device buffers of one persistent task, the way the
 * reference's per-app plugin headers own their cl::Buffers
 * (lonestar/graph_apps/bfs/bfs.h:23-30, pannotia/graph_apps/color/color.h:16-21,
 * pannotia/graph_apps/mis/mis.h:14-20, pannotia/graph_apps/sssp/sssp.h:16-21).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/wgm.h"
#include "wgm_internal.h"
#include "wgm_kernels.cuh"
#include "wgm_mega.cuh"

int wgm_kind_to_kernel(int kind) {
  switch (kind) {
    case WGM_APP_LONESTAR_BFS: return WGM_K_BFS;
    case WGM_APP_LONESTAR_SSSP: return WGM_K_SSSP;
    case WGM_APP_PANNOTIA_COLOR: return WGM_K_COLOR;
    case WGM_APP_PANNOTIA_MIS: return WGM_K_MIS;
    case WGM_APP_PANNOTIA_SSSP: return WGM_K_PSSSP;
    case WGM_APP_PAGERANK: return WGM_K_PAGERANK;
    case WGM_APP_OCTREE: return WGM_K_OCTREE;
    case WGM_APP_CONNECT_FOUR: return WGM_K_C4;
    case WGM_APP_PANNOTIA_BC: return WGM_K_BC;
    default: return -1;
  }
}

extern "C" const char *wgm_persistent_app_name(int kind) {
  switch (kind) {
    case WGM_APP_LONESTAR_BFS: return "lonestar_bfs";   /* bfs.h:193 */
    case WGM_APP_LONESTAR_SSSP: return "lonestar_sssp"; /* sssp.h:195 */
    case WGM_APP_PANNOTIA_COLOR: return "color";        /* color.h:24 */
    case WGM_APP_PANNOTIA_MIS: return "mis";            /* mis.h:23 */
    case WGM_APP_PANNOTIA_SSSP: return "sssp";          /* pannotia sssp.h:25 */
    case WGM_APP_PAGERANK: return "pagerank";
    case WGM_APP_OCTREE: return "octree";               /* octree.h:79 */
    case WGM_APP_CONNECT_FOUR: return "connect_four";   /* connect_four.h:113 */
    case WGM_APP_PANNOTIA_BC: return "bc";              /* bc.h */
    default: return nullptr;
  }
}

extern "C" const char *wgm_persistent_kernel_name(int kind) {
  switch (kind) {
    case WGM_APP_LONESTAR_BFS: return "drelax2";        /* bfs.h:197 */
    case WGM_APP_LONESTAR_SSSP: return "drelax2";
    case WGM_APP_PANNOTIA_COLOR: return "color_combined";
    case WGM_APP_PANNOTIA_MIS: return "mis_combined";
    case WGM_APP_PANNOTIA_SSSP: return "sssp_combined";
    case WGM_APP_PAGERANK: return "pagerank_pull";
    case WGM_APP_OCTREE: return "octree_main";          /* octree.h:85 */
    case WGM_APP_CONNECT_FOUR: return "connect_four";
    case WGM_APP_PANNOTIA_BC: return "bc_combined";     /* bc.cl:144 */
    default: return nullptr;
  }
}

static bool wgm_is_lonestar(int kind) {
  return kind == WGM_APP_LONESTAR_BFS || kind == WGM_APP_LONESTAR_SSSP;
}
static bool wgm_needs_weights(int kind) {
  return kind == WGM_APP_LONESTAR_SSSP || kind == WGM_APP_PANNOTIA_SSSP;
}
static bool wgm_uses_static_hubs(int kind) {
  return kind == WGM_APP_PANNOTIA_COLOR || kind == WGM_APP_PANNOTIA_MIS ||
         kind == WGM_APP_PANNOTIA_SSSP || kind == WGM_APP_PAGERANK;
}

/* Reject graphs the kernels cannot walk safely.  The Lonestar loader quirk
 * (row_ptr[V] one less than the edge count, lonestar bfs.h:43) is accepted for
 * the Lonestar apps; their kernels also skip out-of-range destinations like
 * bfs.cl:116, every other app needs every col[] inside [0, V). */
static int wgm_validate_graph(int kind, const wgm_graph_desc *g) {
  if (!g || g->num_nodes < 1 || !g->row_ptr || g->num_edges < 0) return WGM_ERR_INVALID;
  if (g->num_edges > 0 && !g->col) return WGM_ERR_INVALID;
  if (g->num_edges >= (int64_t)INT32_MAX) return WGM_ERR_INVALID;
  const int V = g->num_nodes;
  const int32_t *rp = g->row_ptr;
  if (rp[0] != 0) return WGM_ERR_INVALID;
  for (int i = 0; i < V - 1; i++)
    if (rp[i + 1] < rp[i]) return WGM_ERR_INVALID;
  int64_t last = rp[V];
  if (wgm_is_lonestar(kind)) {
    if (last < (int64_t)rp[V - 1] - 1 || last > g->num_edges) return WGM_ERR_INVALID;
  } else {
    if (last < rp[V - 1] || last != g->num_edges) return WGM_ERR_INVALID;
    for (int64_t k = 0; k < g->num_edges; k++)
      if ((uint32_t)g->col[k] >= (uint32_t)V) return WGM_ERR_INVALID;
  }
  if (wgm_needs_weights(kind) && g->num_edges > 0 && !g->weights) return WGM_ERR_INVALID;
  if (kind == WGM_APP_PANNOTIA_COLOR || kind == WGM_APP_PANNOTIA_MIS) {
    /* A self loop makes a vertex its own uncoloured/active neighbour: the
     * reference's colour and MIS loops never end on such a graph. */
    for (int v = 0; v < V; v++)
      for (int k = rp[v]; k < rp[v + 1]; k++)
        if (g->col[k] == v) return WGM_ERR_INVALID;
  }
  return WGM_OK;
}

/* Hub layout for the static-frontier apps (see wgm_hubs in wgm_graph.cuh). */
static void wgm_build_hubs(const wgm_graph_desc *g, int T, std::vector<int> &ids,
                           std::vector<int> &prefix, std::vector<int> &wmap) {
  ids.clear();
  prefix.assign(1, 0);
  wmap.clear();
  for (int v = 0; v < g->num_nodes; v++) {
    int d = g->row_ptr[v + 1] - g->row_ptr[v];
    if (d > T) {
      ids.push_back(v);
      prefix.push_back(prefix.back() + d);
    }
  }
  /* per window of 32 hub-edge slots: {h0, edge of slot k*32, slots of h0,
   * first edge of h0+1} (see wgm_hubs) */
  int total = prefix.back();
  int nwin = (total + 31) / 32;
  const int H = (int)ids.size();
  wmap.resize(4 * (size_t)nwin);
  int h = 0;
  for (int k = 0; k < nwin; k++) {
    while (prefix[h + 1] <= k * 32) h++;
    const int split = h + 1 < H ? std::min(32, prefix[h + 1] - k * 32) : 32;
    wmap[4 * (size_t)k + 0] = h;
    wmap[4 * (size_t)k + 1] = g->row_ptr[ids[h]] + (k * 32 - prefix[h]);
    wmap[4 * (size_t)k + 2] = split;
    wmap[4 * (size_t)k + 3] = split < 32 ? g->row_ptr[ids[h + 1]] : 0;
  }
}

static void wgm_app_free_buffers(wgm_app *a) {
  void *ptrs[] = {a->d_row,     a->d_col,       a->d_wt,      a->d_node_value, a->d_out,
                  a->d_wl_start, a->d_wl_cnt,   a->d_wl_u,
                  a->d_cnt,       a->d_stamp,   a->d_stop,       a->d_hub_acc,
                  a->d_status,  a->d_contrib,   a->d_dang,    a->d_hub_sum,    a->d_rounds,
                  a->hubs.ids,  a->hubs.prefix, a->hubs.wmap, a->d_trow, a->d_tcol,
                  a->d_oct_input, a->d_oct_second, a->d_oct_pools, a->d_oct_tree,
                  a->d_oct_ctr, a->d_oct_locks, a->d_oct_heads,
                  a->d_c4_board, a->d_c4_nodes, a->d_c4_pool, a->d_c4_locks,
                  a->d_c4_heads, a->d_c4_ctr, a->d_tcv, a->d_tcv4, a->d_cmax, a->d_cq,
                  a->d_cqctl};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  a->hubs = wgm_dev_hubs();
}

template <class T>
static cudaError_t wgm_dmalloc(T **p, size_t count) {
  return cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T));
}

static int wgm_upload_hubs(wgm_app *a, const wgm_graph_desc *g) {
  std::vector<int> ids, prefix, wmap;
  wgm_build_hubs(g, a->hub_threshold, ids, prefix, wmap);
  cudaStream_t s = a->rt->stream;
  cudaError_t e = cudaSuccess;
  if (a->hubs.ids) {
    cudaFree(a->hubs.ids);
    cudaFree(a->hubs.prefix);
    cudaFree(a->hubs.wmap);
    a->hubs = wgm_dev_hubs();
  }
  if (e == cudaSuccess) e = wgm_dmalloc(&a->hubs.ids, ids.size());
  if (e == cudaSuccess) e = wgm_dmalloc(&a->hubs.prefix, prefix.size());
  if (e == cudaSuccess) e = wgm_dmalloc(&a->hubs.wmap, wmap.size());
  if (e == cudaSuccess && !ids.empty())
    e = cudaMemcpyAsync(a->hubs.ids, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(a->hubs.prefix, prefix.data(), prefix.size() * 4,
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !wmap.empty())
    e = cudaMemcpyAsync(a->hubs.wmap, wmap.data(), wmap.size() * 4, cudaMemcpyHostToDevice, s);
  /* the host vectors die here: finish the copies first */
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return wgm_cuda_fail(a->rt, e);
  a->hubs.H = (int)ids.size();
  a->hubs.total = prefix.back();
  if (a->kind == WGM_APP_PANNOTIA_COLOR || a->kind == WGM_APP_PANNOTIA_MIS ||
      a->kind == WGM_APP_PAGERANK) {
    if (a->d_hub_acc) cudaFree(a->d_hub_acc);
    if (a->d_hub_sum) cudaFree(a->d_hub_sum);
    a->d_hub_acc = nullptr;
    a->d_hub_sum = nullptr;
    if (a->kind == WGM_APP_PAGERANK)
      e = wgm_dmalloc(&a->d_hub_sum, (size_t)a->hubs.H);
    else
      e = wgm_dmalloc(&a->d_hub_acc, (size_t)a->hubs.H * 2);
    if (e != cudaSuccess) return wgm_cuda_fail(a->rt, e);
  }
  return WGM_OK;
}

/* Colour releases in-neighbours, so it needs the in-edge CSR.  Built by a
 * counting sort over sources in increasing order; for a symmetric graph
 * whose rows are sorted this is the graph itself, and the device arrays are
 * shared instead of copied. */
static int wgm_upload_transpose(wgm_app *a, const wgm_graph_desc *g) {
  const int V = g->num_nodes;
  const int64_t E = g->row_ptr[V];
  std::vector<int> trow(V + 1, 0), tcol(std::max<int64_t>(E, 1));
  for (int64_t e = 0; e < E; e++) trow[g->col[e] + 1]++;
  for (int v = 0; v < V; v++) trow[v + 1] += trow[v];
  {
    std::vector<int> fill(trow.begin(), trow.end() - 1);
    for (int v = 0; v < V; v++)
      for (int64_t e = g->row_ptr[v]; e < g->row_ptr[v + 1]; e++) tcol[fill[g->col[e]]++] = v;
  }
  bool same = std::equal(trow.begin(), trow.end(), g->row_ptr) &&
              std::equal(tcol.begin(), tcol.begin() + E, g->col);
  if (a->d_trow) cudaFree(a->d_trow);
  if (a->d_tcol) cudaFree(a->d_tcol);
  a->d_trow = a->d_tcol = nullptr;
  if (same) return WGM_OK;
  cudaError_t e = wgm_dmalloc(&a->d_trow, (size_t)V + 1);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_tcol, (size_t)std::max<int64_t>(E, 1));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(a->d_trow, trow.data(), (size_t)(V + 1) * 4, cudaMemcpyHostToDevice,
                        a->rt->stream);
  if (e == cudaSuccess && E)
    e = cudaMemcpyAsync(a->d_tcol, tcol.data(), (size_t)E * 4, cudaMemcpyHostToDevice,
                        a->rt->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(a->rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(a->rt, e);
  return WGM_OK;
}

extern "C" int wgm_app_upload(wgm_app *a, const wgm_graph_desc *g) {
  if (!a || a->kind == WGM_APP_OCTREE || a->kind == WGM_APP_CONNECT_FOUR ||
      a->kind == WGM_APP_PLUGIN)
    return WGM_ERR_INVALID;
  int s = wgm_validate_graph(a->kind, g);
  if (s) return s;
  if (g->num_nodes != a->V || g->num_edges != a->E) return WGM_ERR_INVALID;
  cudaSetDevice(a->rt->device);
  cudaStream_t st = a->rt->stream;
  cudaError_t e =
      cudaMemcpyAsync(a->d_row, g->row_ptr, (size_t)(a->V + 1) * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && a->E > 0)
    e = cudaMemcpyAsync(a->d_col, g->col, (size_t)a->E * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && wgm_needs_weights(a->kind) && a->E > 0)
    e = cudaMemcpyAsync(a->d_wt, g->weights, (size_t)a->E * 4, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return wgm_cuda_fail(a->rt, e);
  if (wgm_uses_static_hubs(a->kind)) {
    s = wgm_upload_hubs(a, g);
    if (s) return s;
  }
  if (a->kind == WGM_APP_PANNOTIA_COLOR || a->kind == WGM_APP_PANNOTIA_BC) {
    s = wgm_upload_transpose(a, g);
    if (s) return s;
  }
  if (a->kind == WGM_APP_PAGERANK) {
    /* Initial dangling mass: every vertex starts at 1/V. */
    int64_t zero = 0;
    for (int v = 0; v < a->V; v++) zero += (g->row_ptr[v + 1] == g->row_ptr[v]);
    a->dang0 = (float)((double)zero / (double)a->V);
  }
  return WGM_OK;
}

extern "C" int wgm_app_create(wgm_runtime *rt, int kind, const wgm_graph_desc *g,
                              wgm_app **out) {
  if (!rt || !out) return WGM_ERR_INVALID;
  *out = nullptr;
  /* the octree has particles, not a graph: wgm_octree_create */
  if (wgm_kind_to_kernel(kind) < 0 || kind == WGM_APP_OCTREE || kind == WGM_APP_CONNECT_FOUR)
    return WGM_ERR_INVALID;
  int s = wgm_validate_graph(kind, g);
  if (s) return s;
  cudaSetDevice(rt->device);
  wgm_app *a = new (std::nothrow) wgm_app();
  if (!a) return WGM_ERR_OOM;
  a->rt = rt;
  a->kind = kind;
  a->V = g->num_nodes;
  a->E = g->num_edges;
  a->hub_threshold = std::max(rt->cfg.hub_threshold, 32);
  const size_t V = (size_t)a->V, E = (size_t)a->E;
  cudaError_t e = wgm_dmalloc(&a->d_row, V + 1);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_col, E);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_rounds, 1);
  if (e == cudaSuccess && wgm_needs_weights(kind)) e = wgm_dmalloc(&a->d_wt, E);
  switch (kind) {
    case WGM_APP_LONESTAR_BFS:
    case WGM_APP_LONESTAR_SSSP: {
      a->out_bytes = V * 4;
      /* Pieces of at most `piece` edges; piece >= E/V keeps a level's list
       * within V + E/piece <= 2V entries. */
      int64_t avg = (int64_t)((E + V - 1) / std::max<size_t>(V, 1));
      a->piece = (int)std::max<int64_t>(32, avg);
      a->wl_cap = (int)(V + (E + a->piece - 1) / a->piece + 64);
      if (e == cudaSuccess) e = cudaMalloc(&a->d_out, a->out_bytes);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_wl_start, 2 * (size_t)a->wl_cap);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_wl_cnt, 2 * (size_t)a->wl_cap);
      if (e == cudaSuccess && kind == WGM_APP_LONESTAR_SSSP)
        e = wgm_dmalloc(&a->d_wl_u, 2 * (size_t)a->wl_cap);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_cnt, 3 * WGM_LINE);
      /* SSSP: 64-bit {level tag, distance} words (wgm_ls_chunk PACK) */
      if (e == cudaSuccess && kind == WGM_APP_LONESTAR_SSSP) e = wgm_dmalloc(&a->d_stamp, 2 * V);
      break;
    }
    case WGM_APP_PANNOTIA_COLOR:
    case WGM_APP_PANNOTIA_MIS:
      a->out_bytes = V * 4;
      if (e == cudaSuccess) e = cudaMalloc(&a->d_out, a->out_bytes);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_node_value, V);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_stop, 3 * WGM_LINE);
      if (e == cudaSuccess && kind == WGM_APP_PANNOTIA_COLOR) {
        /* frontier pieces of in-edges; every vertex is coloured once, so a
         * round never holds more than V + E/piece pieces */
        int64_t avg = (int64_t)((E + V - 1) / std::max<size_t>(V, 1));
        a->piece = (int)std::max<int64_t>(32, avg);
        a->wl_cap = (int)(V + (E + a->piece - 1) / a->piece + 64);
        e = wgm_dmalloc(&a->d_wl_start, 2 * (size_t)a->wl_cap);
        if (e == cudaSuccess) e = wgm_dmalloc(&a->d_wl_cnt, 2 * (size_t)a->wl_cap);
        if (e == cudaSuccess) e = wgm_dmalloc(&a->d_wl_u, 2 * (size_t)a->wl_cap);
        if (e == cudaSuccess) e = wgm_dmalloc(&a->d_stamp, V); /* pending */
        if (e == cudaSuccess) e = wgm_dmalloc(&a->d_cnt, 3 * WGM_LINE);
        if (e == cudaSuccess) e = wgm_dmalloc(&a->d_tcv, E); /* in-edges with values */
      }
      if (e == cudaSuccess && kind == WGM_APP_PANNOTIA_MIS) e = wgm_dmalloc(&a->d_status, V);
      break;
    case WGM_APP_PANNOTIA_SSSP:
      a->out_bytes = V * 4;
      if (e == cudaSuccess) e = cudaMalloc(&a->d_out, a->out_bytes);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_stop, 3 * WGM_LINE);
      break;
    case WGM_APP_PAGERANK:
      a->out_bytes = V * 4;
      if (e == cudaSuccess) e = cudaMalloc(&a->d_out, a->out_bytes);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_contrib, 2 * V);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_dang, 3 * WGM_LINE);
      break;
    case WGM_APP_PANNOTIA_BC:
      /* bc (out), dist, rho and sigma, the level lists and their starts */
      a->out_bytes = V * 4;
      a->bc_sources = a->V;
      a->bc_mode = a->V <= WGM_BC_CTA_MAX_V ? 1 : 0;
      if (e == cudaSuccess) e = cudaMalloc(&a->d_out, a->out_bytes);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_stamp, V);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_contrib, 2 * V);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_wl_u, V);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_wl_start, V + 2);
      if (e == cudaSuccess) e = wgm_dmalloc(&a->d_cnt, 3 * WGM_LINE);
      break;
  }
  if (e != cudaSuccess) {
    s = wgm_cuda_fail(rt, e);
    wgm_app_free_buffers(a);
    delete a;
    return s;
  }
  s = wgm_app_upload(a, g);
  if (s == WGM_OK && (kind == WGM_APP_PANNOTIA_COLOR || kind == WGM_APP_PANNOTIA_MIS)) {
    /* Default priorities: the reference rule node_value[i] = i/(V+1)
     * (color.h:53, mis.h:55). */
    std::vector<float> nv(V);
    for (size_t i = 0; i < V; i++) nv[i] = (float)i / (float)(a->V + 1);
    s = wgm_app_set_node_values(a, nv.data());
    a->has_node_values = false;
  }
  if (s) {
    wgm_app_free_buffers(a);
    delete a;
    return s;
  }
  *out = a;
  return WGM_OK;
}

extern "C" int wgm_app_set_source(wgm_app *a, int32_t source) {
  if (!a || a->kind == WGM_APP_OCTREE || a->kind == WGM_APP_CONNECT_FOUR ||
      a->kind == WGM_APP_PLUGIN || source < 0 || source >= a->V)
    return WGM_ERR_INVALID;
  a->source = source;
  return WGM_OK;
}

extern "C" int wgm_app_set_node_values(wgm_app *a, const float *nv) {
  if (!a || !nv || !a->d_node_value) return WGM_ERR_INVALID;
  for (int i = 0; i < a->V; i++)
    if (!(nv[i] >= 0.0f && nv[i] < 1.0e30f)) return WGM_ERR_INVALID; /* finite, >= 0 */
  {
    /* Equal priorities on adjacent vertices stall colour and MIS forever (in
     * the reference too): require distinct values. */
    std::vector<float> sorted(nv, nv + a->V);
    std::sort(sorted.begin(), sorted.end());
    for (int i = 1; i < a->V; i++)
      if (sorted[i] == sorted[i - 1]) return WGM_ERR_INVALID;
  }
  cudaSetDevice(a->rt->device);
  cudaError_t e = cudaMemcpyAsync(a->d_node_value, nv, (size_t)a->V * 4, cudaMemcpyHostToDevice,
                                  a->rt->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(a->rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(a->rt, e);
  a->has_node_values = true;
  return WGM_OK;
}

extern "C" int wgm_app_set_bc_mode(wgm_app *a, int32_t mode) {
  if (!a || a->kind != WGM_APP_PANNOTIA_BC || mode < 0 || mode > 1 ||
      (mode == 1 && a->V > WGM_BC_CTA_MAX_V))
    return WGM_ERR_INVALID;
  a->bc_mode = mode;
  return WGM_OK;
}

/* Sources spread over CTAs (bc_mode 1): a plain launch of resident CTAs, no
 * discovery and no host handshake, so the launch generation is untouched. */
static int wgm_bc_cta_launch(wgm_runtime *rt, wgm_app *a, cudaStream_t s) {
  (void)rt->cfg;
  wgm_mega_args A;
  std::memset(&A, 0, sizeof(A));
  int st = wgm_app_fill_mega(a, &A);
  if (st) return st;
  /* 512 threads: on RMAT-12 4.2 ms against 5.7 (256), 8.8 (128), 6.5 (1024) */
  cudaError_t e = wgm_launch_bc_cta(A.bc, a->d_cnt + 2 * WGM_LINE, 512, s);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  return WGM_OK;
}

/* Lonestar BFS on one CTA (wgm_bfs_cta): chosen by default for graphs of
 * at most WGM_BFS_CTA_AUTO_V vertices and average degree at most 8, whose
 * levels carry little work each; possible up to WGM_BFS_CTA_MAX_V vertices
 * (the visited bits in shared memory). */
#define WGM_BFS_CTA_AUTO_V 65536
#define WGM_BFS_CTA_MAX_V (1 << 20)
static bool wgm_bfs_cta_on(const wgm_app *a) {
  if (a->kind != WGM_APP_LONESTAR_BFS || a->V > WGM_BFS_CTA_MAX_V) return false;
  if (a->bfs_mode >= 0) return a->bfs_mode == 1;
  return a->V <= WGM_BFS_CTA_AUTO_V && a->E <= 8LL * a->V;
}

static int wgm_bfs_cta_launch(wgm_runtime *rt, wgm_app *a, cudaStream_t s) {
  wgm_mega_args A;
  std::memset(&A, 0, sizeof(A));
  int st = wgm_app_fill_mega(a, &A);
  if (st) return st;
  /* the frontier buffers take what shared memory the visited bits leave */
  const long long avail = (long long)rt->prop.sharedMemPerBlockOptin - 1024 -
                          (long long)((a->V + 31) / 32) * 4;
  const int F = (int)std::min<long long>(1 << 16, avail / 8);
  if (F < 256) return WGM_ERR_INVALID;
  if (rt->cfg.host_handshake) return WGM_ERR_INVALID; /* no discovery, no handshake */
  cudaError_t e = wgm_launch_bfs_cta(A.ls, a->d_wl_start, a->wl_cap, F, &rt->hf_dev->status,
                                     1024, s);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  return WGM_OK;
}

extern "C" int wgm_app_set_bfs_mode(wgm_app *a, int32_t mode) {
  if (!a || a->kind != WGM_APP_LONESTAR_BFS || mode < -1 || mode > 1 ||
      (mode == 1 && a->V > WGM_BFS_CTA_MAX_V))
    return WGM_ERR_INVALID;
  a->bfs_mode = mode;
  return WGM_OK;
}

extern "C" int wgm_app_set_bc_sources(wgm_app *a, int32_t num_sources) {
  if (!a || a->kind != WGM_APP_PANNOTIA_BC || num_sources < 0 || num_sources > a->V)
    return WGM_ERR_INVALID;
  a->bc_sources = num_sources;
  return WGM_OK;
}

extern "C" int wgm_app_set_color_mode(wgm_app *a, int32_t mode) {
  if (!a || a->kind != WGM_APP_PANNOTIA_COLOR || mode < 0 || mode > 1) return WGM_ERR_INVALID;
  a->color_mode = mode;
  return WGM_OK;
}

extern "C" int wgm_app_set_pagerank(wgm_app *a, float damping, int iterations) {
  if (!a || a->kind != WGM_APP_PAGERANK || iterations < 0 || !(damping >= 0.f && damping <= 1.f))
    return WGM_ERR_INVALID;
  a->damping = damping;
  a->iterations = iterations;
  return WGM_OK;
}

static wgm_hubs wgm_hubs_view(const wgm_app *a) {
  wgm_hubs h;
  h.ids = a->hubs.ids;
  h.prefix = a->hubs.prefix;
  h.wmap = a->hubs.wmap;
  h.H = a->hubs.H;
  h.total = a->hubs.total;
  return h;
}

/* Fill the kernel arguments of the app (also used by the megakernel). */
int wgm_app_fill_mega(wgm_app *a, wgm_mega_args *A) {
  if (a->kind == WGM_APP_PLUGIN) return WGM_ERR_INVALID; /* its own megakernel */
  A->app = wgm_kind_to_kernel(a->kind);
  switch (a->kind) {
    case WGM_APP_OCTREE: {
      wgm_octree_args &x = A->oct;
      x.input = (const float4 *)a->d_oct_input;
      x.particles = (float4 *)a->d_out;
      x.newparticles = (float4 *)a->d_oct_second;
      x.tree = a->d_oct_tree;
      x.tree_cap = a->oct_tree_cap;
      x.tree_size = a->d_oct_ctr;
      x.done = a->d_oct_ctr + 32; /* its own 128-byte line */
      x.n = a->V;
      x.maxchilds = a->oct_maxchilds;
      x.pools = (wgm_octree_task *)a->d_oct_pools;
      x.locks = a->d_oct_locks;
      x.heads = a->d_oct_heads;
      x.num_pools = a->oct_num_pools;
      x.pool_size = a->oct_pool_size;
      x.tasks_out = a->d_rounds;
      x.rlock = (int *)(a->d_oct_ctr + 64); /* a third line */
      return WGM_OK;
    }
    case WGM_APP_PANNOTIA_BC: {
      wgm_bc_args &x = A->bc;
      x.V = a->V;
      x.row = a->d_row;
      x.col = a->d_col;
      x.trow = a->d_trow ? a->d_trow : a->d_row;
      x.tcol = a->d_tcol ? a->d_tcol : a->d_col;
      x.bc = (float *)a->d_out;
      x.dist = a->d_stamp;
      x.rho = a->d_contrib;
      x.sigma = a->d_contrib + a->V;
      x.order = a->d_wl_u;
      x.level_start = a->d_wl_start;
      x.cnt = a->d_cnt;
      x.num_sources = a->bc_sources;
      x.rounds_out = a->d_rounds;
      return WGM_OK;
    }
    case WGM_APP_CONNECT_FOUR: {
      wgm_c4_args &x = A->c4;
      x.base_board = a->d_c4_board;
      x.maxlevel = a->c4_maxlevel;
      x.nodes = (wgm_c4_node *)a->d_c4_nodes;
      x.num_nodes = a->c4_num_nodes;
      x.node_head = a->d_c4_ctr;
      x.root_done = a->d_c4_ctr + 32;
      x.rlock = a->d_c4_ctr + 64;
      x.pool = a->d_c4_pool;
      x.locks = a->d_c4_locks;
      x.heads = a->d_c4_heads;
      x.num_pools = a->c4_num_pools;
      x.pool_size = a->c4_pool_size;
      x.next_move_value = (int *)a->d_out;
      x.tasks_out = a->d_rounds;
      return WGM_OK;
    }
    case WGM_APP_LONESTAR_BFS:
    case WGM_APP_LONESTAR_SSSP: {
      wgm_lonestar_args &x = A->ls;
      x.V = a->V;
      x.row = a->d_row;
      x.col = a->d_col;
      x.wt = a->d_wt;
      x.dist = (unsigned *)a->d_out;
      x.wl_start = a->d_wl_start;
      x.wl_cnt = a->d_wl_cnt;
      x.wl_u = a->d_wl_u;
      x.cap = a->wl_cap;
      x.piece = a->piece;
      x.cnt = a->d_cnt;
      x.stamp = a->d_stamp;
      x.source = a->source;
      x.levels_out = a->d_rounds;
      x.packed = a->kind == WGM_APP_LONESTAR_SSSP ? 1 : 0;
      return WGM_OK;
    }
    case WGM_APP_PANNOTIA_COLOR: {
      wgm_color_args &x = A->color;
      x.V = a->V;
      x.row = a->d_row;
      x.col = a->d_col;
      x.node_value = a->d_node_value;
      x.color = (int *)a->d_out;
      x.stop = a->d_stop;
      x.hub_acc = a->d_hub_acc;
      x.hubs = wgm_hubs_view(a);
      x.hub_threshold = a->hub_threshold;
      x.rounds_out = a->d_rounds;
      x.trow = a->d_trow ? a->d_trow : a->d_row;
      x.tcol = a->d_tcol ? a->d_tcol : a->d_col;
      x.pending = a->d_stamp;
      x.wl_start = a->d_wl_start;
      x.wl_cnt = a->d_wl_cnt;
      x.wl_u = a->d_wl_u;
      x.cap = a->wl_cap;
      x.piece = a->piece;
      x.cnt = a->d_cnt;
      x.tcv = a->d_tcv;
      return WGM_OK;
    }
    case WGM_APP_PANNOTIA_MIS: {
      wgm_mis_args &x = A->mis;
      x.V = a->V;
      x.row = a->d_row;
      x.col = a->d_col;
      x.node_value = a->d_node_value;
      x.s_array = (int *)a->d_out;
      x.status = a->d_status;
      x.stop = a->d_stop;
      x.hub_acc = a->d_hub_acc;
      x.hubs = wgm_hubs_view(a);
      x.hub_threshold = a->hub_threshold;
      x.rounds_out = a->d_rounds;
      return WGM_OK;
    }
    case WGM_APP_PANNOTIA_SSSP: {
      wgm_psssp_args &x = A->psssp;
      x.V = a->V;
      x.row = a->d_row;
      x.col = a->d_col;
      x.data = (const int *)a->d_wt;
      x.x = (int *)a->d_out;
      x.stop = a->d_stop;
      x.hubs = wgm_hubs_view(a);
      x.hub_threshold = a->hub_threshold;
      x.source = a->source;
      x.rounds_out = a->d_rounds;
      return WGM_OK;
    }
    case WGM_APP_PAGERANK: {
      wgm_pr_args &x = A->pr;
      x.V = a->V;
      x.row = a->d_row;
      x.col = a->d_col;
      x.pr = (float *)a->d_out;
      x.contrib = a->d_contrib;
      x.dang = a->d_dang;
      x.hub_sum = a->d_hub_sum;
      x.hubs = wgm_hubs_view(a);
      x.hub_threshold = a->hub_threshold;
      x.iterations = a->iterations;
      x.damping = a->damping;
      x.dang0 = a->dang0;
      return WGM_OK;
    }
  }
  return WGM_ERR_INVALID;
}

/* Colour without rounds: its buffers, on first use. */
static cudaError_t wgm_color_async_alloc(wgm_app *a) {
  if (a->d_tcv4) return cudaSuccess;
  const int64_t ET = a->E; /* in-edges: the graph's, or its transpose's (same count) */
  a->cq_cap = (int)std::min<int64_t>(INT32_MAX - 64, (int64_t)a->V + (ET + 31) / 32 + 64);
  cudaError_t e = wgm_dmalloc(&a->d_tcv4, (size_t)std::max<int64_t>(ET, 1));
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_cmax, (size_t)a->V);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_cq, 4 * (size_t)a->cq_cap);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_cqctl, 5 * (size_t)WGM_LINE);
  return e;
}

static wgm_color_async_args wgm_color_async_view(const wgm_app *a) {
  wgm_color_async_args q;
  q.tcv4 = a->d_tcv4;
  q.cmax = a->d_cmax;
  q.q_start = a->d_cq;
  q.q_cnt = a->d_cq + (size_t)a->cq_cap;
  q.q_val = a->d_cq + 2 * (size_t)a->cq_cap;
  q.q_col = a->d_cq + 3 * (size_t)a->cq_cap;
  q.qcap = a->cq_cap;
  q.ctl = a->d_cqctl;
  return q;
}

static bool wgm_color_async_on(const wgm_app *a) {
  return a->kind == WGM_APP_PANNOTIA_COLOR && a->color_mode == 1;
}

/* Enqueue the app's standalone persistent kernel on `stream`. */
static cudaError_t wgm_app_enqueue(wgm_app *a, const wgm_launch &L, int grid, int block,
                                   cudaStream_t stream) {
  if (a->kind == WGM_APP_PLUGIN) {
    if (a->vt.reset && a->vt.reset(a->vt.user, stream) != WGM_OK) return cudaErrorInvalidValue;
    return a->vt.launch(a->vt.user, &L, grid, block, stream) == WGM_OK ? cudaSuccess
                                                                        : cudaErrorLaunchFailure;
  }
  wgm_mega_args A;
  std::memset(&A, 0, sizeof(A));
  if (wgm_app_fill_mega(a, &A) != WGM_OK) return cudaErrorInvalidValue;
  switch (a->kind) {
    case WGM_APP_LONESTAR_BFS:
    case WGM_APP_LONESTAR_SSSP:
      return wgm_launch_lonestar(a->kind == WGM_APP_LONESTAR_SSSP, L, A.ls, grid, block, stream);
    case WGM_APP_PANNOTIA_COLOR:
      if (wgm_color_async_on(a)) {
        cudaError_t e = wgm_color_async_alloc(a);
        if (e != cudaSuccess) return e;
        return wgm_launch_color_async(L, A.color, wgm_color_async_view(a), grid, block, stream);
      }
      return wgm_launch_color(L, A.color, grid, block, stream);
    case WGM_APP_PANNOTIA_MIS:
      return wgm_launch_mis(L, A.mis, grid, block, stream);
    case WGM_APP_PANNOTIA_SSSP:
      return wgm_launch_psssp(L, A.psssp, grid, block, stream);
    case WGM_APP_PAGERANK:
      return wgm_launch_pagerank(L, A.pr, grid, block, stream);
    case WGM_APP_OCTREE:
      return wgm_launch_octree(L, A.oct, grid, block, stream);
    case WGM_APP_CONNECT_FOUR:
      return wgm_launch_c4(L, A.c4, grid, block, stream);
    case WGM_APP_PANNOTIA_BC:
      return wgm_launch_bc(L, A.bc, grid, block, stream);
  }
  return cudaErrorInvalidValue;
}

/* Co-resident CTAs of a registered app's kernel (mega = 1: its megakernel). */
int wgm_plugin_hw_bound(wgm_app *a, int mega, int block, int *groups) {
  int per_sm = 0;
  int s = a->vt.occupancy(a->vt.user, mega, block, &per_sm);
  if (s) return s;
  const long g = (long)per_sm * a->rt->prop.multiProcessorCount;
  *groups = (int)std::min<long>(g, WGM_MAX_GROUPS);
  return WGM_OK;
}

static int wgm_pick_grid(wgm_app *a, int num_wgs, int block, int *grid) {
  int hw = 0;
  int s = WGM_OK;
  if (a->kind == WGM_APP_PLUGIN) {
    s = wgm_plugin_hw_bound(a, 0, block, &hw);
  } else if (wgm_color_async_on(a)) {
    int per_sm = 0;
    cudaError_t e = wgm_color_async_per_sm(block, &per_sm);
    if (e != cudaSuccess) return wgm_cuda_fail(a->rt, e);
    hw = std::min(per_sm * a->rt->prop.multiProcessorCount, WGM_MAX_GROUPS);
  } else {
    s = wgm_hw_bound_for(a->rt, wgm_kind_to_kernel(a->kind), block, &hw);
  }
  if (s) return s;
  if (hw < 1) return WGM_ERR_INVALID;
  *grid = (num_wgs > 0) ? std::min(num_wgs, hw) : hw;
  /* Pannotia colour by default: 512 threads per SM.  Its rounds (~1600 on
   * RMAT-20) carry little work each and end in a grid barrier, so fewer
   * groups win: 304 x 256 threads ran RMAT-20 in 8.6 ms against 9.7 ms on
   * all 608 co-resident CTAs (and take the counting barrier). */
  if (num_wgs <= 0 && a->kind == WGM_APP_PANNOTIA_COLOR && !wgm_color_async_on(a)) {
    const int sms = a->rt->prop.multiProcessorCount;
    *grid = std::min(hw, std::max(sms, sms * 512 / std::max(block, 1)));
  }
  /* Lonestar BFS/SSSP by default: one group per 8192 edges, rounded up to
   * a multiple of the SM count.  A level costs a grid barrier plus a chain
   * of dependent round trips whatever its size, so a small graph runs its
   * levels faster on fewer groups: the 256x256 grid's 512 BFS levels took
   * 4.1 us each on 152 CTAs against 6.4 us on all 608.  At 256 threads a
   * graph of 5M edges or more keeps every co-resident CTA. */
  if (num_wgs <= 0 &&
      (a->kind == WGM_APP_LONESTAR_BFS || a->kind == WGM_APP_LONESTAR_SSSP)) {
    const long long sms = a->rt->prop.multiProcessorCount;
    const long long want = ((long long)a->E / 8192 + sms - 1) / sms * sms;
    *grid = (int)std::min<long long>(hw, std::max(sms, want));
  }
  /* Pannotia SSSP by default: 1024 threads per SM (four 256-thread CTAs of
   * the six that fit), more only for graphs of more than one 256-thread CTA
   * per 32768 edges: on grids and RMAT graphs up to 7.6M edges four CTAs
   * per SM ran 9-15 % faster than six, on RMAT-20 (33M edges) six won. */
  if (num_wgs <= 0 && a->kind == WGM_APP_PANNOTIA_SSSP) {
    const long long sms = a->rt->prop.multiProcessorCount, b = std::max(block, 1);
    const long long base = sms * std::max(1LL, 1024 / b);
    const long long byE = ((long long)a->E / 128 / b + sms - 1) / sms * sms;
    *grid = (int)std::min<long long>(hw, std::max(base, byE));
  }
  return WGM_OK;
}

static int wgm_block_size(const wgm_runtime *rt) {
  int b = rt->cfg.threads_per_wg;
  if (b < 32 || b > 1024 || b % 32) b = 256;
  return b;
}

extern "C" int wgm_launch_persistent(wgm_runtime *rt, wgm_app *a, int num_wgs, void *stream) {
  if (!rt || !a || a->rt != rt) return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  if (a->kind == WGM_APP_PANNOTIA_BC && a->bc_mode == 1)
    return wgm_bc_cta_launch(rt, a, stream ? (cudaStream_t)stream : rt->stream);
  if (wgm_bfs_cta_on(a) && num_wgs <= 1 && !rt->cfg.host_handshake)
    return wgm_bfs_cta_launch(rt, a, stream ? (cudaStream_t)stream : rt->stream);
  int block = wgm_block_size(rt), grid = 0;
  int s = wgm_pick_grid(a, num_wgs, block, &grid);
  if (s) return s;
  if (rt->cfg.host_handshake) {
    __atomic_store_n(&rt->hf->scheduler_flag, WGM_DEVICE_SCHEDULER_INIT, __ATOMIC_RELEASE);
    __atomic_store_n(&rt->hf->persistent_flag, -1, __ATOMIC_RELEASE);
  }
  wgm_launch L = wgm_make_launch(rt, grid, rt->cfg.host_handshake ? 1 : 0, 0);
  cudaError_t e = wgm_app_enqueue(a, L, grid, block, stream ? (cudaStream_t)stream : rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  return WGM_OK;
}

extern "C" int wgm_run_persistent(wgm_runtime *rt, wgm_app *a, int num_wgs,
                                  wgm_run_stats *stats) {
  if (!rt || !a || a->rt != rt) return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  const bool bfs_cta = wgm_bfs_cta_on(a) && num_wgs <= 1 && !rt->cfg.host_handshake;
  if ((a->kind == WGM_APP_PANNOTIA_BC && a->bc_mode == 1) || bfs_cta) {
    cudaError_t e = cudaEventRecord(rt->ev0, rt->stream);
    if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
    int s = bfs_cta ? wgm_bfs_cta_launch(rt, a, rt->stream) : wgm_bc_cta_launch(rt, a, rt->stream);
    if (s) return s;
    e = cudaEventRecord(rt->ev1, rt->stream);
    if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
    s = wgm_stream_wait(rt, rt->stream);
    if (s) return s;
    if (bfs_cta) { /* a frontier past every buffer reports an overflow */
      s = wgm_finish_launch(rt, nullptr, nullptr);
      if (s) return s;
    }
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      stats->groups = bfs_cta ? 1 : 0;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, rt->ev0, rt->ev1);
      stats->kernel_ms = ms;
      int rounds = 0;
      if (cudaMemcpy(&rounds, a->d_rounds, 4, cudaMemcpyDeviceToHost) == cudaSuccess)
        stats->rounds = rounds;
    }
    return WGM_OK;
  }
  int block = wgm_block_size(rt), grid = 0;
  int s = wgm_pick_grid(a, num_wgs, block, &grid);
  if (s) return s;
  const int handshake = rt->cfg.host_handshake ? 1 : 0;
  if (handshake) {
    __atomic_store_n(&rt->hf->scheduler_flag, WGM_DEVICE_SCHEDULER_INIT, __ATOMIC_RELEASE);
    __atomic_store_n(&rt->hf->persistent_flag, -1, __ATOMIC_RELEASE);
  }
  wgm_launch L = wgm_make_launch(rt, grid, handshake, 0);
  cudaError_t e = cudaEventRecord(rt->ev0, rt->stream);
  if (e == cudaSuccess) e = wgm_app_enqueue(a, L, grid, block, rt->stream);
  if (e == cudaSuccess) e = cudaEventRecord(rt->ev1, rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  double host_ms = 0.0;
  int hs_status = WGM_OK;
  if (handshake) {
    /* skel.cpp:336-340: wait for DEVICE_WAITING, start the clock, release
     * the task, wait for persistent_flag to drain to 0. */
    uint64_t budget = rt->cfg.spin_timeout_ns ? rt->cfg.spin_timeout_ns : 2000000000ull;
    if (!wgm_host_wait(&rt->hf->scheduler_flag, WGM_DEVICE_WAITING, true, budget * 4)) {
      wgm_set_abort(rt, 1);
      hs_status = WGM_ERR_TIMEOUT;
    } else {
      auto t0 = std::chrono::steady_clock::now();
      __atomic_store_n(&rt->hf->scheduler_flag, WGM_DEVICE_TO_PERSISTENT_TASK, __ATOMIC_RELEASE);
      if (!wgm_host_wait(&rt->hf->persistent_flag, 0, true, budget * 16)) {
        wgm_set_abort(rt, 1);
        hs_status = WGM_ERR_TIMEOUT;
      }
      auto t1 = std::chrono::steady_clock::now();
      host_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    }
  }
  int ws = wgm_stream_wait(rt, rt->stream);
  if (ws == WGM_ERR_CUDA) return ws;
  if (hs_status != WGM_OK) wgm_set_abort(rt, 0);
  int dev_status = 0, dev_site = 0;
  int groups = __atomic_load_n(&rt->hf->discovered, __ATOMIC_ACQUIRE);
  s = wgm_finish_launch(rt, &dev_status, &dev_site);
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->groups = groups;
    stats->device_status = dev_status;
    stats->device_site = dev_site;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, rt->ev0, rt->ev1);
    stats->kernel_ms = ms;
    stats->host_ms = host_ms;
    int rounds = 0;
    if (s == WGM_OK && wgm_app_rounds(a, &rounds) == WGM_OK) stats->rounds = rounds;
  }
  if (s == WGM_OK && hs_status != WGM_OK) s = hs_status;
  if (s == WGM_OK && ws != WGM_OK) s = ws;
  return s;
}

/* Octree app (octree.h:98-132 init_persistent_app_for_real): the input
 * particles stay on the device and every run starts from them; pools are
 * min(occupancy bound, 128) stacks of pool_size tasks. */
extern "C" int wgm_octree_create(wgm_runtime *rt, int32_t num_particles, const float *xyzw,
                                 int32_t maxchilds, int32_t pool_size, int64_t tree_cap,
                                 wgm_app **out) {
  if (!rt || !out || !xyzw || num_particles < 1 || maxchilds < 1 || pool_size < 1 ||
      tree_cap < (int64_t)WGM_OCTREE_ROOT_FREE + 8 || tree_cap > (1LL << 31))
    return WGM_ERR_INVALID;
  for (int64_t i = 0; i < 4LL * num_particles; i++)
    if (!(std::fabs(xyzw[i]) < 1.0e30f)) return WGM_ERR_INVALID; /* finite */
  *out = nullptr;
  cudaSetDevice(rt->device);
  wgm_app *a = new (std::nothrow) wgm_app();
  if (!a) return WGM_ERR_OOM;
  a->rt = rt;
  a->kind = WGM_APP_OCTREE;
  a->V = num_particles;
  a->oct_maxchilds = maxchilds;
  a->oct_pool_size = pool_size;
  a->oct_tree_cap = tree_cap;
  int hw = 0;
  int s = wgm_hw_bound_for(rt, WGM_K_OCTREE, wgm_block_size(rt), &hw);
  if (s) {
    delete a;
    return s;
  }
  a->oct_num_pools = std::max(1, std::min(hw, 128));
  const size_t n = (size_t)num_particles;
  a->out_bytes = n * 16;
  cudaError_t e = cudaMalloc(&a->d_out, n * 16);
  if (e == cudaSuccess) e = cudaMalloc(&a->d_oct_input, n * 16);
  if (e == cudaSuccess) e = cudaMalloc(&a->d_oct_second, n * 16);
  if (e == cudaSuccess)
    e = cudaMalloc(&a->d_oct_pools, (size_t)a->oct_num_pools * pool_size * sizeof(wgm_octree_task));
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_oct_tree, (size_t)tree_cap);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_oct_ctr, 96);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_oct_locks, (size_t)a->oct_num_pools);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_oct_heads, (size_t)a->oct_num_pools);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_rounds, 1);
  if (e == cudaSuccess) e = cudaMemset(a->d_oct_tree, 0, (size_t)tree_cap * 4);
  if (e == cudaSuccess) e = cudaMemset(a->d_oct_ctr, 0, 96 * 4);
  if (e == cudaSuccess) e = cudaMemset(a->d_rounds, 0, 4);
  if (e == cudaSuccess)
    e = cudaMemcpy(a->d_oct_input, xyzw, n * 16, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(a->d_out, xyzw, n * 16, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    int st = wgm_cuda_fail(rt, e);
    wgm_app_free_buffers(a);
    delete a;
    return st;
  }
  *out = a;
  return WGM_OK;
}

/* Connect-four app (connect_four.h:198-230): nodes for every move sequence
 * up to maxlevel (compute_num_node, connect_four.h:70-77), pools of node ids
 * (min(occupancy bound, 128) of them). */
extern "C" int wgm_c4_create(wgm_runtime *rt, const uint8_t *board, int32_t maxlevel,
                             int32_t pool_size, wgm_app **out) {
  if (!rt || !out || !board || maxlevel < 1 || maxlevel > WGM_C4_MAX_LOOKAHEAD || pool_size < 1)
    return WGM_ERR_INVALID;
  for (int i = 0; i < WGM_C4_CELLS; i++)
    if (board[i] > WGM_C4_COMPUTER) return WGM_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(rt->device);
  wgm_app *a = new (std::nothrow) wgm_app();
  if (!a) return WGM_ERR_OOM;
  a->rt = rt;
  a->kind = WGM_APP_CONNECT_FOUR;
  a->V = WGM_C4_COLS;
  a->c4_maxlevel = maxlevel;
  a->c4_pool_size = pool_size;
  long long nodes = 1, p7 = 1;
  for (int i = 1; i <= maxlevel; i++) {
    p7 *= 7;
    nodes += p7;
  }
  a->c4_num_nodes = (int)nodes;
  int hw = 0;
  int s = wgm_hw_bound_for(rt, WGM_K_C4, wgm_block_size(rt), &hw);
  if (s) {
    delete a;
    return s;
  }
  a->c4_num_pools = std::max(1, std::min(hw, 128));
  a->out_bytes = WGM_C4_COLS * 4;
  cudaError_t e = cudaMalloc(&a->d_out, a->out_bytes);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_c4_board, WGM_C4_CELLS);
  if (e == cudaSuccess) e = cudaMalloc(&a->d_c4_nodes, (size_t)nodes * sizeof(wgm_c4_node));
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_c4_pool, (size_t)a->c4_num_pools * pool_size);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_c4_locks, (size_t)a->c4_num_pools);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_c4_heads, (size_t)a->c4_num_pools);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_c4_ctr, 96);
  if (e == cudaSuccess) e = wgm_dmalloc(&a->d_rounds, 1);
  if (e == cudaSuccess) e = cudaMemset(a->d_c4_ctr, 0, 96 * 4);
  if (e == cudaSuccess) e = cudaMemset(a->d_rounds, 0, 4);
  if (e == cudaSuccess) e = cudaMemset(a->d_out, 0, a->out_bytes);
  if (e == cudaSuccess) e = cudaMemset(a->d_c4_nodes, 0, (size_t)nodes * sizeof(wgm_c4_node));
  if (e == cudaSuccess)
    e = cudaMemcpy(a->d_c4_board, board, WGM_C4_CELLS, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    int st = wgm_cuda_fail(rt, e);
    wgm_app_free_buffers(a);
    delete a;
    return st;
  }
  *out = a;
  return WGM_OK;
}

/* The built tree: entries [0, tree_size), particles done, tasks run. */
extern "C" int wgm_octree_read(wgm_app *a, uint32_t *tree_out, int64_t tree_len,
                               uint32_t *tree_size, uint32_t *done, int32_t *tasks) {
  if (!a || a->kind != WGM_APP_OCTREE) return WGM_ERR_INVALID;
  cudaSetDevice(a->rt->device);
  uint32_t ctr[64];
  int t = 0;
  cudaError_t e = cudaStreamSynchronize(a->rt->stream);
  if (e == cudaSuccess) e = cudaMemcpy(ctr, a->d_oct_ctr, sizeof(ctr), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&t, a->d_rounds, 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return wgm_cuda_fail(a->rt, e);
  const int64_t used = std::min<int64_t>(ctr[0], a->oct_tree_cap);
  if (tree_size) *tree_size = ctr[0];
  if (done) *done = ctr[32];
  if (tasks) *tasks = t;
  if (tree_out) {
    if (tree_len < used) return WGM_ERR_INVALID;
    e = cudaMemcpy(tree_out, a->d_oct_tree, (size_t)used * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return wgm_cuda_fail(a->rt, e);
  }
  return WGM_OK;
}

/* check_persistent_task (octree.h:190-236): the leaf counts of the tree add
 * up to the particle count, and so does particlesDone. */
extern "C" int wgm_octree_check(wgm_app *a, int32_t *ok) {
  if (!a || !ok || a->kind != WGM_APP_OCTREE) return WGM_ERR_INVALID;
  uint32_t size = 0, done = 0;
  int s = wgm_octree_read(a, nullptr, 0, &size, &done, nullptr);
  if (s) return s;
  const int64_t used = std::min<int64_t>(size, a->oct_tree_cap);
  std::vector<uint32_t> tree((size_t)std::max<int64_t>(used, 1));
  s = wgm_octree_read(a, tree.data(), used, nullptr, nullptr, nullptr);
  if (s) return s;
  uint64_t sum = 0;
  for (int64_t i = 0; i < used; i++)
    if (tree[i] & 0x80000000u) sum += tree[i] & 0x7fffffffu;
  *ok = (sum == (uint64_t)a->V && done == (uint32_t)a->V) ? 1 : 0;
  return WGM_OK;
}

extern "C" int wgm_app_read_result(wgm_app *a, void *host_out, size_t bytes) {
  if (a && a->kind == WGM_APP_PLUGIN) {
    if (!host_out || !a->vt.read_result) return WGM_ERR_INVALID;
    cudaSetDevice(a->rt->device);
    return a->vt.read_result(a->vt.user, host_out, bytes);
  }
  if (!a || !host_out || bytes < a->out_bytes) return WGM_ERR_INVALID;
  cudaSetDevice(a->rt->device);
  cudaError_t e =
      cudaMemcpyAsync(host_out, a->d_out, a->out_bytes, cudaMemcpyDeviceToHost, a->rt->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(a->rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(a->rt, e);
  return WGM_OK;
}

extern "C" int wgm_app_result_device_ptr(wgm_app *a, void **p, size_t *bytes) {
  if (!a || !p || a->kind == WGM_APP_PLUGIN) return WGM_ERR_INVALID;
  *p = a->d_out;
  if (bytes) *bytes = a->out_bytes;
  return WGM_OK;
}

extern "C" int wgm_app_rounds(wgm_app *a, int *rounds) {
  if (!a || !rounds) return WGM_ERR_INVALID;
  cudaSetDevice(a->rt->device);
  if (a->kind == WGM_APP_PLUGIN) {
    *rounds = 0;
    return a->vt.rounds ? a->vt.rounds(a->vt.user, rounds) : WGM_OK;
  }
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, a->d_rounds, 4, cudaMemcpyDeviceToHost, a->rt->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(a->rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(a->rt, e);
  *rounds = h;
  return WGM_OK;
}

extern "C" int wgm_app_destroy(wgm_app *a) {
  if (!a) return WGM_ERR_INVALID;
  cudaSetDevice(a->rt->device);
  cudaStreamSynchronize(a->rt->stream);
  if (a->kind == WGM_APP_PLUGIN) {
    if (a->vt.clean) a->vt.clean(a->vt.user);
  } else {
    wgm_app_free_buffers(a);
  }
  delete a;
  return WGM_OK;
}

extern "C" int wgm_app_register(wgm_runtime *rt, const wgm_app_vtable *vt, wgm_app **out) {
  if (!rt || !vt || !out || vt->version != WGM_APP_VTABLE_VERSION || !vt->occupancy ||
      !vt->launch)
    return WGM_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(rt->device);
  wgm_app *a = new (std::nothrow) wgm_app();
  if (!a) return WGM_ERR_OOM;
  a->rt = rt;
  a->kind = WGM_APP_PLUGIN;
  a->vt = *vt;
  if (vt->init) {
    int s = vt->init(vt->user, rt->device);
    if (s) {
      if (vt->clean) vt->clean(vt->user);
      delete a;
      return s;
    }
  }
  *out = a;
  return WGM_OK;
}

extern "C" int wgm_app_check(wgm_app *a, int *ok) {
  if (!a || !ok) return WGM_ERR_INVALID;
  cudaSetDevice(a->rt->device);
  if (a->kind == WGM_APP_OCTREE) return wgm_octree_check(a, ok);
  if (a->kind != WGM_APP_PLUGIN || !a->vt.check) return WGM_ERR_INVALID;
  return a->vt.check(a->vt.user, ok);
}

extern "C" void *wgm_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaHostAlloc(&p, std::max<size_t>(bytes, 1), cudaHostAllocDefault) != cudaSuccess)
    return nullptr;
  return p;
}

extern "C" void wgm_host_free(void *p) {
  if (p) cudaFreeHost(p);
}
