/*
 * Internal host-side structures of libwgm (not part of the C-ABI).
 */
#ifndef WGM_INTERNAL_H
#define WGM_INTERNAL_H

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/wgm.h"
#include "wgm_common.h"
#include "wgm_device.cuh"

struct wgm_runtime {
  wgm_config cfg{};
  int device = -1;
  cudaDeviceProp prop{};
  cudaStream_t stream = nullptr;
  wgm_dev_state *st = nullptr;        /* device */
  wgm_host_flags *hf = nullptr;       /* mapped pinned host memory */
  wgm_host_flags *hf_dev = nullptr;   /* its device alias */
  char *d_scratch = nullptr;          /* 64 bytes of small kernel outputs */
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t tev0 = nullptr, tev1 = nullptr; /* wgm_timer_* */
  int gen = 1;                        /* launch generation */
  int last_cuda = 0;
  int last_status = 0, last_site = 0, last_detail = 0; /* last device failure */
};

/* Static hub layout on the device (see wgm_hubs in wgm_graph.cuh). */
struct wgm_dev_hubs {
  int *ids = nullptr, *prefix = nullptr, *wmap = nullptr;
  int H = 0, total = 0;
};

struct wgm_app {
  wgm_runtime *rt = nullptr;
  int kind = 0;
  wgm_app_vtable vt{}; /* kind == WGM_APP_PLUGIN: the registered app's table */
  int V = 0;
  int64_t E = 0;
  int hub_threshold = 256;
  /* graph */
  int *d_row = nullptr, *d_col = nullptr;
  uint32_t *d_wt = nullptr; /* Lonestar SSSP weights / Pannotia SSSP data */
  float *d_node_value = nullptr;
  wgm_dev_hubs hubs;
  /* outputs and scratch */
  void *d_out = nullptr;
  size_t out_bytes = 0;
  int *d_wl_start = nullptr, *d_wl_cnt = nullptr, *d_wl_u = nullptr; /* Lonestar pieces */
  int wl_cap = 0, piece = 32;
  int *d_cnt = nullptr, *d_stamp = nullptr, *d_stop = nullptr;
  int *d_hub_acc = nullptr, *d_status = nullptr;
  float *d_contrib = nullptr, *d_dang = nullptr, *d_hub_sum = nullptr;
  int *d_rounds = nullptr;
  /* colour: in-edge CSR when the graph is not symmetric (else the graph) */
  int *d_trow = nullptr, *d_tcol = nullptr;
  int2 *d_tcv = nullptr; /* colour: in-edges beside their neighbour's value */
  /* colour without rounds (standalone runs, color_mode 1): allocated at the
   * first such run */
  int color_mode = 0;
  int bfs_mode = -1; /* Lonestar BFS: -1 automatic, 0 grid, 1 one CTA */
  int4 *d_tcv4 = nullptr;
  int *d_cmax = nullptr, *d_cq = nullptr, *d_cqctl = nullptr;
  int cq_cap = 0;
  int source = 0;
  float damping = 0.85f;
  float dang0 = 0.f;
  int iterations = 20;
  int bc_sources = 0; /* betweenness centrality: sources 0 .. bc_sources-1 */
  int bc_mode = 0;    /* 0: one source at a time over the grid, 1: sources over CTAs */
  bool has_node_values = false;
  /* octree (WGM_APP_OCTREE): d_out holds the particles, V their count */
  void *d_oct_input = nullptr, *d_oct_second = nullptr, *d_oct_pools = nullptr;
  unsigned *d_oct_tree = nullptr, *d_oct_ctr = nullptr; /* ctr: tree size, done */
  int *d_oct_locks = nullptr, *d_oct_heads = nullptr;
  long long oct_tree_cap = 0;
  int oct_maxchilds = 5, oct_num_pools = 0, oct_pool_size = 0;
  /* connect four (WGM_APP_CONNECT_FOUR): d_out holds next_move_value[7] */
  unsigned char *d_c4_board = nullptr;
  void *d_c4_nodes = nullptr;
  int *d_c4_pool = nullptr, *d_c4_locks = nullptr, *d_c4_heads = nullptr;
  int *d_c4_ctr = nullptr; /* node head, root done, offer lock: one line each */
  int c4_maxlevel = 6, c4_num_nodes = 0, c4_num_pools = 0, c4_pool_size = 0;
};

int wgm_cuda_fail(wgm_runtime *rt, cudaError_t e);
wgm_launch wgm_make_launch(wgm_runtime *rt, int grid, int handshake, int im_exit);
int wgm_hw_bound_for(wgm_runtime *rt, int kid, int block, int *groups);
int wgm_status_from_device(int dev);
int wgm_finish_launch(wgm_runtime *rt, int *dev_status, int *dev_site);
bool wgm_host_wait(const volatile int32_t *p, int want, bool equal, uint64_t timeout_ns);
int wgm_kind_to_kernel(int app_kind);
int wgm_stream_wait(wgm_runtime *rt, cudaStream_t stream);
struct wgm_mega_args;
int wgm_app_fill_mega(wgm_app *a, wgm_mega_args *A);
int wgm_plugin_hw_bound(wgm_app *a, int mega, int block, int *groups);

#endif
