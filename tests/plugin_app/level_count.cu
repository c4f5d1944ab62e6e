/*
 * An app built outside libwgm against include/ alone: a level-synchronous
 * BFS that also counts the vertices of every level.  It shows the app side
 * of the plugin interface - one phase function, the two kernels the runtime
 * launches (standalone and inside the megakernel, where it is resized by
 * offer_kill / offer_fork at every barrier) and the wgm_app_vtable that
 * binds them - the way the reference's apps are written against
 * kernel_merge/stubs/stubs.h and bound through their plugin functions
 * (src/lonestar/graph_apps/bfs/bfs.h:192-370).
 *
 * Build: nvcc -gencode arch=compute_103a,code=sm_103a -std=c++17 -shared
 *        -Xcompiler -fPIC -I include level_count.cu -o liblevel_count.so
 */
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <vector>

#include "wgm_device.cuh"

#define LC_INF 0xffffffffu
#define LC_LINE 32 /* ints per 128-byte line */

struct LevelCount {
  struct Args {
    int V;
    const int *row; /* [V+1] */
    const int *col;
    int source;
    unsigned *dist;   /* [V] output: BFS level, LC_INF if unreached */
    int *level_count; /* [max_levels] output: vertices per level */
    int max_levels;
    int *cnt;         /* 3 lines: frontier sizes by level mod 3 */
    int *rounds;      /* levels run */
  };

  /* Phase (0, 0): init.  Phase (1, r): the vertices of level r claim their
   * unvisited neighbours for level r + 1.  The frontier size of level r is
   * read after the barrier that ended level r - 1; the counter two levels
   * ahead is cleared here (it was last read in level r - 1). */
  static __device__ int phase(wgm_ctx &x, const Args &a, wgm_step cur, wgm_step *nxt) {
    const int tid = wgm_global_id(x), nth = wgm_global_size(x);
    if (cur.target == 0) {
      for (int v = tid; v < a.V; v += nth) a.dist[v] = v == a.source ? 0u : LC_INF;
      for (int l = tid; l < a.max_levels; l += nth) a.level_count[l] = 0;
      if (tid == 0) {
        a.cnt[0] = 1;
        a.cnt[LC_LINE] = 0;
        a.cnt[2 * LC_LINE] = 0;
      }
      *nxt = wgm_step{1, 0};
      return WGM_PHASE_NEXT;
    }
    const int r = cur.round;
    const int frontier = __ldcg(&a.cnt[(r % 3) * LC_LINE]);
    if (frontier == 0 || r >= a.max_levels) {
      if (tid == 0) *a.rounds = r;
      return WGM_PHASE_DONE;
    }
    if (tid == 0) {
      a.level_count[r] = frontier;
      a.cnt[((r + 2) % 3) * LC_LINE] = 0;
    }
    int found = 0;
    for (int v = tid; v < a.V; v += nth) {
      if (__ldcg(&a.dist[v]) != (unsigned)r) continue;
      const int e1 = __ldg(&a.row[v + 1]);
      for (int e = __ldg(&a.row[v]); e < e1; e++)
        if (atomicCAS(&a.dist[__ldg(&a.col[e])], LC_INF, (unsigned)(r + 1)) == LC_INF) found++;
    }
    for (int o = 16; o > 0; o >>= 1) found += __shfl_xor_sync(0xffffffffu, found, o);
    if ((threadIdx.x & 31) == 0 && found) atomicAdd(&a.cnt[((r + 1) % 3) * LC_LINE], found);
    *nxt = wgm_step{1, r + 1};
    return WGM_PHASE_NEXT;
  }
};

using LevelCountKernels = wgm_app_kernels<LevelCount>;

namespace {

struct Host {
  int device = 0;
  std::vector<int> row, col;
  int source = 0;
  LevelCount::Args a{};
};

int lc_init(void *u, int device) {
  Host *h = static_cast<Host *>(u);
  h->device = device;
  if (cudaSetDevice(device) != cudaSuccess) return WGM_ERR_CUDA;
  const int V = (int)h->row.size() - 1;
  const size_t E = h->col.size();
  LevelCount::Args &a = h->a;
  a.V = V;
  a.source = h->source;
  a.max_levels = V + 1;
  int *row = nullptr, *col = nullptr;
  if (cudaMalloc(&row, (V + 1) * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&col, (E ? E : 1) * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&a.dist, V * sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&a.level_count, a.max_levels * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&a.cnt, 3 * LC_LINE * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&a.rounds, sizeof(int)) != cudaSuccess)
    return WGM_ERR_OOM;
  a.row = row;
  a.col = col;
  if (cudaMemcpy(row, h->row.data(), (V + 1) * sizeof(int), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      (E && cudaMemcpy(col, h->col.data(), E * sizeof(int), cudaMemcpyHostToDevice) !=
                cudaSuccess) ||
      cudaMemset(a.rounds, 0, sizeof(int)) != cudaSuccess)
    return WGM_ERR_CUDA;
  return WGM_OK;
}

/* check_persistent_task: the levels and their counts against a host BFS. */
int lc_check(void *u, int *ok) {
  Host *h = static_cast<Host *>(u);
  const int V = h->a.V;
  std::vector<unsigned> dist(V), want(V, LC_INF);
  std::vector<int> counts(h->a.max_levels), want_counts(h->a.max_levels, 0);
  if (cudaMemcpy(dist.data(), h->a.dist, V * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(counts.data(), h->a.level_count, counts.size() * 4, cudaMemcpyDeviceToHost) !=
          cudaSuccess)
    return WGM_ERR_CUDA;
  std::vector<int> q{h->source};
  want[h->source] = 0;
  for (size_t i = 0; i < q.size(); i++) {
    const int v = q[i];
    want_counts[want[v]]++;
    for (int e = h->row[v]; e < h->row[v + 1]; e++) {
      const int w = h->col[e];
      if (want[w] == LC_INF) {
        want[w] = want[v] + 1;
        q.push_back(w);
      }
    }
  }
  *ok = dist == want && counts == want_counts;
  return WGM_OK;
}

/* The output: dist[V] (uint32), then level_count[max_levels] (int32) if the
 * buffer has room. */
int lc_read(void *u, void *out, size_t bytes) {
  Host *h = static_cast<Host *>(u);
  const size_t nd = (size_t)h->a.V * 4, nc = (size_t)h->a.max_levels * 4;
  if (bytes < nd) return WGM_ERR_INVALID;
  if (cudaMemcpy(out, h->a.dist, nd, cudaMemcpyDeviceToHost) != cudaSuccess) return WGM_ERR_CUDA;
  if (bytes >= nd + nc &&
      cudaMemcpy(static_cast<char *>(out) + nd, h->a.level_count, nc, cudaMemcpyDeviceToHost) !=
          cudaSuccess)
    return WGM_ERR_CUDA;
  return WGM_OK;
}

int lc_rounds(void *u, int *rounds) {
  Host *h = static_cast<Host *>(u);
  return cudaMemcpy(rounds, h->a.rounds, 4, cudaMemcpyDeviceToHost) == cudaSuccess ? WGM_OK
                                                                                  : WGM_ERR_CUDA;
}

void lc_clean(void *u) {
  Host *h = static_cast<Host *>(u);
  cudaSetDevice(h->device);
  cudaFree(const_cast<int *>(h->a.row));
  cudaFree(const_cast<int *>(h->a.col));
  cudaFree(h->a.dist);
  cudaFree(h->a.level_count);
  cudaFree(h->a.cnt);
  cudaFree(h->a.rounds);
  delete h;
}

int lc_occupancy(void *, int mega, int block, int *per_sm) {
  return LevelCountKernels::occupancy(mega, block, per_sm);
}

int lc_launch(void *u, const void *launch, int grid, int block, void *stream) {
  return LevelCountKernels::launch(static_cast<Host *>(u)->a, launch, grid, block, stream);
}

int lc_launch_mega(void *u, const void *launch, const void *mega, int grid, int block,
                   void *stream) {
  return LevelCountKernels::launch_mega(static_cast<Host *>(u)->a, launch, mega, grid, block,
                                        stream);
}

}  // namespace

/* The app's table over a host CSR (copied): row[V+1], col[row[V]]. */
extern "C" int level_count_vtable(int V, const int *row, const int *col, int source,
                                  wgm_app_vtable *out) {
  if (V < 1 || !row || !out || source < 0 || source >= V || row[0] != 0 || row[V] < 0 ||
      (row[V] > 0 && !col))
    return WGM_ERR_INVALID;
  Host *h = new (std::nothrow) Host();
  if (!h) return WGM_ERR_OOM;
  h->row.assign(row, row + V + 1);
  h->col.assign(col, col + row[V]);
  for (int c : h->col)
    if (c < 0 || c >= V) {
      delete h;
      return WGM_ERR_INVALID;
    }
  h->source = source;
  std::memset(out, 0, sizeof(*out));
  out->version = WGM_APP_VTABLE_VERSION;
  out->user = h;
  out->app_name = "level_count";
  out->kernel_name = "level_count_phase";
  out->init = lc_init;
  out->check = lc_check;
  out->read_result = lc_read;
  out->rounds = lc_rounds;
  out->clean = lc_clean;
  out->occupancy = lc_occupancy;
  out->launch = lc_launch;
  out->launch_mega = lc_launch_mega;
  return WGM_OK;
}

/* For a table that was never registered (wgm_app_destroy cleans up after a
 * registered one). */
extern "C" void level_count_discard(wgm_app_vtable *vt) {
  if (vt && vt->user) delete static_cast<Host *>(vt->user);
}
