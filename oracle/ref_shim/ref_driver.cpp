/*
 * Host side of the one-work-group shim: plays the reference's host driver
 * (host_skeleton/skel.cpp:316-340 run_persistent, and the per-app plugins'
 * init/reset code) around the reference's own kernel compiled as C++.
 *
 * TEST INFRASTRUCTURE ONLY.  Built per app by oracle/build_ref.py with
 * -DREF_APP_<NAME>; outputs go to oracle/_ref/ only.
 *
 * Inputs arrive as a 0-based CSR (row_ptr[V+1], col[row_ptr[V]]); the driver
 * converts them to the layout each reference plugin uploads.
 */
#include <cstring>
#include <thread>
#include <vector>

#include "cl_shim.h"
#include "rt_common/cl_types.h"
#include "rt_host/discovery.h" /* mk_init_discovery_ctx: the reference's own host init */
#include "rt_common/iw_barrier.h"
#include "rt_common/kernel_ctx.h"
#include "rt_common/cl_scheduler.h"

namespace clshim {
thread_local int lid = 0;
int local_size = 128;
std::barrier<> *wg_barrier = nullptr;
}  // namespace clshim

#define SHIM_SCHEDULER_PARAMS                                                  \
  atomic_int *scheduler_flag, int *scheduler_groups, atomic_int *task_array,   \
      int *task_size, atomic_int *available_workgroups, atomic_int *pool_lock, \
      atomic_int *groups_to_kill, atomic_int *persistent_flag,                 \
      Restoration_ctx *r_ctx_arr, atomic_int *check_value

/* Scheduler context in host memory, initialised as restart_scheduler does
 * (rt_host/cl_scheduler.h:35-50). */
struct ShimScheduler {
  atomic_int scheduler_flag{DEVICE_SCHEDULER_INIT};
  int participating_groups = 0;
  atomic_int task_array[MAX_P_GROUPS];
  int task_size = 0;
  atomic_int available_workgroups{0};
  atomic_int pool_lock{0};
  atomic_int groups_to_kill{0};
  atomic_int persistent_flag{-1};
  Restoration_ctx r_ctx_arr[MAX_P_GROUPS];
  atomic_int check_value{-1};
  ShimScheduler() {
    for (int i = 0; i < MAX_P_GROUPS; i++) {
      task_array[i].store(TASK_UNINIT);
      std::memset(&r_ctx_arr[i], 0, sizeof(Restoration_ctx));
      r_ctx_arr[i].target = 0;
    }
  }
};

#define SHIM_SCHEDULER_ARGS(s)                                              \
  &(s).scheduler_flag, &(s).participating_groups, (s).task_array,           \
      &(s).task_size, &(s).available_workgroups, &(s).pool_lock,            \
      &(s).groups_to_kill, &(s).persistent_flag, (s).r_ctx_arr,             \
      &(s).check_value

/* reset_barrier (host_skeleton/skel.cpp:127-141). */
static void shim_reset_barrier(IW_barrier *b) {
  for (int i = 0; i < MAX_P_GROUPS; i++) b->barrier_flags[i].store(0);
  b->phase.store(0);
  b->num_groups = 0;
  b->to_kill = 0;
  b->counter.store(0);
  b->sense.store(0);
}

/* Launch one work-group of `wgs` work-items running `body`, while this thread
 * plays the host handshake of skel.cpp:336-339. */
template <typename F>
static void shim_launch_persistent(int wgs, ShimScheduler &s, F body) {
  std::barrier<> bar(wgs);
  clshim::local_size = wgs;
  clshim::wg_barrier = &bar;
  std::vector<std::thread> items;
  items.reserve(wgs);
  for (int t = 0; t < wgs; t++)
    items.emplace_back([t, &body] {
      clshim::lid = t;
      body();
    });
  while (s.scheduler_flag.load(std::memory_order_acquire) != DEVICE_WAITING) {
    std::this_thread::yield();
  }
  s.scheduler_flag.store(DEVICE_TO_PERSISTENT_TASK, std::memory_order_release);
  while (s.persistent_flag.load(std::memory_order_acquire) != 0) {
    std::this_thread::yield();
  }
  for (auto &th : items) th.join();
  clshim::wg_barrier = nullptr;
}

template <typename F>
static void shim_launch_plain(int wgs, F body) {
  std::barrier<> bar(wgs);
  clshim::local_size = wgs;
  clshim::wg_barrier = &bar;
  std::vector<std::thread> items;
  for (int t = 0; t < wgs; t++)
    items.emplace_back([t, &body] {
      clshim::lid = t;
      body();
    });
  for (auto &th : items) th.join();
  clshim::wg_barrier = nullptr;
}

#define REF_INF 1000000000u /* lonestar/graph_apps/bfs/bfs.h:14 */

#if defined(REF_APP_LONESTAR_BFS) || defined(REF_APP_LONESTAR_SSSP)
void drelax2(uint *dist, int *a_inwl_index, int *a_outwl_index, int *a_inwl_wl,
             int *a_outwl_wl, uint g_nnodes, uint *g_edgessrcdst, uint *g_psrc,
#ifdef REF_APP_LONESTAR_SSSP
             uint *g_edgessrcwt,
#endif
             IW_barrier *__bar, Discovery_ctx *__d_ctx, SHIM_SCHEDULER_PARAMS);

extern "C" int ref_run_lonestar(int V, const int *row_ptr, const int *col,
                                const unsigned *wt, unsigned *dist_out, int wgs) {
  int E = row_ptr[V];
  if (E < 1) E = 1;
  /* bfs.h:40-46 / 137-161: 1-based psrc with psrc[nnodes] = nedges and
   * edgessrcdst[0] unused. */
  std::vector<uint> psrc(V + 1), dst(E + 1, 0), w(E + 1, 0), dist(V);
  for (int i = 0; i <= V; i++) psrc[i] = (uint)row_ptr[i] + 1u;
  for (int k = 0; k < row_ptr[V]; k++) {
    dst[k + 1] = (uint)col[k];
    if (wt) w[k + 1] = wt[k];
  }
  /* bfs.h:250-271: dist = MYINFINITY, dist[0] = 0, both indices 0,
   * worklists of nedges entries. */
  for (int i = 0; i < V; i++) dist[i] = REF_INF;
  dist[0] = 0;
  int in_index = 0, out_index = 0;
  std::vector<int> in_wl(E + 1), out_wl(E + 1);
  auto *bar = new IW_barrier;
  shim_reset_barrier(bar);
  auto *d_ctx = new Discovery_ctx;
  mk_init_discovery_ctx(d_ctx);
  auto *s = new ShimScheduler;
  shim_launch_persistent(wgs, *s, [&] {
    drelax2(dist.data(), &in_index, &out_index, in_wl.data(), out_wl.data(),
            (uint)V, dst.data(), psrc.data(),
#ifdef REF_APP_LONESTAR_SSSP
            w.data(),
#endif
            bar, d_ctx, SHIM_SCHEDULER_ARGS(*s));
  });
  std::memcpy(dist_out, dist.data(), sizeof(uint) * V);
  int count = d_ctx->count;
  delete bar;
  delete d_ctx;
  delete s;
  return count;
}
#endif

#ifdef REF_APP_PANNOTIA_COLOR
void color_combined(int *row, int *col, float *node_value, int *color_array,
                    int *stop1, int *stop2, float *max_d, const int num_nodes,
                    const int num_edges, IW_barrier *__bar,
                    Discovery_ctx *__d_ctx, SHIM_SCHEDULER_PARAMS);

extern "C" int ref_run_color(int V, const int *row_ptr, const int *col,
                             const float *node_value, int *color_out, int wgs) {
  int E = row_ptr[V];
  /* color.h:45-80: color = -1; max_d receives the bytes of the int -1 array;
   * row gets num_nodes entries. */
  std::vector<int> row(row_ptr, row_ptr + V), cols(col, col + E), color(V, -1);
  std::vector<float> nv(node_value, node_value + V), max_d(V);
  for (int i = 0; i < V; i++) {
    int m1 = -1;
    std::memcpy(&max_d[i], &m1, sizeof(float));
  }
  int stop1 = 0, stop2 = 0;
  auto *bar = new IW_barrier;
  shim_reset_barrier(bar);
  auto *d_ctx = new Discovery_ctx;
  mk_init_discovery_ctx(d_ctx);
  auto *s = new ShimScheduler;
  shim_launch_persistent(wgs, *s, [&] {
    color_combined(row.data(), cols.data(), nv.data(), color.data(), &stop1,
                   &stop2, max_d.data(), V, E, bar, d_ctx, SHIM_SCHEDULER_ARGS(*s));
  });
  std::memcpy(color_out, color.data(), sizeof(int) * V);
  int count = d_ctx->count;
  delete bar;
  delete d_ctx;
  delete s;
  return count;
}
#endif

#ifdef REF_APP_PANNOTIA_MIS
void mis_combined(int *row, int *col, float *node_value, int *s_array,
                  int *c_array, int *cu_array, float *min_array, int *stop,
                  int num_nodes, int num_edges, IW_barrier *__bar,
                  Discovery_ctx *__d_ctx, SHIM_SCHEDULER_PARAMS);

extern "C" int ref_run_mis(int V, const int *row_ptr, const int *col,
                           const float *node_value, int *s_out, int wgs) {
  int E = row_ptr[V];
  /* mis.h:58-92 */
  std::vector<int> row(row_ptr, row_ptr + V), cols(col, col + E), s_arr(V, 0),
      c(V, -1), cu(V, -1);
  std::vector<float> nv(node_value, node_value + V), min_array(V, 6666666.0f);
  int stop = 0;
  auto *bar = new IW_barrier;
  shim_reset_barrier(bar);
  auto *d_ctx = new Discovery_ctx;
  mk_init_discovery_ctx(d_ctx);
  auto *s = new ShimScheduler;
  shim_launch_persistent(wgs, *s, [&] {
    mis_combined(row.data(), cols.data(), nv.data(), s_arr.data(), c.data(),
                 cu.data(), min_array.data(), &stop, V, E, bar, d_ctx,
                 SHIM_SCHEDULER_ARGS(*s));
  });
  std::memcpy(s_out, s_arr.data(), sizeof(int) * V);
  int count = d_ctx->count;
  delete bar;
  delete d_ctx;
  delete s;
  return count;
}
#endif

#ifdef REF_APP_PANNOTIA_SSSP
void sssp_combined(const int num_rows, int *row, int *col, int *data, int *x,
                   int *y, int *stop, IW_barrier *__bar, Discovery_ctx *__d_ctx,
                   SHIM_SCHEDULER_PARAMS);

extern "C" int ref_run_pannotia_sssp(int V, const int *row_ptr, const int *col,
                                     const int *data, int *cost_out, int wgs) {
  int E = row_ptr[V];
  /* pannotia/graph_apps/sssp/sssp.h:54-80: x = y = BIG_NUM except source 0. */
  std::vector<int> row(row_ptr, row_ptr + V + 1), cols(col, col + E),
      dat(data, data + E), x(V, 99999999), y(V, 99999999);
  if (V > 0) x[0] = y[0] = 0;
  int stop = 0;
  auto *bar = new IW_barrier;
  shim_reset_barrier(bar);
  auto *d_ctx = new Discovery_ctx;
  mk_init_discovery_ctx(d_ctx);
  auto *s = new ShimScheduler;
  shim_launch_persistent(wgs, *s, [&] {
    sssp_combined(V, row.data(), cols.data(), dat.data(), x.data(), y.data(),
                  &stop, bar, d_ctx, SHIM_SCHEDULER_ARGS(*s));
  });
  std::memcpy(cost_out, x.data(), sizeof(int) * V); /* sssp.h:168 reads x */
  int count = d_ctx->count;
  delete bar;
  delete d_ctx;
  delete s;
  return count;
}
#endif

#ifdef REF_APP_MATMULT
void matmult(int *A, const int A_row, const int A_col, int *B, const int B_row,
             const int B_col, int *C, atomic_int *counter, atomic_int *hash);

extern "C" int ref_run_matmult(const int *A, int A_row, int A_col, const int *B,
                               int B_row, int B_col, int *C_out, int wgs) {
  std::vector<int> a(A, A + (size_t)A_row * A_col), b(B, B + (size_t)B_row * B_col),
      c((size_t)A_row * B_col, 0);
  atomic_int counter{0}, hash{0}; /* matmult.h:226-227 */
  shim_launch_plain(wgs, [&] {
    matmult(a.data(), A_row, A_col, b.data(), B_row, B_col, c.data(), &counter,
            &hash);
  });
  std::memcpy(C_out, c.data(), sizeof(int) * c.size());
  return hash.load();
}
#endif

#ifdef REF_APP_REDUCE
void MY_reduce(int *buffer, int length, atomic_int *result);

extern "C" int ref_run_reduce(const int *buf, int length, int wgs) {
  std::vector<int> b(buf, buf + length);
  atomic_int result{INT_MAX}; /* reduce.h:346 */
  shim_launch_plain(wgs, [&] { MY_reduce(b.data(), length, &result); });
  return result.load();
}
#endif
