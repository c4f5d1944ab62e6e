/*
 * The megakernel (wgm_k_mega) and its host side, the communicator
 * (include/wgm.h "megakernel and communicator").
 *
 * Host side follows src/scheduler_rt/rt_host/cl_communicator.h:19-465 and
 * src/host_skeleton/skel.cpp:387-463 (launch, persistent task with a monitor
 * thread, synchronous non-persistent tasks with response/execution timing,
 * redlines, quit, the merged iteration loop); errors are status codes instead
 * of exit(), and every host wait has a deadline.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/wgm.h"
#include "wgm_internal.h"
#include "wgm_kernels.cuh"
#include "wgm_mega.cuh"

/* ------------------------------------------------------------------------ */
/* Kernel                                                                    */
/* ------------------------------------------------------------------------ */

/* Offers of a task loop without barriers (octree.cl:172-181,
 * connect_four.cl:401-407), thread 0 at the top of every iteration:
 * persistent group 0 offers a fork into the loop (restoration target 1),
 * the others offer to be killed.  With no barrier to separate them, a kill
 * could land between a fork's read of the group count and its growth and
 * leave a hole in the group ids (no group would ever again be "the highest",
 * and the scheduler would wait for kills forever), so both hold the app's
 * own lock (a busy lock only defers the offer).  Not the scheduler's pool
 * lock: the scheduler holds that while it waits for the kills.  Returns true
 * when this group must leave. */
__device__ __forceinline__ bool wgm_task_offer(const wgm_launch &L, wgm_cta *cx, int *rlock) {
  if (!wgm_try_lock(rlock)) return false;
  bool killed = false;
  if (cx->id == 0) {
    wgm_rctx rc;
    for (int k = 0; k < WGM_RCTX_WORDS; k++) rc.w[k] = 0;
    rc.w[WGM_RC_TARGET] = 1;
    rc.w[WGM_RC_GEN] = cx->gen;
    wgm_offer_fork(L, -1, rc);
  } else {
    killed = wgm_offer_kill(L, cx->id);
  }
  wgm_unlock(rlock);
  return killed;
}

template <class Sync>
__device__ __forceinline__ void wgm_mega_run_app(const wgm_launch &L, const wgm_mega_args &A,
                                                 wgm_cta *pc, wgm_warp_smem *sm, wgm_step start,
                                                 Sync &&sync) {
  switch (A.app) {
    case WGM_K_BFS:
      wgm_drive(L, pc, start, sync, [&](wgm_step cur, wgm_step *nxt) {
        return wgm_phase_lonestar<false>(L, pc, A.ls, sm, cur.target, cur.round, &nxt->target,
                                         &nxt->round);
      });
      break;
    case WGM_K_SSSP:
      wgm_drive(L, pc, start, sync, [&](wgm_step cur, wgm_step *nxt) {
        return wgm_phase_lonestar<true>(L, pc, A.ls, sm, cur.target, cur.round, &nxt->target,
                                        &nxt->round);
      });
      break;
    case WGM_K_COLOR:
      wgm_drive(L, pc, start, sync, [&](wgm_step cur, wgm_step *nxt) {
        return wgm_phase_color(L, pc, A.color, sm, cur, nxt);
      });
      break;
    case WGM_K_MIS:
      wgm_drive(L, pc, start, sync, [&](wgm_step cur, wgm_step *nxt) {
        return wgm_phase_mis(L, pc, A.mis, sm, cur, nxt);
      });
      break;
    case WGM_K_PSSSP:
      wgm_drive(L, pc, start, sync, [&](wgm_step cur, wgm_step *nxt) {
        return wgm_phase_pannotia_sssp(L, pc, A.psssp, sm, cur, nxt);
      });
      break;
    case WGM_K_PAGERANK:
      wgm_drive(L, pc, start, sync, [&](wgm_step cur, wgm_step *nxt) {
        return wgm_phase_pagerank(L, pc, A.pr, sm, cur, nxt);
      });
      break;
    case WGM_K_BC:
      wgm_drive(L, pc, start, sync, [&](wgm_step cur, wgm_step *nxt) {
        return wgm_phase_bc(L, pc, A.bc, sm, cur, nxt);
      });
      break;
    case WGM_K_OCTREE:
      /* octree.cl:170-180: init and one resizing barrier, then the task
       * loop with an offer at the top of every iteration */
      if (start.target == 0) {
        wgm_octree_init(L, pc, A.oct);
        if (!sync(L, pc, wgm_step{1, 0})) break;
      }
      wgm_octree_loop(L, pc, A.oct, [&](wgm_cta *cx) { return wgm_task_offer(L, cx, A.oct.rlock); });
      break;
    case WGM_K_C4: /* connect_four.cl:397-415: the same shape as the octree */
      if (start.target == 0) {
        wgm_c4_init(L, pc, A.c4);
        if (!sync(L, pc, wgm_step{1, 0})) break;
      }
      wgm_c4_loop(L, pc, A.c4, [&](wgm_cta *cx) { return wgm_task_offer(L, cx, A.c4.rlock); });
      break;
    default:
      break;
  }
}

/* The built-in megakernel: the worker loop of wgm_device.cuh around the
 * built-in apps' phase functions. */
__global__ void __launch_bounds__(1024) wgm_k_mega(wgm_launch L, wgm_mega_args A) {
  __shared__ wgm_warp_smem sm;
  wgm_mega_body(L, A.ctl, [&](wgm_cta *pc, wgm_step start, auto &sync) {
    wgm_mega_run_app(L, A, pc, &sm, start, sync);
  });
}

/* ------------------------------------------------------------------------ */
/* Communicator                                                              */
/* ------------------------------------------------------------------------ */

using wgm_clock = std::chrono::steady_clock;
static uint64_t wgm_now_ns() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             wgm_clock::now().time_since_epoch())
      .count();
}

/* Results of the non-persistent task, in mapped host memory. */
struct wgm_np_host {
  int32_t hash;
  int32_t result;
};

struct wgm_comm {
  wgm_runtime *rt = nullptr;
  wgm_app *papp = nullptr;
  int np_kind = 0, np_size = 0;
  cudaStream_t side = nullptr; /* copies while the megakernel runs */
  int *dA = nullptr, *dB = nullptr, *dC = nullptr, *dbuf = nullptr;
  float *dAf = nullptr, *dBf = nullptr, *dCf = nullptr, *dbuff = nullptr;
  wgm_np_host *np_host = nullptr, *np_dev = nullptr;
  int ref_hash = 0, ref_min = 0;
  std::vector<float> Af, Bf;
  /* CL_Communicator state (cl_communicator.h:21-38) */
  int participating_groups = 0;
  std::atomic<int> executing_persistent{0};
  std::atomic<int> waiting_for_async{0};
  std::atomic<int> monitor_status{0};
  uint64_t persistent_begin = 0, persistent_end = 0, global_start = 0;
  std::vector<std::pair<uint64_t, int>> time_groups_data;
  std::vector<std::tuple<uint64_t, uint64_t, uint64_t>> response_exec_data;
  std::vector<uint64_t> response_times, execution_times;
  int redlines = 0;
  int non_persistent_wgs = 0;
  bool launched = false;
  std::thread monitor;
};

static int wgm_comm_fail(wgm_comm *c, cudaError_t e) { return wgm_cuda_fail(c->rt, e); }

/* matmult.h:107-119 middle-square fill (the reference's host generator). */
static int wgm_rand_fill(int *M, int n, int seed) {
  for (int i = 0; i < n * n; i++) {
    seed = (int)((unsigned)seed * (unsigned)seed);
    seed = (seed / 1000) % 1000000;
    M[i] = seed % 10;
  }
  return seed;
}

static int wgm_np_init(wgm_comm *c) {
  cudaError_t e = cudaSuccess;
  const int kind = c->np_kind, n = c->np_size;
  if (cudaHostAlloc((void **)&c->np_host, sizeof(wgm_np_host), cudaHostAllocMapped) !=
      cudaSuccess)
    return WGM_ERR_OOM;
  c->np_host->hash = 0;
  c->np_host->result = INT_MAX;
  if ((e = cudaHostGetDevicePointer((void **)&c->np_dev, c->np_host, 0)) != cudaSuccess)
    return wgm_comm_fail(c, e);
  if (kind == WGM_NP_MATMULT_I32 || kind == WGM_NP_MATMULT_F32) {
    if (n < 1 || n > 4096) return WGM_ERR_INVALID;
    std::vector<int> A((size_t)n * n), B((size_t)n * n), C((size_t)n * n);
    int seed = wgm_rand_fill(A.data(), n, 1234); /* matmult.h:73,190 */
    wgm_rand_fill(B.data(), n, seed);
    /* host_matrix_multiply + hash_mat (matmult.h:123-159,214-218) */
    for (int r = 0; r < n; r++)
      for (int cc = 0; cc < n; cc++) {
        unsigned acc = 0;
        for (int j = 0; j < n; j++)
          acc += (unsigned)A[(size_t)r * n + j] * (unsigned)B[(size_t)j * n + cc];
        C[(size_t)r * n + cc] = (int)acc;
      }
    unsigned h = 5381;
    for (int i = 0; i < n; i++) h = h * 33u + (unsigned)C[(size_t)i * n + i];
    c->ref_hash = (int)h;
    size_t bytes = (size_t)n * n * 4;
    if (kind == WGM_NP_MATMULT_I32) {
      if ((e = cudaMalloc(&c->dA, bytes)) || (e = cudaMalloc(&c->dB, bytes)) ||
          (e = cudaMalloc(&c->dC, bytes)) ||
          (e = cudaMemcpy(c->dA, A.data(), bytes, cudaMemcpyHostToDevice)) ||
          (e = cudaMemcpy(c->dB, B.data(), bytes, cudaMemcpyHostToDevice)))
        return wgm_comm_fail(c, e);
    } else {
      c->Af.resize((size_t)n * n);
      c->Bf.resize((size_t)n * n);
      for (size_t i = 0; i < A.size(); i++) {
        c->Af[i] = (float)A[i] * 0.125f;
        c->Bf[i] = (float)B[i] * 0.125f;
      }
      if ((e = cudaMalloc(&c->dAf, bytes)) || (e = cudaMalloc(&c->dBf, bytes)) ||
          (e = cudaMalloc(&c->dCf, bytes)) ||
          (e = cudaMemcpy(c->dAf, c->Af.data(), bytes, cudaMemcpyHostToDevice)) ||
          (e = cudaMemcpy(c->dBf, c->Bf.data(), bytes, cudaMemcpyHostToDevice)))
        return wgm_comm_fail(c, e);
    }
  } else if (kind == WGM_NP_REDUCE_I32 || kind == WGM_NP_REDUCE_F32) {
    if (n < 1) return WGM_ERR_INVALID;
    /* reduce.h:331-340: values rand()+1, host keeps the min.  A seeded
     * SplitMix64 stream stands in for glibc rand(). */
    std::vector<int> buf(n);
    uint64_t x = 0x9e3779b97f4a7c15ull;
    int mn = INT_MAX;
    for (int i = 0; i < n; i++) {
      x += 0x9e3779b97f4a7c15ull;
      uint64_t z = x;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      z ^= z >> 31;
      buf[i] = (int)(z % 2147483646ull) + 1;
      mn = std::min(mn, buf[i]);
    }
    c->ref_min = mn;
    size_t bytes = (size_t)n * 4;
    if (kind == WGM_NP_REDUCE_I32) {
      if ((e = cudaMalloc(&c->dbuf, bytes)) ||
          (e = cudaMemcpy(c->dbuf, buf.data(), bytes, cudaMemcpyHostToDevice)))
        return wgm_comm_fail(c, e);
    } else {
      std::vector<float> bf(n);
      float fm = 3.0e38f;
      for (int i = 0; i < n; i++) {
        bf[i] = (float)buf[i] / 2147483648.0f;
        fm = std::min(fm, bf[i]);
      }
      std::memcpy(&c->ref_min, &fm, 4);
      if ((e = cudaMalloc(&c->dbuff, bytes)) ||
          (e = cudaMemcpy(c->dbuff, bf.data(), bytes, cudaMemcpyHostToDevice)))
        return wgm_comm_fail(c, e);
    }
  } else if (kind != 0) {
    return WGM_ERR_INVALID;
  }
  /* the copies above come from pageable memory and may still be in flight
   * when cudaMemcpy returns; the megakernel runs on a non-blocking stream */
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return wgm_comm_fail(c, e);
  return WGM_OK;
}

extern "C" int wgm_comm_create(wgm_runtime *rt, wgm_app *persistent, int np_kind, int np_size,
                               wgm_comm **out) {
  if (!rt || !out || (persistent && persistent->rt != rt)) return WGM_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(rt->device);
  wgm_comm *c = new (std::nothrow) wgm_comm();
  if (!c) return WGM_ERR_OOM;
  c->rt = rt;
  c->papp = persistent;
  c->np_kind = np_kind;
  c->np_size = np_size;
  int s = WGM_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  if (e != cudaSuccess) s = wgm_comm_fail(c, e);
  if (s == WGM_OK) s = wgm_np_init(c);
  if (s) {
    wgm_comm_destroy(c);
    return s;
  }
  *out = c;
  return WGM_OK;
}

static void wgm_comm_join(wgm_comm *c) {
  if (c->monitor.joinable()) c->monitor.join();
}

extern "C" int wgm_comm_destroy(wgm_comm *c) {
  if (!c) return WGM_ERR_INVALID;
  cudaSetDevice(c->rt->device);
  if (c->launched) {
    wgm_comm_send_quit(c);
    wgm_comm_finish(c);
  }
  wgm_comm_join(c);
  void *ptrs[] = {c->dA, c->dB, c->dC, c->dbuf, c->dAf, c->dBf, c->dCf, c->dbuff};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (c->np_host) cudaFreeHost(c->np_host);
  if (c->side) cudaStreamDestroy(c->side);
  delete c;
  return WGM_OK;
}

static void wgm_store_flag(wgm_comm *c, int v) {
  __atomic_store_n(&c->rt->hf->scheduler_flag, v, __ATOMIC_RELEASE);
}
static uint64_t wgm_idle_budget(wgm_comm *c) {
  uint64_t t = c->rt->cfg.run_timeout_ns ? c->rt->cfg.run_timeout_ns : 120000000000ull;
  return t;
}

/* launch_mega_kernel (cl_communicator.h:71-95) */
extern "C" int wgm_comm_launch_mega_kernel(wgm_comm *c, int num_wgs) {
  if (!c || c->launched) return c ? WGM_ERR_STATE : WGM_ERR_INVALID;
  wgm_runtime *rt = c->rt;
  cudaSetDevice(rt->device);
  wgm_comm_join(c);
  int block = rt->cfg.threads_per_wg;
  if (block < 32 || block > 1024 || block % 32) block = 256;
  /* a registered app brings its own megakernel (wgm_app_mega_kernel) */
  const bool plugin = c->papp && c->papp->kind == WGM_APP_PLUGIN;
  if (plugin && !c->papp->vt.launch_mega) return WGM_ERR_INVALID;
  int per_sm = 0, hw = 0;
  cudaError_t e = cudaSuccess;
  if (plugin) {
    int s = wgm_plugin_hw_bound(c->papp, 1, block, &hw);
    if (s) return s;
  } else {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wgm_k_mega, block, 0);
    if (e != cudaSuccess) return wgm_comm_fail(c, e);
    hw = std::min(per_sm * rt->prop.multiProcessorCount, WGM_MAX_GROUPS);
  }
  int grid = num_wgs > 0 ? std::min(num_wgs, hw) : hw;
  if (grid < 2) return WGM_ERR_INVALID;
  wgm_mega_args A;
  std::memset(&A, 0, sizeof(A));
  A.app = -1;
  if (c->papp && !plugin) {
    int s = wgm_app_fill_mega(c->papp, &A);
    if (s) return s;
  }
  A.ctl.np.kind = c->np_kind;
  A.ctl.np.n = c->np_size;
  A.ctl.np.A = c->dA;
  A.ctl.np.B = c->dB;
  A.ctl.np.C = c->dC;
  A.ctl.np.Af = c->dAf;
  A.ctl.np.Bf = c->dBf;
  A.ctl.np.Cf = c->dCf;
  A.ctl.np.buf = c->dbuf;
  A.ctl.np.buff = c->dbuff;
  A.ctl.np.len = c->np_size;
  A.ctl.np.hash = &c->np_dev->hash;
  A.ctl.np.result = &c->np_dev->result;
  A.ctl.idle_ns = wgm_idle_budget(c);
  A.ctl.use_query_barrier = rt->cfg.use_query_barrier;
  /* restart_scheduler (rt_host/cl_scheduler.h:35-50) for the host words */
  __atomic_store_n(&rt->hf->persistent_flag, -1, __ATOMIC_RELEASE);
  __atomic_store_n(&rt->hf->participating_groups, 0, __ATOMIC_RELEASE);
  wgm_store_flag(c, WGM_DEVICE_SCHEDULER_INIT);
  wgm_launch L = wgm_make_launch(rt, grid, 0, 0);
  if (plugin) {
    if (c->papp->vt.reset) {
      int s = c->papp->vt.reset(c->papp->vt.user, rt->stream);
      if (s) return s;
    }
    int s = c->papp->vt.launch_mega(c->papp->vt.user, &L, &A.ctl, grid, block, rt->stream);
    if (s) return s == WGM_ERR_CUDA ? wgm_comm_fail(c, cudaErrorLaunchFailure) : s;
  } else {
    wgm_k_mega<<<grid, block, 0, rt->stream>>>(L, A);
    if ((e = cudaGetLastError()) != cudaSuccess) return wgm_comm_fail(c, e);
  }
  c->launched = true;
  uint64_t budget = rt->cfg.spin_timeout_ns ? rt->cfg.spin_timeout_ns * 4 : 8000000000ull;
  if (!wgm_host_wait(&rt->hf->scheduler_flag, WGM_DEVICE_WAITING, true, budget)) {
    wgm_set_abort(rt, 1);
    wgm_comm_finish(c);
    return WGM_ERR_TIMEOUT;
  }
  c->participating_groups = __atomic_load_n(&rt->hf->participating_groups, __ATOMIC_ACQUIRE);
  return WGM_OK;
}

extern "C" int wgm_comm_number_of_discovered_groups(wgm_comm *c, int *groups) {
  if (!c || !groups) return WGM_ERR_INVALID;
  *groups = c->participating_groups;
  return WGM_OK;
}

extern "C" int wgm_comm_send_quit(wgm_comm *c) {
  if (!c) return WGM_ERR_INVALID;
  wgm_store_flag(c, WGM_DEVICE_TO_QUIT);
  return WGM_OK;
}

/* Wait for the megakernel to exit and report its status. */
extern "C" int wgm_comm_finish(wgm_comm *c) {
  if (!c) return WGM_ERR_INVALID;
  cudaSetDevice(c->rt->device);
  int s = WGM_OK;
  if (c->launched) {
    s = wgm_stream_wait(c->rt, c->rt->stream);
    int f = wgm_finish_launch(c->rt, nullptr, nullptr);
    if (!s) s = f;
    c->launched = false;
  }
  wgm_comm_join(c);
  int m = c->monitor_status.load();
  if (!s && m) s = m;
  return s;
}

/* monitor_persistent_task (cl_communicator.h:168-205) */
static void wgm_monitor(wgm_comm *c, int groups) {
  wgm_runtime *rt = c->rt;
  uint64_t budget = wgm_idle_budget(c);
  __atomic_store_n(&rt->hf->task_size, groups, __ATOMIC_RELEASE);
  wgm_store_flag(c, WGM_DEVICE_TO_PERSISTENT_TASK);
  if (!wgm_host_wait(&rt->hf->scheduler_flag, WGM_DEVICE_GOT_GROUPS, true, budget)) {
    c->monitor_status = WGM_ERR_TIMEOUT;
    c->waiting_for_async = 0;
    return;
  }
  c->persistent_begin = wgm_now_ns();
  c->global_start = c->persistent_begin;
  wgm_store_flag(c, WGM_DEVICE_TO_EXECUTE);
  c->executing_persistent = 1;
  if (!wgm_host_wait(&rt->hf->scheduler_flag, WGM_DEVICE_WAITING, true, budget)) {
    c->monitor_status = WGM_ERR_TIMEOUT;
    c->executing_persistent = 0;
    c->waiting_for_async = 0;
    return;
  }
  c->waiting_for_async = 0;
  uint64_t t0 = wgm_now_ns();
  for (;;) {
    int g = __atomic_load_n(&rt->hf->persistent_flag, __ATOMIC_ACQUIRE);
    c->time_groups_data.emplace_back(wgm_now_ns(), g);
    if (g == 0) break;
    if (wgm_now_ns() - t0 > budget || __atomic_load_n(&rt->hf->status, __ATOMIC_ACQUIRE)) {
      c->monitor_status = WGM_ERR_TIMEOUT;
      break;
    }
    std::this_thread::sleep_for(std::chrono::milliseconds(1));
  }
  c->persistent_end = wgm_now_ns();
  c->executing_persistent = 0;
}

/* send_persistent_task (cl_communicator.h:207-224) */
extern "C" int wgm_comm_send_persistent_task(wgm_comm *c, int groups) {
  if (!c || !c->launched || !c->papp) return c ? WGM_ERR_STATE : WGM_ERR_INVALID;
  if (groups < 1 || groups > c->participating_groups) return WGM_ERR_TOO_MANY_GROUPS;
  wgm_comm_join(c);
  c->monitor_status = 0;
  c->waiting_for_async = 1;
  c->monitor = std::thread(wgm_monitor, c, groups);
  auto t0 = wgm_clock::now();
  while (c->waiting_for_async.load() != 0) {
    if (wgm_clock::now() - t0 > std::chrono::nanoseconds(wgm_idle_budget(c))) break;
    std::this_thread::yield();
  }
  return c->monitor_status.load();
}

/* send_task_synchronous (cl_communicator.h:123-166): returns the execution
 * and response times in nanoseconds. */
extern "C" int wgm_comm_send_task_synchronous(wgm_comm *c, int groups, uint64_t *exec_ns,
                                              uint64_t *resp_ns) {
  if (!c || !c->launched || c->np_kind == 0) return c ? WGM_ERR_STATE : WGM_ERR_INVALID;
  /* The persistent master group never leaves, so a running persistent task
   * leaves one group fewer to take. */
  int avail = c->participating_groups - (c->executing_persistent.load() ? 1 : 0);
  if (groups < 1 || groups > avail) return WGM_ERR_TOO_MANY_GROUPS;
  wgm_runtime *rt = c->rt;
  uint64_t budget = wgm_idle_budget(c);
  c->non_persistent_wgs = groups;
  __atomic_store_n(&rt->hf->task_size, groups, __ATOMIC_RELEASE);
  wgm_store_flag(c, WGM_DEVICE_TO_TASK);
  uint64_t rb = wgm_now_ns();
  if (!wgm_host_wait(&rt->hf->scheduler_flag, WGM_DEVICE_GOT_GROUPS, true, budget))
    return WGM_ERR_TIMEOUT;
  uint64_t re = wgm_now_ns();
  wgm_store_flag(c, WGM_DEVICE_TO_EXECUTE);
  uint64_t eb = wgm_now_ns();
  if (!wgm_host_wait(&rt->hf->scheduler_flag, WGM_DEVICE_WAITING, true, budget))
    return WGM_ERR_TIMEOUT;
  uint64_t ee = wgm_now_ns();
  c->execution_times.push_back(ee - eb);
  c->response_times.push_back(re - rb);
  c->response_exec_data.emplace_back(rb, re, ee);
  if (exec_ns) *exec_ns = ee - eb;
  if (resp_ns) *resp_ns = re - rb;
  return WGM_OK;
}

extern "C" int wgm_comm_is_executing_persistent(wgm_comm *c, int *executing) {
  if (!c || !executing) return WGM_ERR_INVALID;
  *executing = c->executing_persistent.load();
  return WGM_OK;
}

/* get_persistent_time (cl_communicator.h:230-233), bounded. */
extern "C" int wgm_comm_get_persistent_time(wgm_comm *c, uint64_t *ns) {
  if (!c || !ns) return WGM_ERR_INVALID;
  auto t0 = wgm_clock::now();
  while (c->executing_persistent.load() != 0) {
    if (wgm_clock::now() - t0 > std::chrono::nanoseconds(wgm_idle_budget(c)))
      return WGM_ERR_TIMEOUT;
    std::this_thread::sleep_for(std::chrono::microseconds(100));
  }
  *ns = c->persistent_end - c->persistent_begin;
  return WGM_OK;
}

extern "C" int wgm_comm_add_redline(wgm_comm *c) {
  if (!c) return WGM_ERR_INVALID;
  c->redlines++;
  return WGM_OK;
}

/* reset_communicator (cl_communicator.h:376-393) */
extern "C" int wgm_comm_reset(wgm_comm *c) {
  if (!c || c->launched) return c ? WGM_ERR_STATE : WGM_ERR_INVALID;
  wgm_comm_join(c);
  c->participating_groups = 0;
  c->executing_persistent = 0;
  c->waiting_for_async = 0;
  c->persistent_begin = c->persistent_end = c->global_start = 0;
  c->time_groups_data.clear();
  c->response_exec_data.clear();
  c->response_times.clear();
  c->execution_times.clear();
  c->redlines = 0;
  c->non_persistent_wgs = 0;
  c->monitor_status = 0;
  return WGM_OK;
}

/* reset_non_persistent (matmult.h:251-255, reduce.h:364-366) */
extern "C" int wgm_comm_reset_non_persistent(wgm_comm *c) {
  if (!c) return WGM_ERR_INVALID;
  __atomic_store_n(&c->np_host->hash, 0, __ATOMIC_RELEASE);
  if (c->np_kind == WGM_NP_REDUCE_F32) {
    float big = 3.0e38f;
    int b;
    std::memcpy(&b, &big, 4);
    __atomic_store_n(&c->np_host->result, b, __ATOMIC_RELEASE);
  } else {
    __atomic_store_n(&c->np_host->result, INT_MAX, __ATOMIC_RELEASE);
  }
  return WGM_OK;
}

/* check_non_persistent_task (matmult.h:259-261, reduce.h:368-370); the FP32
 * matmul is checked element-wise against a host product (relative 1e-5). */
extern "C" int wgm_comm_check_non_persistent(wgm_comm *c, int *ok) {
  if (!c || !ok) return WGM_ERR_INVALID;
  *ok = 0;
  switch (c->np_kind) {
    case WGM_NP_MATMULT_I32:
      *ok = __atomic_load_n(&c->np_host->hash, __ATOMIC_ACQUIRE) == c->ref_hash;
      break;
    case WGM_NP_REDUCE_I32:
    case WGM_NP_REDUCE_F32:
      *ok = __atomic_load_n(&c->np_host->result, __ATOMIC_ACQUIRE) == c->ref_min;
      break;
    case WGM_NP_MATMULT_F32: {
      const int n = c->np_size;
      std::vector<float> C((size_t)n * n);
      cudaError_t e = cudaMemcpyAsync(C.data(), c->dCf, C.size() * 4, cudaMemcpyDeviceToHost,
                                      c->side);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->side);
      if (e != cudaSuccess) return wgm_comm_fail(c, e);
      bool good = true;
      for (int r = 0; r < n && good; r++)
        for (int cc = 0; cc < n; cc++) {
          double acc = 0;
          for (int j = 0; j < n; j++)
            acc += (double)c->Af[(size_t)r * n + j] * (double)c->Bf[(size_t)j * n + cc];
          if (std::fabs(C[(size_t)r * n + cc] - acc) > 1e-5 * std::max(1.0, std::fabs(acc))) {
            good = false;
            break;
          }
        }
      *ok = good;
      break;
    }
    default:
      return WGM_ERR_STATE;
  }
  return WGM_OK;
}

static double wgm_ms(uint64_t ns) { return ns / 1000000.0; }

/* summary_str (cl_communicator.h:296-336), same lines and units. */
extern "C" int wgm_comm_summary(wgm_comm *c, char *buf, size_t len) {
  if (!c || !buf || len == 0) return WGM_ERR_INVALID;
  auto stats = [](const std::vector<uint64_t> &v, double *mean, double *tot, double *mx,
                  double *mn, double *sd) {
    *mean = *tot = *mx = *mn = *sd = 0;
    if (v.empty()) return;
    double t = 0, a = 1e300, b = 0;
    for (uint64_t x : v) {
      t += wgm_ms(x);
      a = std::min(a, wgm_ms(x));
      b = std::max(b, wgm_ms(x));
    }
    *tot = t;
    *mean = t / v.size();
    *mn = a;
    *mx = b;
    double s = 0;
    for (uint64_t x : v) s += (wgm_ms(x) - *mean) * (wgm_ms(x) - *mean);
    *sd = std::sqrt(s / v.size());
  };
  std::string out;
  char line[256];
  double pt = wgm_ms(c->persistent_end >= c->persistent_begin
                         ? c->persistent_end - c->persistent_begin
                         : 0);
  snprintf(line, sizeof line, "Persistent task execution time: %g ms\n", pt);
  out += line;
  snprintf(line, sizeof line, "Number of discovered groups: %d\n", c->participating_groups);
  out += line;
  snprintf(line, sizeof line, "Number of non persistent tasks: %zu\n", c->response_times.size());
  out += line;
  snprintf(line, sizeof line, "Number workgroups executing non persistent task: %d\n",
           c->non_persistent_wgs);
  out += line;
  if (!c->response_times.empty()) {
    double m, t, mx, mn, sd;
    const char *names[3] = {"response", "execution", "back-to-back"};
    std::vector<uint64_t> b2b;
    for (size_t i = 0; i < c->execution_times.size(); i++)
      b2b.push_back(c->execution_times[i] + c->response_times[i]);
    const std::vector<uint64_t> *vs[3] = {&c->response_times, &c->execution_times, &b2b};
    for (int k = 0; k < 3; k++) {
      stats(*vs[k], &m, &t, &mx, &mn, &sd);
      snprintf(line, sizeof line,
               "\nNon persistent %s times:\n-----------------------\n"
               "Mean %s time: %g ms\nTotal %s time: %g ms\nMax %s time: %g ms\n"
               "Min %s time: %g ms\nStandard deviation %s time: %g ms\n",
               names[k], names[k], m, names[k], t, names[k], mx, names[k], mn, names[k], sd);
      out += line;
    }
    double avg = 0;
    for (auto &p : c->time_groups_data) avg += p.second;
    if (!c->time_groups_data.empty()) avg /= c->time_groups_data.size();
    snprintf(line, sizeof line,
             "-----------------------\nAverage observed workgroups executing persistent task: "
             "%g\nNumber of redlines: %d\n",
             avg, c->redlines);
    out += line;
  }
  size_t n = std::min(len - 1, out.size());
  std::memcpy(buf, out.data(), n);
  buf[n] = 0;
  return WGM_OK;
}

/* Raw timing vectors for callers computing percentiles. */
extern "C" int wgm_comm_task_times(wgm_comm *c, uint64_t *resp_ns, uint64_t *exec_ns,
                                   int capacity, int *count) {
  if (!c || !count) return WGM_ERR_INVALID;
  int n = (int)c->response_times.size();
  *count = n;
  for (int i = 0; i < n && i < capacity; i++) {
    if (resp_ns) resp_ns[i] = c->response_times[i];
    if (exec_ns) exec_ns[i] = c->execution_times[i];
  }
  return WGM_OK;
}

extern "C" int wgm_comm_average_persistent_groups(wgm_comm *c, double *avg) {
  if (!c || !avg) return WGM_ERR_INVALID;
  double a = 0;
  for (auto &p : c->time_groups_data) a += p.second;
  *avg = c->time_groups_data.empty() ? 0 : a / c->time_groups_data.size();
  return WGM_OK;
}

/* get_occupancy_bound (cl_communicator.h:350-374): launch the megakernel
 * on every co-resident group, read the discovered count, quit. */
extern "C" int wgm_comm_get_occupancy_bound(wgm_comm *c, int *groups) {
  if (!c || !groups || c->launched) return c ? WGM_ERR_STATE : WGM_ERR_INVALID;
  int s = wgm_comm_launch_mega_kernel(c, 0);
  if (s) return s;
  *groups = c->participating_groups;
  wgm_comm_send_quit(c);
  s = wgm_comm_finish(c);
  wgm_comm_reset(c);
  return s;
}

/* execute_merged_iteration (skel.cpp:405-463): launch, give the persistent
 * task every participating group, and every `frequency_ms` (at once after an
 * overrun: a "redline") run the non-persistent task synchronously on
 * np_groups groups until the persistent task ends; then quit.  np_errors
 * counts non-persistent results that failed their check. */
extern "C" int wgm_run_merged_iteration(wgm_comm *c, int num_wgs, int np_groups,
                                        int frequency_ms, int skip_tasks, int *np_errors,
                                        int *np_tasks) {
  if (!c) return WGM_ERR_INVALID;
  int s = wgm_comm_launch_mega_kernel(c, num_wgs);
  if (s) return s;
  int errors = 0, tasks = 0;
  s = wgm_comm_send_persistent_task(c, c->participating_groups);
  if (s == WGM_OK && !skip_tasks && c->np_kind != 0) {
    uint64_t begin = wgm_now_ns();
    for (;;) {
      if (!c->executing_persistent.load()) break;
      uint64_t end = wgm_now_ns();
      if (wgm_ms(end - begin) >= frequency_ms) {
        c->redlines++;
      } else {
        while (wgm_ms((end = wgm_now_ns()) - begin) < frequency_ms) {
          if (!c->executing_persistent.load()) break;
          std::this_thread::yield();
        }
        if (!c->executing_persistent.load()) break;
      }
      wgm_comm_reset_non_persistent(c);
      s = wgm_comm_send_task_synchronous(c, np_groups, nullptr, nullptr);
      if (s) break;
      tasks++;
      int ok = 0;
      wgm_comm_check_non_persistent(c, &ok);
      if (!ok) errors++;
      begin = end;
    }
  }
  if (s == WGM_OK) {
    uint64_t ns = 0;
    s = wgm_comm_get_persistent_time(c, &ns);
  }
  wgm_comm_send_quit(c);
  int f = wgm_comm_finish(c);
  if (!s) s = f;
  if (np_errors) *np_errors = errors;
  if (np_tasks) *np_tasks = tasks;
  return s;
}
