/*
 * Host runtime of libwgm: the C-ABI declared in include/wgm.h.
 *
 * Plays the role of the reference's rt_host headers (cl_scheduler.h,
 * discovery.h, cl_communicator.h) and of the per-app host plugins, on CUDA:
 * device state in HBM, host-polled words in mapped pinned memory, one CUDA
 * stream per runtime, CUDA events for kernel time.
 */
#include <cuda_profiler_api.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "../../include/wgm.h"
#include "wgm_internal.h"
#include "wgm_kernels.cuh"

/* ------------------------------------------------------------------------ */
/* Runtime                                                                   */
/* ------------------------------------------------------------------------ */

extern "C" void wgm_config_default(wgm_config *cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->device = 0;
  cfg->threads_per_wg = 256;
  cfg->num_wgs = 0;
  cfg->use_query_barrier = 0;
  cfg->non_persistent_wgs = 2;
  cfg->non_persistent_frequency_ms = 100;
  cfg->skip_tasks = 0;
  cfg->host_handshake = 0;
  cfg->discovery_mode = WGM_DISCOVERY_TICKET;
  cfg->discovery_extra_rounds = 10;
  cfg->barrier_kind = WGM_BARRIER_AUTO;
  cfg->tree_fanin = 8;
  cfg->hub_threshold = 256;
  cfg->spin_timeout_ns = 2000000000ull;   /* 2 s */
  cfg->run_timeout_ns = 120000000000ull;  /* 120 s */
  cfg->discovery_window_ns = 200000ull;   /* 200 us */
}

extern "C" const char *wgm_status_string(int s) {
  switch (s) {
    case WGM_OK: return "ok";
    case WGM_ERR_INVALID: return "invalid argument";
    case WGM_ERR_TOO_MANY_GROUPS: return "more groups requested than discovered";
    case WGM_ERR_TIMEOUT: return "a wait exceeded its time budget";
    case WGM_ERR_OOM: return "out of memory";
    case WGM_ERR_CUDA: return "CUDA error";
    case WGM_ERR_OVERFLOW: return "worklist overflow";
    case WGM_ERR_NO_DEVICE: return "no CUDA device";
    case WGM_ERR_ABORTED: return "aborted by the host";
    case WGM_ERR_STATE: return "call not valid in the current state";
    default: return "unknown status";
  }
}

int wgm_cuda_fail(wgm_runtime *rt, cudaError_t e) {
  if (rt) rt->last_cuda = (int)e;
  if (e == cudaErrorMemoryAllocation) return WGM_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return WGM_ERR_NO_DEVICE;
  return WGM_ERR_CUDA;
}

static void wgm_clear_flags(wgm_host_flags *hf) {
  std::memset((void *)hf, 0, sizeof(wgm_host_flags));
  hf->scheduler_flag = WGM_DEVICE_SCHEDULER_INIT;
  hf->persistent_flag = -1;
  hf->check_value = -1;
}

extern "C" int wgm_runtime_create(const wgm_config *cfg, wgm_runtime **out) {
  if (!out) return WGM_ERR_INVALID;
  *out = nullptr;
  wgm_runtime *rt = new (std::nothrow) wgm_runtime();
  if (!rt) return WGM_ERR_OOM;
  if (cfg)
    rt->cfg = *cfg;
  else
    wgm_config_default(&rt->cfg);
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    int st = (e == cudaSuccess) ? WGM_ERR_NO_DEVICE : wgm_cuda_fail(rt, e);
    delete rt;
    return st == WGM_ERR_CUDA ? WGM_ERR_NO_DEVICE : st;
  }
  if (rt->cfg.device < 0 || rt->cfg.device >= ndev) {
    delete rt;
    return WGM_ERR_INVALID;
  }
  rt->device = rt->cfg.device;
#define RT_TRY(x)                       \
  do {                                  \
    cudaError_t _e = (x);               \
    if (_e != cudaSuccess) {            \
      int _s = wgm_cuda_fail(rt, _e);   \
      wgm_runtime_destroy(rt);          \
      return _s;                        \
    }                                   \
  } while (0)
  RT_TRY(cudaSetDevice(rt->device));
  RT_TRY(cudaGetDeviceProperties(&rt->prop, rt->device));
  RT_TRY(cudaStreamCreateWithFlags(&rt->stream, cudaStreamNonBlocking));
  RT_TRY(cudaMalloc((void **)&rt->st, sizeof(wgm_dev_state)));
  RT_TRY(cudaMemset(rt->st, 0, sizeof(wgm_dev_state)));
  RT_TRY(cudaHostAlloc((void **)&rt->hf, sizeof(wgm_host_flags), cudaHostAllocMapped));
  wgm_clear_flags(rt->hf);
  RT_TRY(cudaHostGetDevicePointer((void **)&rt->hf_dev, rt->hf, 0));
  RT_TRY(cudaMalloc((void **)&rt->d_scratch, 64));
  RT_TRY(cudaMemset(rt->d_scratch, 0, 64));
  RT_TRY(cudaEventCreate(&rt->ev0));
  RT_TRY(cudaEventCreate(&rt->ev1));
  RT_TRY(cudaEventCreate(&rt->tev0));
  RT_TRY(cudaEventCreate(&rt->tev1));
  RT_TRY(cudaDeviceSynchronize());
#undef RT_TRY
  rt->gen = 1;
  *out = rt;
  return WGM_OK;
}

extern "C" int wgm_runtime_destroy(wgm_runtime *rt) {
  if (!rt) return WGM_ERR_INVALID;
  if (rt->device >= 0) cudaSetDevice(rt->device);
  if (rt->stream) cudaStreamSynchronize(rt->stream);
  if (rt->st) cudaFree(rt->st);
  if (rt->d_scratch) cudaFree(rt->d_scratch);
  if (rt->hf) cudaFreeHost(rt->hf);
  if (rt->ev0) cudaEventDestroy(rt->ev0);
  if (rt->ev1) cudaEventDestroy(rt->ev1);
  if (rt->tev0) cudaEventDestroy(rt->tev0);
  if (rt->tev1) cudaEventDestroy(rt->tev1);
  if (rt->stream) cudaStreamDestroy(rt->stream);
  delete rt;
  return WGM_OK;
}

extern "C" int wgm_reset(wgm_runtime *rt) {
  if (!rt) return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  cudaError_t e = cudaStreamSynchronize(rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  e = cudaMemsetAsync(rt->st, 0, sizeof(wgm_dev_state), rt->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  wgm_clear_flags(rt->hf);
  rt->gen = 1;
  return WGM_OK;
}

extern "C" int wgm_last_cuda_error(const wgm_runtime *rt) { return rt ? rt->last_cuda : 0; }

extern "C" int wgm_device_status(const wgm_runtime *rt, int *status, int *site, int *detail) {
  if (!rt) return WGM_ERR_INVALID;
  int cur = __atomic_load_n(&rt->hf->status, __ATOMIC_ACQUIRE);
  if (cur) {
    if (status) *status = cur;
    if (site) *site = rt->hf->status_site;
    if (detail) *detail = rt->hf->status_detail;
  } else {
    if (status) *status = rt->last_status;
    if (site) *site = rt->last_site;
    if (detail) *detail = rt->last_detail;
  }
  return WGM_OK;
}

extern "C" int wgm_set_abort(wgm_runtime *rt, int value) {
  if (!rt) return WGM_ERR_INVALID;
  __atomic_store_n(&rt->hf->abort_flag, value, __ATOMIC_RELEASE);
  return WGM_OK;
}

extern "C" int wgm_sm_count(const wgm_runtime *rt, int *sms) {
  if (!rt || !sms) return WGM_ERR_INVALID;
  *sms = rt->prop.multiProcessorCount;
  return WGM_OK;
}

/* Launch parameters for the next launch; advances the generation. */
wgm_launch wgm_make_launch(wgm_runtime *rt, int grid, int handshake, int im_exit) {
  wgm_launch L;
  std::memset(&L, 0, sizeof(L));
  L.st = rt->st;
  L.hf = rt->hf_dev;
  L.spin_ns = rt->cfg.spin_timeout_ns ? rt->cfg.spin_timeout_ns : 2000000000ull;
  L.window_ns = rt->cfg.discovery_window_ns ? rt->cfg.discovery_window_ns : 200000ull;
  L.gen = rt->gen++;
  /* Wrap by an even amount: the discovery slot parity must keep alternating
   * and every stale `published` stays different from the new generations. */
  if (rt->gen >= (1 << 29)) rt->gen -= (1 << 28);
  L.expected = grid;
  L.disc_mode = rt->cfg.discovery_mode;
  L.extra_rounds = rt->cfg.discovery_extra_rounds;
  L.im_exit = im_exit;
  L.barrier_kind = rt->cfg.barrier_kind;
  L.handshake = handshake;
  L.tree_fanin = rt->cfg.tree_fanin > 0 ? rt->cfg.tree_fanin : 8;
  return L;
}

int wgm_hw_bound_for(wgm_runtime *rt, int kid, int block, int *groups) {
  int per_sm = 0;
  cudaError_t e =
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wgm_kernel_fn(kid), block, 0);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  long g = (long)per_sm * rt->prop.multiProcessorCount;
  if (g > WGM_MAX_GROUPS) g = WGM_MAX_GROUPS;
  *groups = (int)g;
  return WGM_OK;
}

/* Map a device status word to a C-ABI status. */
int wgm_status_from_device(int dev) {
  switch (dev) {
    case WGM_DEV_OK: return WGM_OK;
    case WGM_DEV_TIMEOUT: return WGM_ERR_TIMEOUT;
    case WGM_DEV_ABORTED: return WGM_ERR_ABORTED;
    case WGM_DEV_OVERFLOW: return WGM_ERR_OVERFLOW;
    default: return WGM_ERR_INVALID;
  }
}

/* After a launch completed: report a device failure and, if there was one,
 * reset the device state (a failed barrier leaves counters mid-flight). */
int wgm_finish_launch(wgm_runtime *rt, int *dev_status, int *dev_site) {
  int dev = __atomic_load_n(&rt->hf->status, __ATOMIC_ACQUIRE);
  if (dev_status) *dev_status = dev;
  if (dev_site) *dev_site = rt->hf->status_site;
  if (dev == WGM_DEV_OK) return WGM_OK;
  int st = wgm_status_from_device(dev);
  int site = rt->hf->status_site, detail = rt->hf->status_detail;
  rt->last_status = dev;
  rt->last_site = site;
  rt->last_detail = detail;
  wgm_reset(rt);
  return st;
}

bool wgm_host_wait(const volatile int32_t *p, int want, bool equal, uint64_t timeout_ns) {
  auto t0 = std::chrono::steady_clock::now();
  unsigned n = 0;
  for (;;) {
    int v = __atomic_load_n((const int32_t *)p, __ATOMIC_ACQUIRE);
    if ((v == want) == equal) return true;
    if ((++n & 1023u) == 0) {
      auto dt = std::chrono::steady_clock::now() - t0;
      if ((uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(dt).count() > timeout_ns)
        return false;
      std::this_thread::yield();
    }
  }
}

/* Wait for `stream` with a host deadline: past run_timeout_ns raise the
 * abort word (every device wait and every 64th barrier polls it) and give the
 * kernel a bounded grace period to unwind. */
int wgm_stream_wait(wgm_runtime *rt, cudaStream_t stream) {
  uint64_t budget = rt->cfg.run_timeout_ns ? rt->cfg.run_timeout_ns : 120000000000ull;
  auto t0 = std::chrono::steady_clock::now();
  bool aborted = false;
  for (unsigned n = 0;; n++) {
    cudaError_t e = cudaStreamQuery(stream);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) return wgm_cuda_fail(rt, e);
    uint64_t dt = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
                      std::chrono::steady_clock::now() - t0)
                      .count();
    if (!aborted && dt > budget) {
      wgm_set_abort(rt, 1);
      aborted = true;
    }
    if (aborted && dt > budget + 30000000000ull) return WGM_ERR_TIMEOUT;
    if (n > 20000) std::this_thread::sleep_for(std::chrono::microseconds(50));
    else std::this_thread::yield();
  }
  if (aborted) {
    wgm_set_abort(rt, 0);
    return WGM_ERR_ABORTED;
  }
  return WGM_OK;
}

extern "C" int wgm_synchronize(wgm_runtime *rt) {
  if (!rt) return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  int s = wgm_stream_wait(rt, rt->stream);
  int f = wgm_finish_launch(rt, nullptr, nullptr);
  return s ? s : f;
}

/* ------------------------------------------------------------------------ */
/* Discovery and the barrier microbenchmark                                  */
/* ------------------------------------------------------------------------ */

extern "C" int wgm_hw_occupancy_bound(wgm_runtime *rt, int app_kind, int threads_per_wg,
                                      int *groups) {
  if (!rt || !groups || threads_per_wg < 32 || threads_per_wg > 1024 || threads_per_wg % 32)
    return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  int kid = wgm_kind_to_kernel(app_kind);
  if (kid < 0) kid = WGM_K_BARRIER_BENCH;
  return wgm_hw_bound_for(rt, kid, threads_per_wg, groups);
}

extern "C" int wgm_get_occupancy_bound(wgm_runtime *rt, int threads_per_wg, int *groups) {
  if (!rt || !groups || threads_per_wg < 32 || threads_per_wg > 1024 || threads_per_wg % 32)
    return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  int hw = 0;
  int s = wgm_hw_bound_for(rt, WGM_K_BARRIER_BENCH, threads_per_wg, &hw);
  if (s) return s;
  /* The reference launches MAX_P_GROUPS groups and counts who made it
   * (skel.cpp:228-232); here the launch is the hardware bound. */
  wgm_launch L = wgm_make_launch(rt, hw, 0, 1);
  wgm_barrier_bench_args a;
  a.iterations = 0;
  a.groups_out = (int *)rt->d_scratch;
  a.t_first = (unsigned long long *)(rt->d_scratch + 8);
  a.t_last = (unsigned long long *)(rt->d_scratch + 16);
  cudaError_t e = wgm_launch_barrier_bench(L, a, hw, threads_per_wg, rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  int st = wgm_stream_wait(rt, rt->stream);
  int f = wgm_finish_launch(rt, nullptr, nullptr);
  if (!st) st = f;
  if (st) return st;
  *groups = __atomic_load_n(&rt->hf->discovered, __ATOMIC_ACQUIRE);
  return WGM_OK;
}

extern "C" int wgm_barrier_bench(wgm_runtime *rt, int threads_per_wg, int num_wgs,
                                 int iterations, int barrier_kind, double *ns_per_barrier,
                                 double *kernel_ms, int *groups) {
  if (!rt || threads_per_wg < 32 || threads_per_wg > 1024 || threads_per_wg % 32 ||
      iterations < 1)
    return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  int hw = 0;
  int s = wgm_hw_bound_for(rt, WGM_K_BARRIER_BENCH, threads_per_wg, &hw);
  if (s) return s;
  int grid = (num_wgs > 0) ? std::min(num_wgs, hw) : hw;
  int saved = rt->cfg.barrier_kind;
  rt->cfg.barrier_kind = barrier_kind;
  wgm_launch L = wgm_make_launch(rt, grid, 0, 0);
  rt->cfg.barrier_kind = saved;
  wgm_barrier_bench_args a;
  a.iterations = iterations;
  a.groups_out = (int *)rt->d_scratch;
  a.t_first = (unsigned long long *)(rt->d_scratch + 8);
  a.t_last = (unsigned long long *)(rt->d_scratch + 16);
  cudaError_t e = cudaEventRecord(rt->ev0, rt->stream);
  if (e == cudaSuccess) e = wgm_launch_barrier_bench(L, a, grid, threads_per_wg, rt->stream);
  if (e == cudaSuccess) e = cudaEventRecord(rt->ev1, rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  int st = wgm_stream_wait(rt, rt->stream);
  int f = wgm_finish_launch(rt, nullptr, nullptr);
  if (!st) st = f;
  if (st) return st;
  unsigned char host[64];
  e = cudaMemcpy(host, rt->d_scratch, 64, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  int ngroups = 0;
  unsigned long long t0 = 0, t1 = 0;
  std::memcpy(&ngroups, host, sizeof(int));
  std::memcpy(&t0, host + 8, 8);
  std::memcpy(&t1, host + 16, 8);
  if (groups) *groups = ngroups;
  long nb = (long)iterations * 10 - 1;
  if (ns_per_barrier) *ns_per_barrier = nb > 0 ? (double)(t1 - t0) / (double)nb : 0.0;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, rt->ev0, rt->ev1);
  if (kernel_ms) *kernel_ms = ms;
  return WGM_OK;
}

extern "C" int wgm_barrier_bench_cluster(wgm_runtime *rt, int threads_per_wg, int cluster_size,
                                         int num_clusters, int iterations, double *ns_per_barrier,
                                         double *kernel_ms, int *groups) {
  if (!rt || threads_per_wg < 32 || threads_per_wg > 1024 || threads_per_wg % 32 ||
      iterations < 1 || cluster_size < 1 || cluster_size > 8)
    return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  int fit = 0;
  cudaError_t e = wgm_barrier_bench_clusters(cluster_size, threads_per_wg, &fit);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  if (fit < 1) return WGM_ERR_TOO_MANY_GROUPS;
  const int clusters = num_clusters > 0 ? std::min(num_clusters, fit) : fit;
  if ((long)clusters * cluster_size > WGM_MAX_GROUPS) return WGM_ERR_TOO_MANY_GROUPS;
  int saved = rt->cfg.barrier_kind;
  rt->cfg.barrier_kind = WGM_BARRIER_CLUSTER;
  wgm_launch L = wgm_make_launch(rt, clusters * cluster_size, 0, 0);
  rt->cfg.barrier_kind = saved;
  wgm_barrier_bench_args a;
  a.iterations = iterations;
  a.groups_out = (int *)rt->d_scratch;
  a.t_first = (unsigned long long *)(rt->d_scratch + 8);
  a.t_last = (unsigned long long *)(rt->d_scratch + 16);
  e = cudaEventRecord(rt->ev0, rt->stream);
  if (e == cudaSuccess)
    e = wgm_launch_barrier_bench_cluster(L, a, clusters, cluster_size, threads_per_wg,
                                         rt->stream);
  if (e == cudaSuccess) e = cudaEventRecord(rt->ev1, rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  int st = wgm_stream_wait(rt, rt->stream);
  int f = wgm_finish_launch(rt, nullptr, nullptr);
  if (!st) st = f;
  if (st) return st;
  unsigned char host[64];
  e = cudaMemcpy(host, rt->d_scratch, 64, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  int ngroups = 0;
  unsigned long long t0 = 0, t1 = 0;
  std::memcpy(&ngroups, host, sizeof(int));
  std::memcpy(&t0, host + 8, 8);
  std::memcpy(&t1, host + 16, 8);
  if (groups) *groups = ngroups;
  /* every CTA must have been discovered for whole clusters */
  if (ngroups != clusters * cluster_size) return WGM_ERR_TIMEOUT;
  long nb = (long)iterations * 10 - 1;
  if (ns_per_barrier) *ns_per_barrier = nb > 0 ? (double)(t1 - t0) / (double)nb : 0.0;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, rt->ev0, rt->ev1);
  if (kernel_ms) *kernel_ms = ms;
  return WGM_OK;
}

extern "C" int wgm_timer_start(wgm_runtime *rt) {
  if (!rt) return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  cudaError_t e = cudaEventRecord(rt->tev0, rt->stream);
  return e == cudaSuccess ? WGM_OK : wgm_cuda_fail(rt, e);
}

extern "C" int wgm_timer_stop(wgm_runtime *rt, double *elapsed_ms) {
  if (!rt || !elapsed_ms) return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  cudaError_t e = cudaEventRecord(rt->tev1, rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  int s = wgm_stream_wait(rt, rt->stream);
  int f = wgm_finish_launch(rt, nullptr, nullptr);
  if (s) return s;
  if (f) return f;
  float ms = 0.f;
  e = cudaEventElapsedTime(&ms, rt->tev0, rt->tev1);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  *elapsed_ms = ms;
  return WGM_OK;
}

extern "C" int wgm_profiler_start(wgm_runtime *rt) {
  if (!rt) return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  cudaError_t e = cudaProfilerStart();
  return e == cudaSuccess ? WGM_OK : wgm_cuda_fail(rt, e);
}

extern "C" int wgm_profiler_stop(wgm_runtime *rt) {
  if (!rt) return WGM_ERR_INVALID;
  cudaSetDevice(rt->device);
  cudaError_t e = cudaProfilerStop();
  return e == cudaSuccess ? WGM_OK : wgm_cuda_fail(rt, e);
}
