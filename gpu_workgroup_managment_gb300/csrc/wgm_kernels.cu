/*
 * Standalone persistent kernels (one per app) and the barrier
 * microbenchmark, compiled for sm_103a.
 */
#include "wgm_kernels.cuh"

#define WGM_PERSISTENT_PROLOGUE                                  \
  __shared__ wgm_cta c;                                          \
  __shared__ wgm_warp_smem sm;                                   \
  if (!wgm_discover(L, &c)) return;                              \
  if (L.handshake && !wgm_standalone_handshake(L, &c)) {         \
    wgm_standalone_exit(L);                                      \
    return;                                                      \
  }

/* The same for task loops that need no per-warp edge tables. */
#define WGM_PERSISTENT_PROLOGUE_TASKS                            \
  __shared__ wgm_cta c;                                          \
  if (!wgm_discover(L, &c)) return;                              \
  if (L.handshake && !wgm_standalone_handshake(L, &c)) {         \
    wgm_standalone_exit(L);                                      \
    return;                                                      \
  }

#define WGM_PERSISTENT_EPILOGUE \
  if (L.handshake) wgm_standalone_exit(L);

/* Run a phase function from its init phase with plain barriers between. */
#define WGM_DRIVE(PHASE_CALL)                                                        \
  wgm_drive(L, &c, wgm_step{0, 0}, wgm_plain_sync(),                                \
            [&](wgm_step cur, wgm_step *nxt) { return PHASE_CALL; })

template <bool SSSP>
__device__ __forceinline__ int wgm_lonestar_step(const wgm_launch &L, wgm_cta *c,
                                                 const wgm_lonestar_args &a, wgm_warp_smem *sm,
                                                 wgm_step cur, wgm_step *nxt) {
  return wgm_phase_lonestar<SSSP>(L, c, a, sm, cur.target, cur.round, &nxt->target,
                                  &nxt->round);
}

__global__ void __launch_bounds__(1024) wgm_k_bfs(wgm_launch L, wgm_lonestar_args a) {
  WGM_PERSISTENT_PROLOGUE
  WGM_DRIVE(wgm_lonestar_step<false>(L, &c, a, &sm, cur, nxt));
  WGM_PERSISTENT_EPILOGUE
}

__global__ void __launch_bounds__(1024) wgm_k_sssp(wgm_launch L, wgm_lonestar_args a) {
  WGM_PERSISTENT_PROLOGUE
  WGM_DRIVE(wgm_lonestar_step<true>(L, &c, a, &sm, cur, nxt));
  WGM_PERSISTENT_EPILOGUE
}

__global__ void __launch_bounds__(1024) wgm_k_color(wgm_launch L, wgm_color_args a) {
  WGM_PERSISTENT_PROLOGUE
  WGM_DRIVE(wgm_phase_color(L, &c, a, &sm, cur, nxt));
  WGM_PERSISTENT_EPILOGUE
}

__global__ void __launch_bounds__(1024) wgm_k_mis(wgm_launch L, wgm_mis_args a) {
  WGM_PERSISTENT_PROLOGUE
  WGM_DRIVE(wgm_phase_mis(L, &c, a, &sm, cur, nxt));
  WGM_PERSISTENT_EPILOGUE
}

/* Pannotia colour without rounds (wgm_color_async_run): the counts of
 * wgm_phase_color between plain barriers, then the release loop, then one
 * barrier before the round count (the largest colour) is written.  Dynamic
 * shared memory: one release stack per warp. */
__global__ void __launch_bounds__(1024) wgm_k_color_async(wgm_launch L, wgm_color_args a,
                                                          wgm_color_async_args q) {
  WGM_PERSISTENT_PROLOGUE
  extern __shared__ wgm_ca_stack wgm_ca_stacks[];
  wgm_ca_stack *st = &wgm_ca_stacks[threadIdx.x >> 5];
  bool ok = true;
  wgm_color_async_init(&c, a, q);
  if (wgm_barrier(L, &c)) {
    wgm_step nx;
    wgm_phase_color(L, &c, a, &sm, wgm_step{3, 0}, &nx); /* larger out-neighbours */
    if (wgm_barrier(L, &c)) {
      ok = wgm_color_async_seed(&c, a, q, st);
      if (wgm_barrier(L, &c)) {
        ok &= wgm_color_async_run(L, a, q, st);
        if (!ok && threadIdx.x % 32 == 0) wgm_fail(L, WGM_DEV_OVERFLOW, WGM_SITE_QUEUE, 0);
        if (wgm_barrier(L, &c) && c.id == 0 && threadIdx.x == 0 && a.rounds_out)
          *a.rounds_out = __ldcg(&q.ctl[4 * WGM_LINE]);
      }
    }
  }
  WGM_PERSISTENT_EPILOGUE
}

size_t wgm_color_async_smem(int block) { return (size_t)(block / 32) * sizeof(wgm_ca_stack); }

cudaError_t wgm_color_async_per_sm(int block, int *per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, wgm_k_color_async, block,
                                                       wgm_color_async_smem(block));
}

cudaError_t wgm_launch_color_async(const wgm_launch &L, const wgm_color_args &a,
                                   const wgm_color_async_args &q, int grid, int block,
                                   cudaStream_t s) {
  wgm_k_color_async<<<grid, block, wgm_color_async_smem(block), s>>>(L, a, q);
  return cudaGetLastError();
}

/* Lonestar BFS on one CTA (wgm_bfs_cta): a plain one-CTA launch, no
 * discovery and no grid barrier.  Dynamic shared memory: the visited bits,
 * then the two frontier buffers of F vertices each. */
__global__ void __launch_bounds__(1024) wgm_k_bfs_cta(wgm_lonestar_args a, int *spill,
                                                      int spill_cap, int F, int *status) {
  extern __shared__ unsigned wgm_bfs_cta_dyn[];
  __shared__ int s_cnt[8];
  wgm_bfs_cta_smem S;
  S.bits = wgm_bfs_cta_dyn;
  S.front = reinterpret_cast<int *>(wgm_bfs_cta_dyn + ((a.V + 31) >> 5));
  S.F = F;
  wgm_bfs_cta(a, spill, spill_cap, S, s_cnt);
  if (threadIdx.x == 0 && s_cnt[3] && status) *status = WGM_DEV_OVERFLOW;
}

size_t wgm_bfs_cta_smem_bytes(int V, int F) {
  return (size_t)((V + 31) / 32) * 4 + (size_t)2 * F * 4;
}

cudaError_t wgm_launch_bfs_cta(const wgm_lonestar_args &a, int *spill, int spill_cap, int F,
                               int *status, int block, cudaStream_t s) {
  const size_t smem = wgm_bfs_cta_smem_bytes(a.V, F);
  cudaError_t e = cudaFuncSetAttribute(wgm_k_bfs_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  wgm_k_bfs_cta<<<1, block, smem, s>>>(a, spill, spill_cap, F, status);
  return cudaGetLastError();
}

/* 40 registers (no spills): six 256-thread CTAs per SM instead of four */
__global__ void __maxnreg__(40) wgm_k_psssp(wgm_launch L, wgm_psssp_args a) {
  WGM_PERSISTENT_PROLOGUE
  WGM_DRIVE(wgm_phase_pannotia_sssp(L, &c, a, &sm, cur, nxt));
  WGM_PERSISTENT_EPILOGUE
}

/* 48 registers (no spills): five 256-thread CTAs per SM instead of four,
 * more gathers in flight for a kernel bound by their latency */
__global__ void __maxnreg__(48) wgm_k_pagerank(wgm_launch L, wgm_pr_args a) {
  WGM_PERSISTENT_PROLOGUE
  WGM_DRIVE(wgm_phase_pagerank(L, &c, a, &sm, cur, nxt));
  WGM_PERSISTENT_EPILOGUE
}

/* os_freq (test_suite/os_freq/device/os_freq.cl:8-46): discovery, then
 * num_iterations x 10 barriers over every discovered CTA. */
__global__ void __launch_bounds__(1024) wgm_k_barrier_bench(wgm_launch L,
                                                            wgm_barrier_bench_args a) {
  __shared__ wgm_cta c;
  if (!wgm_discover(L, &c)) return;
  unsigned long long t0 = 0;
  for (int i = 0; i < a.iterations; i++) {
    for (int j = 0; j < 10; j++) {
      if (!wgm_barrier(L, &c)) return;
      if (i == 0 && j == 0) t0 = wgm_globaltimer();
    }
  }
  if (c.id == 0 && threadIdx.x == 0) {
    *a.t_first = t0;
    *a.t_last = wgm_globaltimer();
    *a.groups_out = c.ngroups;
  }
}

/* Standalone octree build (octree.cl:150-320 without a scheduler): init,
 * one barrier, then the task loop; nothing is offered to kill or fork. */
__global__ void __launch_bounds__(1024) wgm_k_octree(wgm_launch L, wgm_octree_args a) {
  WGM_PERSISTENT_PROLOGUE_TASKS
  wgm_octree_init(L, &c, a);
  if (wgm_barrier(L, &c)) wgm_octree_loop(L, &c, a, [](wgm_cta *) { return false; });
  WGM_PERSISTENT_EPILOGUE
}

__global__ void __launch_bounds__(1024) wgm_k_bc(wgm_launch L, wgm_bc_args a) {
  WGM_PERSISTENT_PROLOGUE
  WGM_DRIVE(wgm_phase_bc(L, &c, a, &sm, cur, nxt));
  WGM_PERSISTENT_EPILOGUE
}

/* Betweenness centrality, sources spread over CTAs (wgm_bc_cta_source):
 * a plain grid of resident CTAs pulling sources from a queue, no discovery
 * and no grid barrier. */
__global__ void __launch_bounds__(1024) wgm_k_bc_cta(wgm_bc_args a, int *queue) {
  extern __shared__ int wgm_bc_dyn[];
  __shared__ int tab[32 * 32];
  __shared__ int s_cnt, s_src;
  int *dist = wgm_bc_dyn;
  float *rho = reinterpret_cast<float *>(dist + a.V);
  float *sig = rho + a.V;
  int *order = reinterpret_cast<int *>(sig + a.V);
  int *ls = order + a.V;
  for (;;) {
    if (threadIdx.x == 0) s_src = atomicAdd(queue, 1);
    __syncthreads();
    const int src = s_src;
    __syncthreads();
    if (src >= a.num_sources) break;
    wgm_bc_cta_source(a, src, dist, rho, sig, order, ls, &s_cnt, tab);
    if (threadIdx.x == 0 && a.rounds_out) atomicAdd(a.rounds_out, 1);
  }
}

/* Standalone connect-four look-ahead (connect_four.cl:350-487 without a
 * scheduler). */
__global__ void __launch_bounds__(1024) wgm_k_c4(wgm_launch L, wgm_c4_args a) {
  WGM_PERSISTENT_PROLOGUE_TASKS
  wgm_c4_init(L, &c, a);
  if (wgm_barrier(L, &c)) wgm_c4_loop(L, &c, a, [](wgm_cta *) { return false; });
  WGM_PERSISTENT_EPILOGUE
}

const void *wgm_kernel_fn(int kid) {
  switch (kid) {
    case WGM_K_BFS: return (const void *)wgm_k_bfs;
    case WGM_K_SSSP: return (const void *)wgm_k_sssp;
    case WGM_K_COLOR: return (const void *)wgm_k_color;
    case WGM_K_MIS: return (const void *)wgm_k_mis;
    case WGM_K_PSSSP: return (const void *)wgm_k_psssp;
    case WGM_K_PAGERANK: return (const void *)wgm_k_pagerank;
    case WGM_K_BARRIER_BENCH: return (const void *)wgm_k_barrier_bench;
    case WGM_K_OCTREE: return (const void *)wgm_k_octree;
    case WGM_K_C4: return (const void *)wgm_k_c4;
    case WGM_K_BC: return (const void *)wgm_k_bc;
    default: return nullptr;
  }
}

cudaError_t wgm_launch_lonestar(bool sssp, const wgm_launch &L, const wgm_lonestar_args &a,
                                int grid, int block, cudaStream_t s) {
  if (sssp)
    wgm_k_sssp<<<grid, block, 0, s>>>(L, a);
  else
    wgm_k_bfs<<<grid, block, 0, s>>>(L, a);
  return cudaGetLastError();
}
cudaError_t wgm_launch_color(const wgm_launch &L, const wgm_color_args &a, int grid, int block,
                             cudaStream_t s) {
  wgm_k_color<<<grid, block, 0, s>>>(L, a);
  return cudaGetLastError();
}
cudaError_t wgm_launch_mis(const wgm_launch &L, const wgm_mis_args &a, int grid, int block,
                           cudaStream_t s) {
  wgm_k_mis<<<grid, block, 0, s>>>(L, a);
  return cudaGetLastError();
}
cudaError_t wgm_launch_psssp(const wgm_launch &L, const wgm_psssp_args &a, int grid, int block,
                             cudaStream_t s) {
  wgm_k_psssp<<<grid, block, 0, s>>>(L, a);
  return cudaGetLastError();
}
cudaError_t wgm_launch_pagerank(const wgm_launch &L, const wgm_pr_args &a, int grid, int block,
                                cudaStream_t s) {
  wgm_k_pagerank<<<grid, block, 0, s>>>(L, a);
  return cudaGetLastError();
}
cudaError_t wgm_launch_octree(const wgm_launch &L, const wgm_octree_args &a, int grid, int block,
                              cudaStream_t s) {
  wgm_k_octree<<<grid, block, 0, s>>>(L, a);
  return cudaGetLastError();
}
cudaError_t wgm_launch_bc(const wgm_launch &L, const wgm_bc_args &a, int grid, int block,
                          cudaStream_t s) {
  wgm_k_bc<<<grid, block, 0, s>>>(L, a);
  return cudaGetLastError();
}
cudaError_t wgm_launch_bc_cta(const wgm_bc_args &a, int *queue, int block, cudaStream_t s) {
  const size_t smem = (size_t)a.V * 20 + 16;
  cudaError_t e = cudaFuncSetAttribute(wgm_k_bc_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  int per_sm = 0, dev = 0, sms = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wgm_k_bc_cta, block, smem);
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  e = cudaMemsetAsync(a.bc, 0, (size_t)a.V * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, 4, s);
  if (e == cudaSuccess && a.rounds_out) e = cudaMemsetAsync(a.rounds_out, 0, 4, s);
  if (e != cudaSuccess) return e;
  wgm_k_bc_cta<<<per_sm * sms, block, smem, s>>>(a, queue);
  return cudaGetLastError();
}
cudaError_t wgm_launch_c4(const wgm_launch &L, const wgm_c4_args &a, int grid, int block,
                          cudaStream_t s) {
  wgm_k_c4<<<grid, block, 0, s>>>(L, a);
  return cudaGetLastError();
}
cudaError_t wgm_launch_barrier_bench(const wgm_launch &L, const wgm_barrier_bench_args &a,
                                     int grid, int block, cudaStream_t s) {
  wgm_k_barrier_bench<<<grid, block, 0, s>>>(L, a);
  return cudaGetLastError();
}

/* The barrier microbenchmark as a cluster grid: `clusters` clusters of
 * `csize` CTAs (WGM_BARRIER_CLUSTER needs whole clusters). */
cudaError_t wgm_barrier_bench_clusters(int csize, int block, int *clusters) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)csize, 1, 1);
  cfg.blockDim = dim3((unsigned)block, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaOccupancyMaxActiveClusters(clusters, (void *)wgm_k_barrier_bench, &cfg);
}

cudaError_t wgm_launch_barrier_bench_cluster(const wgm_launch &L, const wgm_barrier_bench_args &a,
                                             int clusters, int csize, int block, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)(clusters * csize), 1, 1);
  cfg.blockDim = dim3((unsigned)block, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, wgm_k_barrier_bench, L, a);
}
