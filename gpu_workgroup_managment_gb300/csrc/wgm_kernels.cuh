/*
 * Kernel entry points of the standalone persistent form and their host-side
 * launch helpers (internal to libwgm; the public C-ABI is include/wgm.h).
 *
 * Every persistent kernel has the reference's standalone shape
 * (lonestar/graph_apps/bfs/device/standalone.cl:247-320): discovery, optional
 * host handshake, the app's barrier-synchronised loop, and a persistent_flag
 * decrement per group when the host handshake is on.
 */
#ifndef WGM_KERNELS_CUH
#define WGM_KERNELS_CUH

#include <cuda_runtime.h>

#include "wgm_graph.cuh"
#include "wgm_octree.cuh"
#include "wgm_c4.cuh"

enum wgm_kernel_id {
  WGM_K_BFS = 0,
  WGM_K_SSSP,
  WGM_K_COLOR,
  WGM_K_MIS,
  WGM_K_PSSSP,
  WGM_K_PAGERANK,
  WGM_K_BARRIER_BENCH,
  WGM_K_OCTREE,
  WGM_K_C4,
  WGM_K_BC,
  WGM_K_COUNT
};

struct wgm_barrier_bench_args {
  int iterations;              /* os_freq.cl:35: num_iterations x 10 barriers */
  int *groups_out;
  unsigned long long *t_first; /* %globaltimer after the first barrier */
  unsigned long long *t_last;  /* %globaltimer after the last barrier */
};

/* Host helpers (wgm_kernels.cu). */
const void *wgm_kernel_fn(int kid);
cudaError_t wgm_launch_lonestar(bool sssp, const wgm_launch &L, const wgm_lonestar_args &a,
                                int grid, int block, cudaStream_t s);
cudaError_t wgm_launch_color(const wgm_launch &L, const wgm_color_args &a, int grid, int block,
                             cudaStream_t s);
cudaError_t wgm_launch_mis(const wgm_launch &L, const wgm_mis_args &a, int grid, int block,
                           cudaStream_t s);
size_t wgm_bfs_cta_smem_bytes(int V, int F);
cudaError_t wgm_launch_bfs_cta(const wgm_lonestar_args &a, int *spill, int spill_cap, int F,
                               int *status, int block, cudaStream_t s);
size_t wgm_color_async_smem(int block);
cudaError_t wgm_color_async_per_sm(int block, int *per_sm);
cudaError_t wgm_launch_color_async(const wgm_launch &L, const wgm_color_args &a,
                                   const wgm_color_async_args &q, int grid, int block,
                                   cudaStream_t s);
cudaError_t wgm_launch_psssp(const wgm_launch &L, const wgm_psssp_args &a, int grid, int block,
                             cudaStream_t s);
cudaError_t wgm_launch_pagerank(const wgm_launch &L, const wgm_pr_args &a, int grid, int block,
                                cudaStream_t s);
cudaError_t wgm_launch_octree(const wgm_launch &L, const wgm_octree_args &a, int grid, int block,
                              cudaStream_t s);
cudaError_t wgm_launch_bc(const wgm_launch &L, const wgm_bc_args &a, int grid, int block,
                          cudaStream_t s);
cudaError_t wgm_launch_bc_cta(const wgm_bc_args &a, int *queue, int block, cudaStream_t s);
cudaError_t wgm_launch_c4(const wgm_launch &L, const wgm_c4_args &a, int grid, int block,
                          cudaStream_t s);
cudaError_t wgm_launch_barrier_bench(const wgm_launch &L, const wgm_barrier_bench_args &a,
                                     int grid, int block, cudaStream_t s);
cudaError_t wgm_barrier_bench_clusters(int csize, int block, int *clusters);
cudaError_t wgm_launch_barrier_bench_cluster(const wgm_launch &L, const wgm_barrier_bench_args &a,
                                             int clusters, int csize, int block, cudaStream_t s);

#endif
