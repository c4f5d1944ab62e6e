/*
 * Batched form (include/wgm.h "batched form"): the discovery-free job-queue
 * kernel of wgm_batch.cuh, its CUDA-graph capture, the per-graph baseline
 * (one standalone persistent launch per job, the plain form) and the
 * autotuner over block size, blocks per SM and worklist piece size.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "../../include/wgm.h"
#include "wgm_batch.cuh"
#include "wgm_internal.h"
#include "wgm_kernels.cuh"

/* The batched kernel under three register budgets: launch bounds of 1024,
 * 768 and 640 threads let ptxas use 64, 80 and 96 registers per thread.
 * At 64 the K-window walkers spill (hundreds of MB of local-memory traffic
 * per launch); at 96 nothing spills but fewer warps fit on an SM.  The
 * autotuner picks (wgm_batch_configure_kernel).  Each mode (plain, the
 * warp-local continuation when lq_rounds > 0, heavy-edge deferral when a
 * job has light > 0) is its own instantiation: code inlined into the plain
 * kernel that a launch never runs raised its spills and slowed every job
 * 10-20 % in measurements. */
/* Kernel modes: the plain job loops, the warp-local continuation, and the
 * near-far schedule with heavy edges deferred (each its own instantiation:
 * code a launch does not run still costs the others registers). */
#define WGM_BATCH_MODE_PLAIN 0
#define WGM_BATCH_MODE_ASYNC 1
#define WGM_BATCH_MODE_DEFER 2

template <int MAXT, int MODE>
__global__ void __launch_bounds__(MAXT) wgm_k_batch(wgm_batch_args B) {
  constexpr bool ASYNC = MODE == WGM_BATCH_MODE_ASYNC;
  constexpr bool DEFER = MODE == WGM_BATCH_MODE_DEFER;
  __shared__ wgm_warp_smem sm;
  extern __shared__ wgm_lq wgm_lqs[]; /* one local queue per warp */
  wgm_lq *q = &wgm_lqs[threadIdx.x >> 5];
  __shared__ int s_cnt[WGM_BATCH_SCNT];
  __shared__ int s_slot;
  for (;;) {
    if (threadIdx.x == 0) s_slot = atomicAdd(&B.ctl[0], 1);
    __syncthreads();
    const int slot = s_slot;
    if (slot >= B.nslots) break;
    const int2 sr = B.slots[slot];
    const wgm_batch_job j = B.jobs[sr.x];
    if (sr.y == 0 && threadIdx.x == 0) B.times[2 * sr.x] = wgm_globaltimer();
    if (j.team <= 1) {
      if (j.algo == 0) wgm_cta_lonestar<false, ASYNC>(B, j, sr.x, s_cnt, &sm, q);
      else wgm_cta_lonestar<true, ASYNC, DEFER>(B, j, sr.x, s_cnt, &sm, q);
    } else {
      if (j.algo == 0) wgm_team_lonestar<false, ASYNC>(B, j, sr.x, sr.y, &sm, q);
      else wgm_team_lonestar<true, ASYNC, DEFER>(B, j, sr.x, sr.y, &sm, q);
    }
    if (sr.y == 0 && threadIdx.x == 0) B.times[2 * sr.x + 1] = wgm_globaltimer();
    __syncthreads();
  }
}

/* Dynamic shared memory of a launch: one local queue per warp. */
static size_t wgm_batch_dyn_smem(int threads) { return (size_t)(threads / 32) * sizeof(wgm_lq); }

static const int wgm_batch_kmax[3] = {1024, 768, 640};   /* threads per CTA */
static const int wgm_batch_kregs[3] = {64, 80, 96};      /* register budget */
template <int MAXT>
static const void *wgm_batch_kfn_t(int mode) {
  switch (mode) {
    case WGM_BATCH_MODE_ASYNC: return (const void *)wgm_k_batch<MAXT, WGM_BATCH_MODE_ASYNC>;
    case WGM_BATCH_MODE_DEFER: return (const void *)wgm_k_batch<MAXT, WGM_BATCH_MODE_DEFER>;
    default: return (const void *)wgm_k_batch<MAXT, WGM_BATCH_MODE_PLAIN>;
  }
}
static const void *wgm_batch_kfn(int v, int mode = WGM_BATCH_MODE_PLAIN) {
  switch (v) {
    case 1: return wgm_batch_kfn_t<768>(mode);
    case 2: return wgm_batch_kfn_t<640>(mode);
    default: return wgm_batch_kfn_t<1024>(mode);
  }
}
static int wgm_batch_per_sm(int v, int threads) {
  /* the smallest of the modes' occupancies: a grid sized from it fits on
   * the GPU whichever runs, which the teams' waits rely on */
  int per_sm = 1 << 30;
  for (int mode = 0; mode < 3; mode++) {
    int n = 0;
    if (threads > wgm_batch_kmax[v] ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, wgm_batch_kfn(v, mode), threads,
                                                      wgm_batch_dyn_smem(threads)) != cudaSuccess)
      return 0;
    per_sm = std::min(per_sm, n);
  }
  return per_sm;
}

struct wgm_batch {
  wgm_runtime *rt = nullptr;
  int ngraphs = 0, njobs = 0;
  std::vector<int> gV;
  std::vector<long long> gE, g_row_off, g_col_off;
  std::vector<wgm_batch_job> jobs; /* queue order (largest first) */
  std::vector<int> queue_of;       /* caller's job index -> queue position */
  int *d_rows = nullptr, *d_cols = nullptr;
  unsigned *d_wts = nullptr, *d_dist = nullptr;
  int *d_scratch = nullptr, *d_stamp = nullptr, *d_levels = nullptr;
  int *d_ctl = nullptr;  /* control block: queue head + 4 lines per job */
  int *d_err = nullptr;  /* first device error of a batched launch, its site */
  int *d_cnt = nullptr;  /* level counters of the per-graph launches */
  int2 *d_slots = nullptr;
  unsigned long long *d_times = nullptr; /* per queue position: start, end ns */
  int nslots = 0;
  long long team_edges = 0; /* edges per team member; 0 = total edges / grid */
  int max_team = 0;         /* 0 = a quarter of the grid */
  wgm_batch_job *d_jobs = nullptr;
  long long rows_total = 0, cols_total = 0, dist_total = 0, scratch_total = 0,
            stamp_total = 0;
  bool has_weights = false;
  int threads = 256, ctas_per_sm = 0, piece = 0;
  int kvar = 0; /* register budget of the kernel: wgm_batch_kregs[kvar] */
  int lq_rounds = 0; /* warp-local continuation rounds per level (0: off) */
  /* SSSP near-far schedule: bucket width = nf_mult x the graph's mean edge
   * weight (0: the Bellman-Ford worklist); far lists of far_cap_cfg entries
   * (0: 2V + 64) */
  double nf_mult = 20.0;
  int far_cap_cfg = 0;
  /* SSSP jobs on dense graphs (average degree >= WGM_BATCH_DENSE_DEGREE):
   * buckets of light_mult x the mean weight with heavy edges deferred
   * (wgm_batch_job.light); 0 (the default): the schedule of the other SSSP
   * jobs.  Off by default: on the 512-graph batch at fixed shapes the RMAT
   * SSSP jobs ran 6-58 % longer with it (widths 0.05-1 x the mean weight):
   * their levels grew from ~11 to 27-135, and the relaxations the split
   * saves are mostly the failed ones the distance pre-check already makes
   * cheap.  The autotuner still tries 0.1, 0.2 and 0.4. */
  double light_mult = 0.0;
  /* BFS jobs on graphs of average degree at most this run on one CTA
   * whatever their size (0: teams by edges for every job).  Their levels
   * are short chains over small frontiers: a 512x512 grid BFS takes ~3 ms
   * on one CTA against ~4 ms on a team of four (16 CTA-ms), and BFS jobs
   * are not the batch's critical path (the SSSP jobs on the same grids
   * are). */
  double bfs_one_cta_deg = 5.0;
  std::vector<double> gmeanw; /* mean weight per graph (1 without weights) */
  int teams_grid = 0; /* grid the team sizes were computed for (0 = stale) */
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  /* pipelined submits: two arenas (graphs in, distances out) used in turn;
   * arena 0 is the batch's own, arena 1 is allocated by the first submit */
  struct arena {
    int *rows = nullptr, *cols = nullptr;
    unsigned *wts = nullptr, *dist = nullptr;
  } ar[2];
  cudaGraphExec_t pexec[2] = {nullptr, nullptr};
  cudaStream_t s_up = nullptr, s_down = nullptr;
  cudaEvent_t ev_up[2] = {}, ev_run[2] = {}, ev_down[2] = {};
  bool used[2] = {false, false};
  long long nsub = 0;
};

static void wgm_batch_free_graph(wgm_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  for (int a = 0; a < 2; a++) {
    if (b->pexec[a]) cudaGraphExecDestroy(b->pexec[a]);
    b->pexec[a] = nullptr;
  }
}

extern "C" int wgm_batch_destroy(wgm_batch *b) {
  if (!b) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStreamSynchronize(b->rt->stream);
  wgm_batch_free_graph(b);
  if (b->s_up) cudaStreamSynchronize(b->s_up);
  if (b->s_down) cudaStreamSynchronize(b->s_down);
  cudaFree(b->ar[1].rows);
  cudaFree(b->ar[1].cols);
  cudaFree(b->ar[1].wts);
  cudaFree(b->ar[1].dist);
  for (int a = 0; a < 2; a++) {
    if (b->ev_up[a]) cudaEventDestroy(b->ev_up[a]);
    if (b->ev_run[a]) cudaEventDestroy(b->ev_run[a]);
    if (b->ev_down[a]) cudaEventDestroy(b->ev_down[a]);
  }
  if (b->s_up) cudaStreamDestroy(b->s_up);
  if (b->s_down) cudaStreamDestroy(b->s_down);
  void *ptrs[] = {b->d_rows, b->d_cols, b->d_wts, b->d_dist, b->d_scratch, b->d_stamp,
                  b->d_levels, b->d_ctl, b->d_err, b->d_slots, b->d_jobs, b->d_cnt,
                  b->d_times};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  delete b;
  return WGM_OK;
}

/* Graphs whose SSSP jobs take the dense schedule: average degree at least
 * this (the batch's RMAT graphs have 8-32, its grids under 4). */
#define WGM_BATCH_DENSE_DEGREE 6

static bool wgm_batch_deferred(const wgm_batch *b, const wgm_batch_job &j) {
  return j.algo == 1 && b->nf_mult > 0 && b->light_mult > 0 &&
         b->gE[j.graph] >= (long long)WGM_BATCH_DENSE_DEGREE * b->gV[j.graph];
}

/* Piece size of a job: the configured one, else max(32, ceil(E/V)); the
 * worklist capacity V + E/piece + 64 then bounds every level. */
static void wgm_batch_layout(wgm_batch *b) {
  long long wl = 0;
  for (auto &j : b->jobs) {
    const int g = j.graph;
    long long V = b->gV[g], E = b->gE[g];
    long long p = b->piece > 0 ? b->piece : std::max(32LL, (E + V - 1) / std::max(V, 1LL));
    j.piece = (int)p;
    j.cap = (int)(V + (E + p - 1) / p + 64);
    const long long fc = 2 * V + 64;
    j.far_cap = j.algo ? (int)(b->far_cap_cfg > 0 ? std::min<long long>(b->far_cap_cfg, fc) : fc) : 0;
    j.wl_off = wl;
    wl += 3LL * 2 * j.cap + 2LL * j.far_cap;
    /* deferred heavy edges: two heavy lists and a settle stamp per vertex */
    if (wgm_batch_deferred(b, j)) wl += 6LL * j.cap + V;
  }
  b->scratch_total = wl;
}

/* Near-far bucket width of every SSSP job from its graph's mean weight. */
static void wgm_batch_set_deltas(wgm_batch *b) {
  for (auto &j : b->jobs) {
    j.light = 0;
    if (!j.algo || b->nf_mult <= 0) {
      j.delta = 0;
      continue;
    }
    const double w = b->gmeanw.empty() ? 1.0 : b->gmeanw[j.graph];
    const bool dense = wgm_batch_deferred(b, j);
    const double mult = dense ? b->light_mult : b->nf_mult;
    j.delta = (unsigned)std::min(1e9, std::max(1.0, std::round(mult * w)));
    /* heavy = at least one bucket width: a heavy edge from the bucket lands
     * at or above its end */
    if (dense) j.light = j.delta;
  }
}

extern "C" int wgm_batch_create(wgm_runtime *rt, int num_graphs, const wgm_graph_desc *graphs,
                                int num_jobs, const int32_t *job_graph, const int32_t *job_algo,
                                const int32_t *job_source, wgm_batch **out) {
  if (!rt || !out || num_graphs < 1 || !graphs || num_jobs < 1 || !job_graph || !job_algo ||
      !job_source)
    return WGM_ERR_INVALID;
  *out = nullptr;
  wgm_batch *b = new (std::nothrow) wgm_batch();
  if (!b) return WGM_ERR_OOM;
  b->rt = rt;
  b->ngraphs = num_graphs;
  b->njobs = num_jobs;
  b->threads = rt->cfg.threads_per_wg;
  /* graph arena layout and validation (as wgm_app_create does) */
  for (int g = 0; g < num_graphs; g++) {
    const wgm_graph_desc &d = graphs[g];
    if (d.num_nodes < 1 || !d.row_ptr || d.num_edges < 0 || (d.num_edges && !d.col) ||
        d.row_ptr[0] != 0) {
      delete b;
      return WGM_ERR_INVALID;
    }
    for (int i = 0; i < d.num_nodes; i++)
      if (d.row_ptr[i + 1] < d.row_ptr[i] && i + 1 < d.num_nodes) {
        delete b;
        return WGM_ERR_INVALID;
      }
    if (d.row_ptr[d.num_nodes] > d.num_edges) {
      delete b;
      return WGM_ERR_INVALID;
    }
    b->gV.push_back(d.num_nodes);
    b->gE.push_back(d.num_edges);
    b->g_row_off.push_back(b->rows_total);
    b->g_col_off.push_back(b->cols_total);
    b->rows_total += d.num_nodes + 1;
    b->cols_total += d.num_edges;
    if (d.weights) b->has_weights = true;
  }
  /* jobs, queued largest first (edges, then vertices) */
  std::vector<int> order(num_jobs);
  std::iota(order.begin(), order.end(), 0);
  for (int k = 0; k < num_jobs; k++) {
    int g = job_graph[k];
    if (g < 0 || g >= num_graphs || job_source[k] < 0 || job_source[k] >= b->gV[g] ||
        (job_algo[k] != 0 && job_algo[k] != 1) || (job_algo[k] == 1 && !graphs[g].weights &&
                                                   graphs[g].num_edges > 0)) {
      delete b;
      return WGM_ERR_INVALID;
    }
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    long long ex = b->gE[job_graph[x]], ey = b->gE[job_graph[y]];
    if (ex != ey) return ex > ey;
    return b->gV[job_graph[x]] > b->gV[job_graph[y]];
  });
  b->queue_of.assign(num_jobs, 0);
  /* distances in the caller's job order, so one copy returns them all */
  std::vector<long long> dist_at(num_jobs);
  long long dist_off = 0, stamp_off = 0;
  for (int k = 0; k < num_jobs; k++) {
    dist_at[k] = dist_off;
    dist_off += b->gV[job_graph[k]];
  }
  for (int q = 0; q < num_jobs; q++) {
    int k = order[q], g = job_graph[k];
    wgm_batch_job j;
    std::memset(&j, 0, sizeof(j));
    j.V = b->gV[g];
    j.algo = job_algo[k];
    j.source = job_source[k];
    j.row_off = b->g_row_off[g];
    j.col_off = b->g_col_off[g];
    j.graph = g;
    j.team = 1;
    j.boost = 100;
    j.dist_off = dist_at[k];
    /* every job: claims of the warp-local queues, or (SSSP) one 64-bit
     * {level tag, distance} word per vertex; offsets stay even, so the
     * words are 8-byte aligned */
    j.stamp_off = stamp_off;
    stamp_off += 2LL * j.V;
    b->jobs.push_back(j);
    b->queue_of[k] = q;
  }
  b->dist_total = dist_off;
  b->stamp_total = stamp_off;
  wgm_batch_layout(b);
  cudaSetDevice(rt->device);
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void **p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(bytes, 4));
  };
  alloc((void **)&b->d_rows, b->rows_total * 4);
  alloc((void **)&b->d_cols, b->cols_total * 4);
  alloc((void **)&b->d_wts, b->has_weights ? b->cols_total * 4 : 4);
  alloc((void **)&b->d_dist, b->dist_total * 4);
  alloc((void **)&b->d_stamp, b->stamp_total * 4);
  alloc((void **)&b->d_levels, (size_t)num_jobs * 4);
  alloc((void **)&b->d_ctl, (size_t)(1 + WGM_BATCH_CTL_LINES_PER_JOB * num_jobs) * WGM_LINE * 4);
  alloc((void **)&b->d_err, 2 * 4);
  alloc((void **)&b->d_times, (size_t)num_jobs * 16);
  if (e == cudaSuccess) e = cudaMemset(b->d_err, 0, 2 * 4);
  alloc((void **)&b->d_cnt, 3 * WGM_LINE * 4);
  alloc((void **)&b->d_jobs, sizeof(wgm_batch_job) * (size_t)num_jobs);
  alloc((void **)&b->d_scratch, b->scratch_total * 4);
  if (e != cudaSuccess) {
    int s = wgm_cuda_fail(rt, e);
    wgm_batch_destroy(b);
    return s;
  }
  int s = wgm_batch_upload(b, graphs);
  if (s) {
    wgm_batch_destroy(b);
    return s;
  }
  *out = b;
  return WGM_OK;
}

static cudaError_t wgm_batch_plain_fence(wgm_batch *b, cudaStream_t s);

extern "C" int wgm_batch_upload(wgm_batch *b, const wgm_graph_desc *graphs) {
  if (!b || !graphs) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStream_t s = b->rt->stream;
  cudaError_t e = wgm_batch_plain_fence(b, s);
  b->gmeanw.assign(b->ngraphs, 1.0);
  for (int g = 0; g < b->ngraphs; g++) {
    const wgm_graph_desc &d = graphs[g];
    if (d.num_nodes != b->gV[g] || d.num_edges != b->gE[g]) return WGM_ERR_INVALID;
    if (d.weights && d.num_edges) {
      double sum = 0;
      long long cnt = 0;
      for (long long k = 0; k < d.num_edges; k++)
        if (d.weights[k] < WGM_LONESTAR_INF) {
          sum += d.weights[k];
          cnt++;
        }
      if (cnt) b->gmeanw[g] = std::max(1.0, sum / (double)cnt);
    }
  }
  wgm_batch_set_deltas(b);
  for (int g = 0; g < b->ngraphs && e == cudaSuccess; g++) {
    const wgm_graph_desc &d = graphs[g];
    e = cudaMemcpyAsync(b->d_rows + b->g_row_off[g], d.row_ptr, (size_t)(d.num_nodes + 1) * 4,
                        cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && d.num_edges)
      e = cudaMemcpyAsync(b->d_cols + b->g_col_off[g], d.col, (size_t)d.num_edges * 4,
                          cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && d.num_edges && d.weights && b->has_weights)
      e = cudaMemcpyAsync(b->d_wts + b->g_col_off[g], d.weights, (size_t)d.num_edges * 4,
                          cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_jobs, b->jobs.data(), sizeof(wgm_batch_job) * b->jobs.size(),
                        cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  return WGM_OK;
}

/* All graphs at once from host arrays laid out like the device arena (rows of
 * graph g at row_offset(g), cols and weights at col_offset(g)): three copies
 * instead of three per graph. */
extern "C" int wgm_batch_upload_packed(wgm_batch *b, const int32_t *rows, const int32_t *cols,
                                       const uint32_t *weights) {
  if (!b || !rows || (b->cols_total && !cols)) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStream_t s = b->rt->stream;
  cudaError_t e = wgm_batch_plain_fence(b, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_rows, rows, (size_t)b->rows_total * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && b->cols_total)
    e = cudaMemcpyAsync(b->d_cols, cols, (size_t)b->cols_total * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && b->cols_total && weights && b->has_weights)
    e = cudaMemcpyAsync(b->d_wts, weights, (size_t)b->cols_total * 4, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  return WGM_OK;
}

/* Where graph g sits in the packed layout. */
extern "C" int wgm_batch_graph_offsets(wgm_batch *b, int64_t *row_off, int64_t *col_off) {
  if (!b) return WGM_ERR_INVALID;
  for (int g = 0; g < b->ngraphs; g++) {
    if (row_off) row_off[g] = b->g_row_off[g];
    if (col_off) col_off[g] = b->g_col_off[g];
  }
  return WGM_OK;
}

static wgm_batch_args wgm_batch_kargs(wgm_batch *b) {
  wgm_batch_args B;
  B.jobs = b->d_jobs;
  B.slots = b->d_slots;
  B.nslots = b->nslots;
  B.ctl = b->d_ctl;
  B.err = b->d_err;
  B.times = b->d_times;
  B.lq_rounds = b->lq_rounds;
  B.spin_ns = b->rt->cfg.spin_timeout_ns ? b->rt->cfg.spin_timeout_ns : 2000000000ull;
  B.rows = b->d_rows;
  B.cols = b->d_cols;
  B.wts = b->d_wts;
  B.dist = b->d_dist;
  B.scratch = b->d_scratch;
  B.stamp = b->d_stamp;
  B.levels = b->d_levels;
  return B;
}

static int wgm_batch_grid(wgm_batch *b, int *grid) {
  const int per_sm = wgm_batch_per_sm(b->kvar, b->threads);
  if (per_sm < 1) return WGM_ERR_INVALID;
  int k = b->ctas_per_sm > 0 ? std::min(b->ctas_per_sm, per_sm) : per_sm;
  *grid = k * b->rt->prop.multiProcessorCount;
  return WGM_OK;
}

/* Team sizes and the slot queue for a grid of `grid` CTAs: a job of E edges
 * gets ceil(E / team_edges) CTAs, at most max_team; its slots (job, rank)
 * follow each other in the queue, largest job first. */
static int wgm_batch_teams(wgm_batch *b, int grid) {
  long long etot = 0;
  for (auto &j : b->jobs) etot += b->gE[j.graph];
  long long te = b->team_edges > 0 ? b->team_edges
                                   : std::max(1LL << 15, (etot + grid - 1) / std::max(grid, 1));
  int mt = b->max_team > 0 ? std::min(b->max_team, grid) : std::max(1, grid / 4);
  std::vector<int2> slots;
  for (int q = 0; q < b->njobs; q++) {
    wgm_batch_job &j = b->jobs[q];
    const long long g0 = (b->gE[j.graph] + te - 1) / te;
    long long g = (g0 * std::max(j.boost, 100) + 99) / 100;
    j.team = (int)std::max(1LL, std::min<long long>(g, mt));
    if (j.algo == 0 && b->bfs_one_cta_deg > 0 &&
        (double)b->gE[j.graph] <= b->bfs_one_cta_deg * (double)b->gV[j.graph])
      j.team = 1;
    for (int r = 0; r < j.team; r++) slots.push_back(make_int2(q, r));
  }
  cudaError_t e = cudaSuccess;
  if ((int)slots.size() > b->nslots || !b->d_slots) {
    if (b->d_slots) cudaFree(b->d_slots);
    b->d_slots = nullptr;
    e = cudaMalloc((void **)&b->d_slots, slots.size() * sizeof(int2));
  }
  b->nslots = (int)slots.size();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_slots, slots.data(), slots.size() * sizeof(int2),
                        cudaMemcpyHostToDevice, b->rt->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_jobs, b->jobs.data(), sizeof(wgm_batch_job) * b->jobs.size(),
                        cudaMemcpyHostToDevice, b->rt->stream);
  /* pageable sources: wait until the copies are done before they change */
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  return WGM_OK;
}

/* First device error of the batched launches since the last check. */
static int wgm_batch_check(wgm_batch *b) {
  int h[2] = {0, 0};
  cudaError_t e = cudaMemcpy(h, b->d_err, sizeof(h), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  if (h[0] == 0) return WGM_OK;
  b->rt->last_status = h[0];
  b->rt->last_site = h[1];
  b->rt->last_detail = 0;
  cudaMemsetAsync(b->d_err, 0, sizeof(h), b->rt->stream);
  return wgm_status_from_device(h[0]);
}

/* Enqueue one batched launch: clear the control block, launch. */
/* Queue reset + batched kernel; arena 1 (pipelined submits) swaps in the
 * second set of graph and distance buffers. */
static cudaError_t wgm_batch_enqueue(wgm_batch *b, int grid, cudaStream_t s, int arena = 0) {
  cudaError_t e = cudaMemsetAsync(
      b->d_ctl, 0, (size_t)(1 + WGM_BATCH_CTL_LINES_PER_JOB * b->njobs) * WGM_LINE * 4, s);
  if (e != cudaSuccess) return e;
  wgm_batch_args B = wgm_batch_kargs(b);
  if (arena == 1) {
    B.rows = b->ar[1].rows;
    B.cols = b->ar[1].cols;
    B.wts = b->ar[1].wts;
    B.dist = b->ar[1].dist;
  }
  const size_t smem = wgm_batch_dyn_smem(b->threads);
  int mode = WGM_BATCH_MODE_PLAIN;
  if (b->lq_rounds > 0) {
    mode = WGM_BATCH_MODE_ASYNC;
  } else {
    for (const auto &j : b->jobs)
      if (j.light > 0) mode = WGM_BATCH_MODE_DEFER;
  }
  switch (b->kvar * 3 + mode) {
#define WGM_BATCH_LAUNCH(V, T)                                      \
  case V * 3 + WGM_BATCH_MODE_PLAIN:                                \
    wgm_k_batch<T, WGM_BATCH_MODE_PLAIN><<<grid, b->threads, smem, s>>>(B); \
    break;                                                          \
  case V * 3 + WGM_BATCH_MODE_ASYNC:                                \
    wgm_k_batch<T, WGM_BATCH_MODE_ASYNC><<<grid, b->threads, smem, s>>>(B); \
    break;                                                          \
  case V * 3 + WGM_BATCH_MODE_DEFER:                                \
    wgm_k_batch<T, WGM_BATCH_MODE_DEFER><<<grid, b->threads, smem, s>>>(B); \
    break;
    WGM_BATCH_LAUNCH(0, 1024)
    WGM_BATCH_LAUNCH(1, 768)
    WGM_BATCH_LAUNCH(2, 640)
#undef WGM_BATCH_LAUNCH
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

/* New scratch layout (piece size or far lists changed): reallocate the
 * scratch and send the jobs again. */
static int wgm_batch_relayout(wgm_batch *b) {
  wgm_batch_layout(b);
  cudaFree(b->d_scratch);
  b->d_scratch = nullptr;
  cudaError_t e = cudaMalloc((void **)&b->d_scratch, std::max<long long>(b->scratch_total, 1) * 4);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_jobs, b->jobs.data(), sizeof(wgm_batch_job) * b->jobs.size(),
                        cudaMemcpyHostToDevice, b->rt->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  return WGM_OK;
}

extern "C" int wgm_batch_configure(wgm_batch *b, int threads_per_cta, int ctas_per_sm,
                                   int piece) {
  if (!b || threads_per_cta < 32 || threads_per_cta > 1024 || threads_per_cta % 32 ||
      ctas_per_sm < 0 || piece < 0 || (piece > 0 && piece < 1))
    return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStreamSynchronize(b->rt->stream);
  bool relayout = piece != b->piece;
  /* a block larger than the variant's launch bounds needs the 64-register build */
  if (threads_per_cta > wgm_batch_kmax[b->kvar]) b->kvar = 0;
  b->threads = threads_per_cta;
  b->ctas_per_sm = ctas_per_sm;
  b->piece = piece;
  if (relayout) {
    int st = wgm_batch_relayout(b);
    if (st) return st;
  }
  b->teams_grid = 0;
  wgm_batch_free_graph(b);
  return WGM_OK;
}

extern "C" int wgm_batch_configure_sssp(wgm_batch *b, double delta_mult, int far_cap) {
  if (!b || !(delta_mult >= 0) || delta_mult > 1e6 || far_cap < 0) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStreamSynchronize(b->rt->stream);
  b->nf_mult = delta_mult;
  b->far_cap_cfg = far_cap;
  wgm_batch_set_deltas(b);
  int st = wgm_batch_relayout(b);
  if (st) return st;
  wgm_batch_free_graph(b);
  return WGM_OK;
}

extern "C" int wgm_batch_configure_bfs_one_cta(wgm_batch *b, double max_avg_degree) {
  if (!b || !(max_avg_degree >= 0) || max_avg_degree > 1e6) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStreamSynchronize(b->rt->stream);
  b->bfs_one_cta_deg = max_avg_degree;
  b->teams_grid = 0;
  wgm_batch_free_graph(b);
  return WGM_OK;
}

extern "C" int wgm_batch_configure_sssp_dense(wgm_batch *b, double light_mult) {
  if (!b || !(light_mult >= 0) || light_mult > 1e6) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStreamSynchronize(b->rt->stream);
  b->light_mult = light_mult;
  wgm_batch_set_deltas(b);
  int st = wgm_batch_relayout(b);
  if (st) return st;
  wgm_batch_free_graph(b);
  return WGM_OK;
}

extern "C" int wgm_batch_sssp_dense_info(wgm_batch *b, double *light_mult) {
  if (!b || !light_mult) return WGM_ERR_INVALID;
  *light_mult = b->light_mult;
  return WGM_OK;
}

extern "C" int wgm_batch_configure_teams(wgm_batch *b, int64_t team_edges, int max_team) {
  if (!b || team_edges < 0 || max_team < 0) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStreamSynchronize(b->rt->stream);
  b->team_edges = team_edges;
  b->max_team = max_team;
  b->teams_grid = 0;
  wgm_batch_free_graph(b);
  return WGM_OK;
}

/* Grid size and team layout for the current configuration. */
static int wgm_batch_prepare(wgm_batch *b, int *grid) {
  int st = wgm_batch_grid(b, grid);
  if (st) return st;
  if (b->teams_grid != *grid) {
    cudaStreamSynchronize(b->rt->stream);
    wgm_batch_free_graph(b);
    st = wgm_batch_teams(b, *grid);
    if (st) return st;
    b->teams_grid = *grid;
  }
  return WGM_OK;
}

/* A plain launch reuses arena 0: it waits for a pipelined upload or read-back
 * of that arena still in flight, and marks its own use for later submits. */
static cudaError_t wgm_batch_plain_fence(wgm_batch *b, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  if (b->s_up && b->used[0]) {
    e = cudaStreamWaitEvent(s, b->ev_up[0], 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, b->ev_down[0], 0);
  }
  return e;
}
static cudaError_t wgm_batch_plain_mark(wgm_batch *b, cudaStream_t s) {
  if (!b->s_up) return cudaSuccess;
  b->used[0] = true;
  cudaError_t e = cudaEventRecord(b->ev_run[0], s);
  /* a later read-back of arena 0 must also wait for this launch */
  if (e == cudaSuccess) e = cudaEventRecord(b->ev_down[0], s);
  if (e == cudaSuccess) e = cudaEventRecord(b->ev_up[0], s);
  return e;
}

extern "C" int wgm_batch_launch(wgm_batch *b, int use_cuda_graph) {
  if (!b) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStream_t s = b->rt->stream;
  int grid = 0;
  int st = wgm_batch_prepare(b, &grid);
  if (st) return st;
  cudaError_t e = wgm_batch_plain_fence(b, s);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  if (use_cuda_graph) {
    if (!b->exec) {
      /* capture once: queue reset + batched kernel */
      e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) e = wgm_batch_enqueue(b, grid, s);
      cudaError_t e2 = cudaStreamEndCapture(s, &b->graph);
      if (e == cudaSuccess) e = e2;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
      if (e != cudaSuccess) {
        wgm_batch_free_graph(b);
        return wgm_cuda_fail(b->rt, e);
      }
    }
    e = cudaGraphLaunch(b->exec, s);
  } else {
    e = wgm_batch_enqueue(b, grid, s);
  }
  if (e == cudaSuccess) e = wgm_batch_plain_mark(b, s);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  return WGM_OK;
}

/* Pipelined form of upload_packed + launch + read_all.  Step k uses arena
 * k & 1: its upload (stream s_up) waits only for the launch that last read
 * that arena, its launch (the runtime's stream) for its upload and for the
 * read-back that last emptied the arena's distances, its read-back (stream
 * s_down) for its launch.  So the upload of step k+1 and the read-back of
 * step k-1 run under the kernel of step k; every step still copies all of
 * its graphs in and all of its distances out. */
extern "C" int wgm_batch_submit_packed(wgm_batch *b, const int32_t *rows, const int32_t *cols,
                                       const uint32_t *weights, uint32_t *out) {
  if (!b || !rows || !out || (b->cols_total && !cols)) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStream_t s = b->rt->stream;
  cudaError_t e = cudaSuccess;
  if (!b->s_up) {
    e = cudaStreamCreateWithFlags(&b->s_up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->s_down, cudaStreamNonBlocking);
    for (int a = 0; a < 2 && e == cudaSuccess; a++) {
      e = cudaEventCreateWithFlags(&b->ev_up[a], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_run[a], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_down[a], cudaEventDisableTiming);
    }
    b->ar[0].rows = b->d_rows;
    b->ar[0].cols = b->d_cols;
    b->ar[0].wts = b->d_wts;
    b->ar[0].dist = b->d_dist;
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->ar[1].rows, std::max(b->rows_total, 1LL) * 4);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->ar[1].cols, std::max(b->cols_total, 1LL) * 4);
    if (e == cudaSuccess)
      e = cudaMalloc((void **)&b->ar[1].wts, b->has_weights ? std::max(b->cols_total, 1LL) * 4 : 4);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->ar[1].dist, std::max(b->dist_total, 1LL) * 4);
    /* arena 0's first submit must follow whatever the runtime's stream holds */
    if (e == cudaSuccess) e = cudaEventRecord(b->ev_run[0], s);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev_down[0], s);
    b->used[0] = true;
    if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  }
  int grid = 0;
  int st = wgm_batch_prepare(b, &grid);
  if (st) return st;
  const int a = (int)(b->nsub & 1);
  if (!b->pexec[a]) {
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) e = wgm_batch_enqueue(b, grid, s, a);
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->pexec[a], g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  }
  const wgm_batch::arena &A = b->ar[a];
  if (b->used[a]) e = cudaStreamWaitEvent(b->s_up, b->ev_run[a], 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(A.rows, rows, (size_t)b->rows_total * 4, cudaMemcpyHostToDevice, b->s_up);
  if (e == cudaSuccess && b->cols_total)
    e = cudaMemcpyAsync(A.cols, cols, (size_t)b->cols_total * 4, cudaMemcpyHostToDevice, b->s_up);
  if (e == cudaSuccess && b->cols_total && weights && b->has_weights)
    e = cudaMemcpyAsync(A.wts, weights, (size_t)b->cols_total * 4, cudaMemcpyHostToDevice,
                        b->s_up);
  if (e == cudaSuccess) e = cudaEventRecord(b->ev_up[a], b->s_up);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, b->ev_up[a], 0);
  if (e == cudaSuccess && b->used[a]) e = cudaStreamWaitEvent(s, b->ev_down[a], 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(b->pexec[a], s);
  if (e == cudaSuccess) e = cudaEventRecord(b->ev_run[a], s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(b->s_down, b->ev_run[a], 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, A.dist, (size_t)b->dist_total * 4, cudaMemcpyDeviceToHost,
                        b->s_down);
  if (e == cudaSuccess) e = cudaEventRecord(b->ev_down[a], b->s_down);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  b->used[a] = true;
  b->nsub++;
  return WGM_OK;
}

extern "C" int wgm_batch_wait(wgm_batch *b) {
  if (!b) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaError_t e = cudaStreamSynchronize(b->rt->stream);
  if (e == cudaSuccess && b->s_up) e = cudaStreamSynchronize(b->s_up);
  if (e == cudaSuccess && b->s_down) e = cudaStreamSynchronize(b->s_down);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  return wgm_batch_check(b);
}

extern "C" int wgm_batch_run(wgm_batch *b, int use_cuda_graph, double *device_ms) {
  if (!b) return WGM_ERR_INVALID;
  int s = wgm_timer_start(b->rt);
  if (!s) s = wgm_batch_launch(b, use_cuda_graph);
  double ms = 0;
  int t = wgm_timer_stop(b->rt, &ms);
  if (!s) s = t;
  if (!s) s = wgm_batch_check(b);
  if (device_ms) *device_ms = ms;
  return s;
}

/* The plain form: one standalone persistent launch (discovery, barrier per
 * level) per job, on every co-resident CTA (policy WGM_PER_GRAPH_ALL) or on
 * the group count wgm_run_persistent picks by default for a Lonestar app
 * (WGM_PER_GRAPH_DEFAULT: one group per 8192 edges, rounded up to a
 * multiple of the SM count, at least one per SM). */
extern "C" int wgm_batch_launch_per_graph_sized(wgm_batch *b, int policy) {
  if (!b || (policy != WGM_PER_GRAPH_ALL && policy != WGM_PER_GRAPH_DEFAULT))
    return WGM_ERR_INVALID;
  wgm_runtime *rt = b->rt;
  cudaSetDevice(rt->device);
  int block = rt->cfg.threads_per_wg;
  if (block < 32 || block > 1024 || block % 32) block = 256;
  int hw[2] = {0, 0};
  int s = wgm_hw_bound_for(rt, WGM_K_BFS, block, &hw[0]);
  if (!s) s = wgm_hw_bound_for(rt, WGM_K_SSSP, block, &hw[1]);
  if (s) return s;
  for (int q = 0; q < b->njobs; q++) {
    const wgm_batch_job &j = b->jobs[q];
    wgm_lonestar_args a;
    std::memset(&a, 0, sizeof(a));
    a.V = j.V;
    a.row = b->d_rows + j.row_off;
    a.col = b->d_cols + j.col_off;
    a.wt = j.algo ? b->d_wts + j.col_off : nullptr;
    a.dist = b->d_dist + j.dist_off;
    a.wl_start = b->d_scratch + j.wl_off;
    a.wl_cnt = a.wl_start + 2 * (size_t)j.cap;
    a.wl_u = j.algo ? a.wl_cnt + 2 * (size_t)j.cap : nullptr;
    a.cap = j.cap;
    a.piece = j.piece;
    a.cnt = b->d_cnt;
    a.stamp = j.algo ? b->d_stamp + j.stamp_off : nullptr;
    a.source = j.source;
    a.levels_out = b->d_levels + q;
    int grid = hw[j.algo];
    if (policy == WGM_PER_GRAPH_DEFAULT) {
      const long long sms = rt->prop.multiProcessorCount;
      const long long want = (b->gE[j.graph] / 8192 + sms - 1) / sms * sms;
      grid = (int)std::min<long long>(grid, std::max(sms, want));
    }
    wgm_launch L = wgm_make_launch(rt, grid, 0, 0);
    cudaError_t e = wgm_launch_lonestar(j.algo == 1, L, a, grid, block, rt->stream);
    if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  }
  return WGM_OK;
}

extern "C" int wgm_batch_launch_per_graph(wgm_batch *b) {
  return wgm_batch_launch_per_graph_sized(b, WGM_PER_GRAPH_ALL);
}

extern "C" int wgm_batch_run_per_graph_sized(wgm_batch *b, int policy, double *device_ms) {
  if (!b) return WGM_ERR_INVALID;
  int s = wgm_timer_start(b->rt);
  if (!s) s = wgm_batch_launch_per_graph_sized(b, policy);
  double ms = 0;
  int t = wgm_timer_stop(b->rt, &ms);
  if (!s) s = t;
  if (device_ms) *device_ms = ms;
  return s;
}

extern "C" int wgm_batch_run_per_graph(wgm_batch *b, double *device_ms) {
  return wgm_batch_run_per_graph_sized(b, WGM_PER_GRAPH_ALL, device_ms);
}

extern "C" int wgm_batch_read(wgm_batch *b, int job, uint32_t *out, int64_t n) {
  if (!b || !out || job < 0 || job >= b->njobs) return WGM_ERR_INVALID;
  const wgm_batch_job &j = b->jobs[b->queue_of[job]];
  if (n < j.V) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaError_t e = cudaMemcpyAsync(out, b->d_dist + j.dist_off, (size_t)j.V * 4,
                                  cudaMemcpyDeviceToHost, b->rt->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->rt->stream);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  return wgm_batch_check(b);
}

/* All results, in the caller's job order, concatenated. */
extern "C" int wgm_batch_read_all(wgm_batch *b, uint32_t *out, int64_t n) {
  if (!b || !out || n < b->dist_total) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStream_t s = b->rt->stream;
  /* the distance arena is laid out in the caller's job order: one copy */
  cudaError_t e = cudaMemcpyAsync(out, b->d_dist, (size_t)b->dist_total * 4,
                                  cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  return wgm_batch_check(b);
}

extern "C" int wgm_batch_info(wgm_batch *b, int64_t *total_nodes, int64_t *total_edges,
                              int *threads, int *ctas_per_sm, int *piece) {
  if (!b) return WGM_ERR_INVALID;
  if (total_nodes) *total_nodes = b->dist_total;
  if (total_edges) {
    long long e = 0;
    for (auto &j : b->jobs) e += b->gE[j.graph];
    *total_edges = e;
  }
  if (threads) *threads = b->threads;
  if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
  if (piece) *piece = b->piece;
  return WGM_OK;
}

/* Autotuner: block size x blocks per SM x worklist piece first, then the
 * team size (edges per team member as a multiple of total edges / grid) with
 * the queue ordered by a run at that size, each point the best of `reps`
 * CUDA-graph replays; leaves the batch configured with the winner. */
static int wgm_batch_time(wgm_batch *b, int reps, double *out) {
  double ms = 0, mn = 1e300;
  int s = wgm_batch_run(b, 1, &ms); /* warm-up and capture */
  if (s) return s;
  for (int r = 0; r < reps; r++) {
    s = wgm_batch_run(b, 1, &ms);
    if (s) return s;
    mn = std::min(mn, ms);
  }
  *out = mn;
  return WGM_OK;
}

extern "C" int wgm_batch_autotune(wgm_batch *b, int reps, int *best_threads,
                                  int *best_ctas_per_sm, int *best_piece, double *best_ms) {
  if (!b || reps < 1) return WGM_ERR_INVALID;
  const int threads_set[3] = {128, 256, 512};
  const int piece_set[3] = {16, 32, 64};
  const double factors[6] = {1.0 / 32, 1.0 / 16, 0.125, 0.25, 0.5, 1.0};
  const int saved_mt = b->max_team;
  long long etot = 0;
  for (auto &j : b->jobs) etot += b->gE[j.graph];
  /* one point: configure, run once, queue ordered from that run, time */
  auto point = [&](int t, int c, int p, long long te, double *ms) {
    int s = wgm_batch_configure(b, t, c, p);
    if (!s) s = wgm_batch_configure_teams(b, te, saved_mt);
    double x = 0;
    if (!s) s = wgm_batch_run(b, 1, &x);
    if (!s) s = wgm_batch_reorder_by_last_run(b);
    if (!s) s = wgm_batch_time(b, reps, ms);
    return s;
  };
  auto grid_of = [&](int t, int c) {
    int per_sm = wgm_batch_per_sm(b->kvar, t);
    if (c > 0) per_sm = std::min(per_sm, c);
    return std::max(1, per_sm * b->rt->prop.multiProcessorCount);
  };
  double best = 1e300;
  int bt = 256, bc = 0, bp = 0;
  long long bte = 0;
  /* 1. team size at the default shape */
  for (double f : factors) {
    long long te = std::max(1LL << 12, (long long)(etot / grid_of(bt, bc) * f));
    double ms = 0;
    int s = point(bt, bc, bp, te, &ms);
    if (s) return s;
    if (ms < best) {
      best = ms;
      bte = te;
    }
  }
  /* 2. shape at that team size (team_edges scaled with the grid) */
  const double per_cta = (double)bte * grid_of(256, 0);
  int bv = b->kvar;
  for (int v = 0; v < 3; v++)
    for (int t : threads_set) {
      const int per_sm = wgm_batch_per_sm(v, t);
      if (per_sm < 1) continue;
      b->kvar = v;
      std::vector<int> ctas;
      for (int c = std::max(1, per_sm / 2); c < per_sm; c *= 2) ctas.push_back(c);
      ctas.push_back(per_sm);
      for (int c : ctas) {
        for (int p : piece_set) {
          long long te = std::max(1LL << 12, (long long)(per_cta / grid_of(t, c)));
          double ms = 0;
          int s = point(t, c, p, te, &ms);
          if (s) return s;
          if (ms < best) {
            best = ms;
            bt = t;
            bc = c;
            bp = p;
            bte = te;
            bv = v;
          }
        }
      }
    }
  b->kvar = bv;
  /* 3. team size again at the winning shape */
  const long long base = bte;
  for (double f : {0.5, 0.75, 0.85, 1.2, 1.5, 2.0}) {
    long long te = std::max(1LL << 12, (long long)(base * f));
    double ms = 0;
    int s = point(bt, bc, bp, te, &ms);
    if (s) return s;
    if (ms < best) {
      best = ms;
      bte = te;
    }
  }
  /* 4. warp-local continuation rounds at the winning point */
  int blq = 0;
  for (int lq : {4, 12}) {
    int s = wgm_batch_configure_local(b, lq);
    double ms = 0;
    if (!s) s = point(bt, bc, bp, bte, &ms);
    if (s) return s;
    if (ms < best) {
      best = ms;
      blq = lq;
    }
  }
  int s = wgm_batch_configure_local(b, blq);
  if (s) return s;
  /* 4b. near-far bucket width (packed SSSP runs without local rounds) */
  if (blq == 0) {
    const double m0 = b->nf_mult;
    double bm = m0;
    for (double m : {m0 * 0.5, m0 * 2.0}) {
      if (m0 <= 0) break;
      s = wgm_batch_configure_sssp(b, m, b->far_cap_cfg);
      double ms = 0;
      if (!s) s = point(bt, bc, bp, bte, &ms);
      if (s) return s;
      if (ms < best) {
        best = ms;
        bm = m;
      }
    }
    s = wgm_batch_configure_sssp(b, bm, b->far_cap_cfg);
    if (s) return s;
    /* 4c. bucket width of the dense graphs' SSSP jobs (heavy edges
     * deferred), 0 = their schedule is the others' */
    const double l0 = b->light_mult;
    double bl = l0;
    for (double lm : {0.0, 0.1, 0.2, 0.4}) {
      if (lm == l0) continue;
      s = wgm_batch_configure_sssp_dense(b, lm);
      double ms = 0;
      if (!s) s = point(bt, bc, bp, bte, &ms);
      if (s) return s;
      if (ms < best) {
        best = ms;
        bl = lm;
      }
    }
    s = wgm_batch_configure_sssp_dense(b, bl);
    if (s) return s;
  }
  /* 5. critical path: the jobs that run longest (over 0.8 x the launch)
   * grow their team by a quarter, while that shortens the launch; a step
   * that does not is undone and the search ends.  Quarter steps: on the
   * 512-graph batch the SSSP jobs on the 512x512 grids are the critical
   * path, and their best team (5 CTAs) sits between the edge rule's 4 and
   * a doubling's 8. */
  s = point(bt, bc, bp, bte, &best);
  if (s) return s;
  for (int it = 0; it < 10; it++) {
    std::vector<unsigned long long> t(2 * (size_t)b->njobs);
    if (cudaMemcpy(t.data(), b->d_times, t.size() * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
      break;
    unsigned long long t0 = ~0ull, t1 = 0;
    for (int q = 0; q < b->njobs; q++) {
      t0 = std::min(t0, t[2 * q]);
      t1 = std::max(t1, t[2 * q + 1]);
    }
    const double span = (double)(t1 - t0);
    std::map<long long, int> saved; /* job (by its distance offset) -> boost */
    int boosted = 0;
    for (int q = 0; q < b->njobs; q++) {
      saved[b->jobs[q].dist_off] = b->jobs[q].boost;
      if ((double)(t[2 * q + 1] - t[2 * q]) > 0.8 * span && b->jobs[q].team < grid_of(bt, bc) / 4) {
        b->jobs[q].boost = b->jobs[q].boost * 5 / 4;
        boosted++;
      }
    }
    if (!boosted) break;
    b->teams_grid = 0;
    wgm_batch_free_graph(b);
    double x = 0, ms = 0;
    s = wgm_batch_run(b, 1, &x);
    if (!s) s = wgm_batch_reorder_by_last_run(b);
    if (!s) s = wgm_batch_time(b, reps, &ms);
    if (s) return s;
    if (ms < best) {
      best = ms;
      continue;
    }
    /* no gain: undo (the queue was re-ordered, so match jobs by offset) */
    for (int q = 0; q < b->njobs; q++) b->jobs[q].boost = saved[b->jobs[q].dist_off];
    b->teams_grid = 0;
    wgm_batch_free_graph(b);
    break;
  }
  double ms = 0;
  s = wgm_batch_run(b, 1, &ms);
  if (!s) s = wgm_batch_reorder_by_last_run(b);
  if (best_threads) *best_threads = bt;
  if (best_ctas_per_sm) *best_ctas_per_sm = bc;
  if (best_piece) *best_piece = bp;
  if (best_ms) *best_ms = best;
  return s;
}

/* Device timestamps of the last batched launch, in the caller's job order:
 * start and end of each job (ns, relative to the earliest start), its team
 * size and its level count. */
extern "C" int wgm_batch_job_stats(wgm_batch *b, int64_t *start_ns, int64_t *end_ns,
                                   int32_t *team, int32_t *levels) {
  if (!b) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  std::vector<unsigned long long> t(2 * (size_t)b->njobs);
  std::vector<int> lv(b->njobs);
  cudaError_t e = cudaStreamSynchronize(b->rt->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy(t.data(), b->d_times, t.size() * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess)
    e = cudaMemcpy(lv.data(), b->d_levels, lv.size() * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  unsigned long long t0 = ~0ull;
  for (int q = 0; q < b->njobs; q++) t0 = std::min(t0, t[2 * q]);
  for (int k = 0; k < b->njobs; k++) {
    const int q = b->queue_of[k];
    if (start_ns) start_ns[k] = (int64_t)(t[2 * q] - t0);
    if (end_ns) end_ns[k] = (int64_t)(t[2 * q + 1] - t0);
    if (team) team[k] = b->jobs[q].team;
    if (levels) levels[k] = lv[q];
  }
  return WGM_OK;
}

/* Edges each job of the last batched launch walked (caller's order): the
 * degree of every vertex visit summed, so a job that relaxes each reached
 * vertex once walks its component's edges and re-relaxations count again. */
extern "C" int wgm_batch_job_work(wgm_batch *b, int64_t *edges_walked) {
  if (!b || !edges_walked) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  const size_t n = (size_t)(1 + WGM_BATCH_CTL_LINES_PER_JOB * b->njobs) * WGM_LINE;
  std::vector<int> ctl(n);
  cudaError_t e = cudaStreamSynchronize(b->rt->stream);
  if (e == cudaSuccess) e = cudaMemcpy(ctl.data(), b->d_ctl, n * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  for (int k = 0; k < b->njobs; k++) {
    const int q = b->queue_of[k];
    const size_t at = (size_t)(1 + q * WGM_BATCH_CTL_LINES_PER_JOB + 3) * WGM_LINE +
                      WGM_BATCH_WORK_OFF;
    unsigned long long w;
    std::memcpy(&w, &ctl[at], 8);
    edges_walked[k] = (int64_t)w;
  }
  return WGM_OK;
}

/* Profile-guided queue order: sort the jobs by their device duration in the
 * last batched launch, longest first (longest-processing-time-first list
 * scheduling), so the jobs on the critical path - high-diameter graphs run
 * level after level - start at once instead of behind jobs with more edges
 * but fewer levels.  Outputs and offsets do not move; the next launch
 * recaptures its CUDA graph. */
extern "C" int wgm_batch_reorder_by_last_run(wgm_batch *b) {
  if (!b) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  std::vector<unsigned long long> t(2 * (size_t)b->njobs);
  cudaError_t e = cudaStreamSynchronize(b->rt->stream);
  if (e == cudaSuccess)
    e = cudaMemcpy(t.data(), b->d_times, t.size() * 8, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return wgm_cuda_fail(b->rt, e);
  std::vector<int> order(b->njobs);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return t[2 * x + 1] - t[2 * x] > t[2 * y + 1] - t[2 * y];
  });
  std::vector<wgm_batch_job> jobs(b->njobs);
  std::vector<int> new_pos(b->njobs);
  for (int q = 0; q < b->njobs; q++) {
    jobs[q] = b->jobs[order[q]];
    new_pos[order[q]] = q;
  }
  for (int k = 0; k < b->njobs; k++) b->queue_of[k] = new_pos[b->queue_of[k]];
  b->jobs.swap(jobs);
  b->teams_grid = 0;
  wgm_batch_free_graph(b);
  return WGM_OK;
}

extern "C" int wgm_batch_configure_local(wgm_batch *b, int rounds) {
  if (!b || rounds < 0 || rounds > WGM_LQ_ROUNDS_MAX) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStreamSynchronize(b->rt->stream);
  b->lq_rounds = rounds;
  wgm_batch_free_graph(b);
  return WGM_OK;
}

extern "C" int wgm_batch_configure_kernel(wgm_batch *b, int max_regs) {
  if (!b) return WGM_ERR_INVALID;
  int v = -1;
  for (int k = 0; k < 3; k++)
    if (wgm_batch_kregs[k] == max_regs) v = k;
  if (v < 0 || b->threads > wgm_batch_kmax[v]) return WGM_ERR_INVALID;
  cudaSetDevice(b->rt->device);
  cudaStreamSynchronize(b->rt->stream);
  b->kvar = v;
  b->teams_grid = 0;
  wgm_batch_free_graph(b);
  return WGM_OK;
}

extern "C" int wgm_batch_kernel_info(wgm_batch *b, int *max_regs) {
  if (!b) return WGM_ERR_INVALID;
  if (max_regs) *max_regs = wgm_batch_kregs[b->kvar];
  return WGM_OK;
}

extern "C" int wgm_batch_sssp_info(wgm_batch *b, double *delta_mult, int *far_cap) {
  if (!b) return WGM_ERR_INVALID;
  if (delta_mult) *delta_mult = b->nf_mult;
  if (far_cap) *far_cap = b->far_cap_cfg;
  return WGM_OK;
}

extern "C" int wgm_batch_team_info(wgm_batch *b, int64_t *team_edges, int *max_team) {
  if (!b) return WGM_ERR_INVALID;
  if (team_edges) *team_edges = b->team_edges;
  if (max_team) *max_team = b->max_team;
  return WGM_OK;
}
