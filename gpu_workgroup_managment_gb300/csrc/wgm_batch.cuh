/*
 * Batched form: many graphs, many (graph, algorithm, source) jobs, one
 * persistent launch.  A job runs on a team of G CTAs (G = 1 for most jobs,
 * more for the large ones, in proportion to their edges): CTAs pull team
 * slots from a device queue in job order, largest job first, and the
 * members of a team synchronise with a counting barrier of their own.  A
 * one-CTA job uses __syncthreads as the level barrier and keeps its level
 * counters in shared memory.
 *
 * The per-level work is the persistent kernel's (wgm_ls_chunk in
 * wgm_graph.cuh): pieces of at most `piece` edges, 32 pieces per warp, edges
 * walked in batches of 32*K with coalesced col[] loads and one counter atomic
 * per batch; the relaxation rules are the reference's (bfs.cl:115-125,
 * sssp.cl:115-131), so every job's output equals a standalone launch on
 * that graph.
 *
 * No grid-wide barrier: slots are taken in order and a CTA takes a slot only
 * when it is free, so the members of a team are CTAs that are running; with
 * every team no larger than the grid and the grid no larger than what fits
 * on the GPU at once, every team fills up.  Each team wait is bounded
 * (a timeout sets the batch's error word).  Nothing of a launch is baked
 * into device state, which lets a launch be captured in a CUDA graph and
 * replayed: the control block (queue head, team counters) is cleared by a
 * memset node before the kernel.
 */
#ifndef WGM_BATCH_CUH
#define WGM_BATCH_CUH

#include "wgm_graph.cuh"

/* Whether batch jobs read dist[dst] before the atomic (one more dependent
 * load, fewer atomics).  The batch's graphs are small and its critical path
 * is latency: go straight to the atomic. */
#ifndef WGM_BATCH_PRECHECK
#define WGM_BATCH_PRECHECK false
#endif

struct wgm_batch_job {
  int V;
  int algo;   /* 0 = BFS, 1 = SSSP */
  int source;
  int piece;
  long long row_off;  /* row_ptr of the graph: rows[row_off .. row_off+V] */
  long long col_off;  /* col / weights of the graph start here */
  long long dist_off; /* output dist[V] */
  long long wl_off;   /* scratch: 3 x 2 x cap ints (start, cnt, u) */
  long long stamp_off;/* SSSP scratch: stamp[V] */
  int cap;
  int graph; /* graph index (host bookkeeping) */
  int team;  /* CTAs working on the job */
  int boost; /* host: team multiplier from the critical-path pass */
};

/* Control block, cleared before every launch: line 0 = queue head, then per
 * job 4 lines (3 level counters, 1 barrier arrival counter). */
#define WGM_BATCH_CTL_LINES_PER_JOB 4

struct wgm_batch_args {
  const wgm_batch_job *jobs;
  const int2 *slots; /* (job, rank in team), in queue order */
  int nslots;
  int *ctl;
  const int *rows;
  const int *cols;
  const unsigned *wts;
  unsigned *dist;
  int *scratch;
  int *stamp;
  int *levels; /* per job */
  int *err;    /* first error (WGM_DEV_*), site in err[1] */
  unsigned long long *times; /* per job: start, end (%globaltimer ns) */
  unsigned long long spin_ns;
};

/* Queue a warp's flagged vertices as pieces, CTA-local counter in smem. */
__device__ __forceinline__ void wgm_cta_push(const int *row, int piece, bool flag, int u,
                                             int *s_counter, int *o_start, int *o_cnt, int *o_u,
                                             int *tab) {
  int start = 0, deg = 0, np = 0;
  if (flag) {
    start = __ldg(&row[u]);
    deg = max(__ldg(&row[u + 1]) - start, 0);
    np = (deg + piece - 1) / piece;
  }
  int incl = wgm_warp_incl_scan(np);
  int total = __shfl_sync(WGM_FULL, incl, 31);
  if (total == 0) return;
  int base = 0;
  if (wgm_lane() == 0) base = atomicAdd(s_counter, total);
  base = __shfl_sync(WGM_FULL, base, 0);
  int off = incl - np;
  wgm_for_each_edge(off, np, -off, total, 0, 32, tab, [&](bool valid, int k, int owner) {
    int s = __shfl_sync(WGM_FULL, start, owner);
    int d = __shfl_sync(WGM_FULL, deg, owner);
    int v = __shfl_sync(WGM_FULL, u, owner);
    int o = __shfl_sync(WGM_FULL, off, owner);
    if (valid) {
      int slot = base + o + k;
      o_start[slot] = s + k * piece;
      o_cnt[slot] = min(piece, d - k * piece);
      if (o_u) o_u[slot] = v;
    }
  });
}

/* One job on one CTA.  s_cnt: 3 shared level counters. */
template <bool SSSP>
__device__ void wgm_cta_lonestar(const wgm_batch_args &B, const wgm_batch_job &j, int job,
                                 int *s_cnt, wgm_warp_smem *sm) {
  const int V = j.V;
  const int *row = B.rows + j.row_off;
  const int *col = B.cols + j.col_off;
  const unsigned *wt = SSSP ? B.wts + j.col_off : nullptr;
  unsigned *dist = B.dist + j.dist_off;
  int *stamp = SSSP ? B.stamp + j.stamp_off : nullptr;
  const int cap = j.cap;
  int *wl_start = B.scratch + j.wl_off;
  int *wl_cnt = wl_start + 2 * (size_t)cap;
  int *wl_u = SSSP ? wl_cnt + 2 * (size_t)cap : nullptr;
  const int lane = wgm_lane(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = threadIdx.x; i < V; i += blockDim.x) {
    dist[i] = (i == j.source) ? 0u : WGM_LONESTAR_INF;
    if (SSSP) stamp[i] = 0;
  }
  if (threadIdx.x < 3) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  if (threadIdx.x < 32)
    wgm_cta_push(row, j.piece, threadIdx.x == 0, j.source, &s_cnt[1], wl_start + cap,
                 wl_cnt + cap, wl_u ? wl_u + cap : nullptr, sm->acc[0]);
  __syncthreads();
  int L = 1;
  for (;;) {
    const int n = s_cnt[L % 3];
    if (n == 0 || L > V + 2) break;
    /* the counter of level L-1, read before the previous barrier */
    if (threadIdx.x == 0) s_cnt[(L + 2) % 3] = 0;
    wgm_ls_out o;
    o.counter = &s_cnt[(L + 1) % 3];
    const size_t io = (size_t)(L & 1) * cap, oo = (size_t)((L + 1) & 1) * cap;
    o.o_start = wl_start + oo;
    o.o_cnt = wl_cnt + oo;
    o.o_u = wl_u ? wl_u + oo : nullptr;
    o.cap = cap;
    /* pieces per warp: 32, or fewer when the list is short, so a small
     * frontier spreads over every warp instead of queueing on a few */
    const int per = max(1, min(32, (n + nw - 1) / nw));
    for (int b = warp * per; b < n; b += nw * per) {
      int i = b + lane, deg = 0, start = 0, src = 0;
      if (lane < per && i < n) {
        start = wl_start[io + i];
        deg = wl_cnt[io + i];
        if (SSSP) src = wl_u[io + i];
      }
      wgm_ls_chunk<SSSP, WGM_BATCH_PRECHECK>(row, col, wt, dist, stamp, V, j.piece, L, start,
                                             deg, src, o);
    }
    __syncthreads();
    L++;
  }
  if (threadIdx.x == 0 && B.levels) B.levels[job] = L;
}

/* Team barrier: a counting barrier on the job's arrival line.  `nb` holds
 * the arrivals this member has waited for so far.  Returns false when the
 * wait ran out (err[0] = WGM_DEV_TIMEOUT, err[1] = site) or another CTA
 * already failed. */
__device__ __forceinline__ bool wgm_team_barrier(int *err, unsigned long long spin_ns, int *arr,
                                                 int G, unsigned *nb) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned target = *nb + (unsigned)G;
    *nb = target;
    int ok = 1;
    wgm_red_add_release_gpu(arr, 1);
    const unsigned long long deadline = wgm_globaltimer() + spin_ns;
    unsigned it = 0;
    while ((int)((unsigned)wgm_ld_relaxed_gpu(arr) - target) < 0) {
      if ((++it & 63u) == 0) {
        if (wgm_ld_relaxed_gpu(err) != 0) {
          ok = 0;
          break;
        }
        if (wgm_globaltimer() > deadline) {
          if (atomicCAS(err, 0, WGM_DEV_TIMEOUT) == 0) err[1] = WGM_SITE_BARRIER;
          ok = 0;
          break;
        }
        if (it > 8192u) __nanosleep(64);
      }
    }
    wgm_fence_acqrel_gpu();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

/* One Lonestar BFS/SSSP job as seen by one member of its team. */
struct wgm_ls_job {
  int V, source, piece, cap;
  int G, rank; /* team size, this CTA's rank */
  const int *row, *col;
  const unsigned *wt;
  unsigned *dist;
  int *stamp;
  int *wl_start, *wl_cnt, *wl_u; /* [2][cap] each */
  int *cnt;                      /* 3 level-counter lines, zero at start */
  int *arr;                      /* team barrier arrival line, zero at start */
};

/* Run a job on a team of G > 1 CTAs.  The level loop is the persistent
 * kernel's (wgm_phase_lonestar): device-side init, then one barrier per
 * level with the level counters triple-buffered in the job's control lines.
 * Returns the number of levels (the Lonestar iteration count), or -1 when a
 * team wait failed. */
template <bool SSSP>
__device__ int wgm_team_ls_run(const wgm_ls_job &J, wgm_warp_smem *sm, int *err,
                               unsigned long long spin_ns) {
  const int V = J.V, G = J.G, rank = J.rank, cap = J.cap;
  const int lane = wgm_lane(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  unsigned nb = 0;
  const int tid = rank * blockDim.x + threadIdx.x, nth = G * blockDim.x;
  for (int i = tid; i < V; i += nth) {
    J.dist[i] = (i == J.source) ? 0u : WGM_LONESTAR_INF;
    if (SSSP) J.stamp[i] = 0;
  }
  if (rank == 0 && threadIdx.x < 32)
    wgm_cta_push(J.row, J.piece, threadIdx.x == 0, J.source, &J.cnt[1 * WGM_LINE],
                 J.wl_start + cap, J.wl_cnt + cap, J.wl_u ? J.wl_u + cap : nullptr, sm->acc[0]);
  if (!wgm_team_barrier(err, spin_ns, J.arr, G, &nb)) return -1;
  const int gw = rank * nw + warp, NW = G * nw;
  int L = 1;
  for (;;) {
    const int n = __ldcg(&J.cnt[(L % 3) * WGM_LINE]);
    if (n == 0 || L > V + 2) break;
    if (rank == 0 && threadIdx.x == 0) J.cnt[((L + 2) % 3) * WGM_LINE] = 0;
    wgm_ls_out o;
    o.counter = &J.cnt[((L + 1) % 3) * WGM_LINE];
    const size_t io = (size_t)(L & 1) * cap, oo = (size_t)((L + 1) & 1) * cap;
    o.o_start = J.wl_start + oo;
    o.o_cnt = J.wl_cnt + oo;
    o.o_u = J.wl_u ? J.wl_u + oo : nullptr;
    o.cap = cap;
    /* pieces per warp: 32, or fewer when the list is short, so a small
     * frontier spreads over every warp instead of queueing on a few */
    const int per = max(1, min(32, (n + NW - 1) / NW));
    for (int b = gw * per; b < n; b += NW * per) {
      int i = b + lane, deg = 0, start = 0, src = 0;
      if (lane < per && i < n) {
        start = __ldcg(&J.wl_start[io + i]);
        deg = __ldcg(&J.wl_cnt[io + i]);
        if (SSSP) src = __ldcg(&J.wl_u[io + i]);
      }
      wgm_ls_chunk<SSSP, WGM_BATCH_PRECHECK>(J.row, J.col, J.wt, J.dist, J.stamp, V, J.piece, L,
                                             start, deg, src, o);
    }
    if (!wgm_team_barrier(err, spin_ns, J.arr, G, &nb)) return -1;
    L++;
  }
  return L;
}

/* One batch job on a team of G > 1 CTAs; this CTA is member `rank`. */
template <bool SSSP>
__device__ void wgm_team_lonestar(const wgm_batch_args &B, const wgm_batch_job &j, int job,
                                  int rank, wgm_warp_smem *sm) {
  wgm_ls_job J;
  J.V = j.V;
  J.source = j.source;
  J.piece = j.piece;
  J.cap = j.cap;
  J.G = j.team;
  J.rank = rank;
  J.row = B.rows + j.row_off;
  J.col = B.cols + j.col_off;
  J.wt = SSSP ? B.wts + j.col_off : nullptr;
  J.dist = B.dist + j.dist_off;
  J.stamp = SSSP ? B.stamp + j.stamp_off : nullptr;
  J.wl_start = B.scratch + j.wl_off;
  J.wl_cnt = J.wl_start + 2 * (size_t)j.cap;
  J.wl_u = SSSP ? J.wl_cnt + 2 * (size_t)j.cap : nullptr;
  int *ctl = B.ctl + (size_t)(1 + job * WGM_BATCH_CTL_LINES_PER_JOB) * WGM_LINE;
  J.cnt = ctl;
  J.arr = ctl + 3 * WGM_LINE;
  const int L = wgm_team_ls_run<SSSP>(J, sm, B.err, B.spin_ns);
  if (L > 0 && rank == 0 && threadIdx.x == 0 && B.levels) B.levels[job] = L;
}

#endif
