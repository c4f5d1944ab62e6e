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

/* Whether batch BFS jobs read dist[dst] before the atomic (one more
 * dependent load, fewer atomics): no.  Most BFS claims fail (one per
 * reached vertex out of one per edge: 6 % succeed on the batch's RMAT
 * graphs, 25 % on its grids), yet the CAS alone measured as fast or faster
 * (7.06-7.12 against 7.08-7.32 ms at 512 x 2 CTAs, 7.8-8.0 against 8.2-8.4
 * at 256 x 3): the load it would save sits on the same chain.  SSSP jobs
 * always pre-check: on the RMAT graphs most relaxations fail, and the
 * 64-bit atomics they skip cost more than the load (the batch's RMAT SSSP
 * CTA time fell 12 %, the launch 3.5 %). */
#ifndef WGM_BATCH_PRECHECK
#define WGM_BATCH_PRECHECK false
#endif

/* Edge windows per warp batch in the batched kernel.  Fewer than the
 * standalone walker's four: the batched kernel is one function inlining
 * every job loop, so each window's registers are scarce, and a warp's
 * pieces on the batch's small and sparse graphs rarely fill four windows.
 * Measured on the 512-graph batch at 512 x 2 CTAs, 64 registers: 9.07 ms
 * with 4 windows, 8.05 with 3, 7.5 with 2, 8.9 with 1 (the same order at
 * 256 x 3 / 80 registers and 1024 x 1). */
#ifndef WGM_BATCH_LS_K
#define WGM_BATCH_LS_K 2
#endif

/* Shared-memory counters of a one-CTA job: three level counters, far-list
 * counts and least distances, heavy-list counts, three chunk-grab counters. */
#define WGM_BATCH_SCNT 13

struct wgm_batch_job {
  int V;
  int algo;   /* 0 = BFS, 1 = SSSP */
  int source;
  int piece;
  long long row_off;  /* row_ptr of the graph: rows[row_off .. row_off+V] */
  long long col_off;  /* col / weights of the graph start here */
  long long dist_off; /* output dist[V] */
  long long wl_off;   /* scratch: 3 x 2 x cap ints (start, cnt, u), then (SSSP)
                         2 x far_cap ints: the near-far schedule's far lists */
  long long stamp_off;/* scratch: 2V ints (stamps, or SSSP {tag, dist} words) */
  int cap;
  unsigned delta; /* SSSP near-far bucket width (0: Bellman-Ford worklist) */
  int far_cap;    /* entries per far list */
  unsigned light; /* near-far SSSP: edges of weight >= light are heavy, relaxed
                     once per bucket (0: every edge at every visit); the
                     scratch then also holds two heavy lists (3 x cap ints
                     each) and a settle stamp per vertex after the far lists */
  int graph; /* graph index (host bookkeeping) */
  int team;  /* CTAs working on the job */
  int boost; /* host: team size in percent of the edge rule's (critical-path
                pass of the autotuner; 100 = the rule) */
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
  int lq_rounds;             /* 0: plain levels; > 0: warp-local continuation */
  unsigned long long spin_ns;
};

/* ---- warp-local continuation (batch jobs) --------------------------------
 *
 * A batch job relaxes by atomic_min for BFS too (unit weights: the fixpoint
 * is the hop distance, which is the Lonestar BFS level), so the order of
 * relaxations does not matter and a warp may relax a vertex it has just
 * improved again within the same level instead of queueing it for the next
 * one.  High-diameter graphs (the 512x512 grids of the batch run ~1000
 * levels) then advance several hops per level.
 *
 * Stamps: stamp[v] == L means "v is queued (globally for level L+1, or in
 * some warp's local queue) and nobody has started to relax it".  The claim
 * after an improvement is an acq_rel exchange to L; a warp about to relax a
 * locally queued vertex first exchanges the stamp away (acq_rel) and only
 * then reads dist[v].  An improvement that lands after that exchange sees a
 * stamp != L and queues v again; one that landed before it is ordered
 * before the exchange (its claim exchange was read by ours), so our read of
 * dist[v] sees it.  Every improvement is therefore followed by a relaxation
 * that reads it, which is all the fixpoint needs. */
#define WGM_LQ 32   /* local queue entries per warp and buffer */
#define WGM_LQ_ROUNDS_MAX 12

struct wgm_lq {     /* per warp, dynamic shared memory */
  int v[2][WGM_LQ];
  int rs[2][WGM_LQ];
  int d[2][WGM_LQ];
  int n[2];
};

__device__ __forceinline__ int wgm_atom_exch_acqrel_gpu(int *p, int v) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;"
               : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

/* wgm_ls_chunk with atomic_min relaxation for both algorithms and a local
 * sink: a claimed vertex of at most one piece goes to the warp's next local
 * buffer while it has room, everything else to the global list. */
template <bool SSSP>
__device__ __forceinline__ bool wgm_ls_chunk_async(const int *row, const int *col,
                                                   const unsigned *wt, unsigned *dist,
                                                   int *stamp, int V, int P, int L, int start,
                                                   int deg, int src, const wgm_ls_out &o,
                                                   wgm_lq *q, int nb) {
  constexpr int K = WGM_LS_K;
  const int lane = wgm_lane();
  const int incl = wgm_warp_incl_scan(deg);
  const int total = __shfl_sync(WGM_FULL, incl, 31);
  const int off = incl - deg;
  const int base = start - off;
  bool ok = true;
  for (int w = 0; w < total; w += 32 * K) {
    int e[K], u[K], rs[K], d[K], np[K], sv[K];
    unsigned alt[K];
    bool f[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const int s = w + 32 * k + lane;
      f[k] = s < total;
      const int own = wgm_owner_of(off, min(s, total - 1));
      e[k] = __shfl_sync(WGM_FULL, base, own) + s;
      sv[k] = __shfl_sync(WGM_FULL, src, own);
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      u[k] = f[k] ? __ldg(&col[e[k]]) : -1;
      unsigned wk = 1u;
      if (SSSP) wk = f[k] ? __ldg(&wt[e[k]]) : WGM_LONESTAR_INF;
      const unsigned dvk = f[k] ? __ldcg(&dist[sv[k]]) : 0u;
      f[k] = f[k] && wk < WGM_LONESTAR_INF && dvk < WGM_LONESTAR_INF; /* sssp.cl:120 */
      alt[k] = dvk + wk;
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      f[k] = f[k] && (unsigned)u[k] < (unsigned)V; /* bfs.cl:116 */
      rs[k] = 0;
      d[k] = 0;
      if (f[k]) {
        f[k] = alt[k] < atomicMin(&dist[u[k]], alt[k]);
        rs[k] = __ldg(&row[u[k]]);
        d[k] = __ldg(&row[u[k] + 1]);
      }
    }
    int mine = 0;
    bool loc[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      if (f[k]) f[k] = wgm_atom_exch_acqrel_gpu(&stamp[u[k]], L) != L;
      d[k] = f[k] ? max(d[k] - rs[k], 0) : 0; /* a vertex without edges is not queued */
      np[k] = (d[k] + P - 1) / P;
      /* one-piece vertices go to the local queue while it has room */
      const unsigned want = __ballot_sync(WGM_FULL, np[k] == 1);
      const int have = q->n[nb];
      const int pos = have + __popc(want & wgm_lanemask_lt());
      loc[k] = np[k] == 1 && pos < WGM_LQ;
      if (loc[k]) {
        q->v[nb][pos] = u[k];
        q->rs[nb][pos] = rs[k];
        q->d[nb][pos] = d[k];
        np[k] = 0;
      }
      __syncwarp();
      if (lane == 0) q->n[nb] = min(WGM_LQ, have + __popc(want));
      __syncwarp();
      mine += np[k];
    }
    const int pincl = wgm_warp_incl_scan(mine);
    const int ptotal = __shfl_sync(WGM_FULL, pincl, 31);
    if (ptotal == 0) continue;
    int pbase = 0;
    if (lane == 31) pbase = wgm_out_reserve(o, ptotal);
    pbase = __shfl_sync(WGM_FULL, pbase, 31);
    if (pbase + ptotal > o.cap) {
      ok = false;
      continue;
    }
    int slot = pbase + pincl - mine;
    int sl[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      sl[k] = slot;
      if (np[k] <= WGM_LS_LANE_PIECES) {
        for (int qq = 0; qq < np[k]; qq++) {
          o.o_start[slot + qq] = rs[k] + qq * P;
          o.o_cnt[slot + qq] = min(P, d[k] - qq * P);
          o.o_u[slot + qq] = u[k];
        }
      }
      slot += np[k];
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      unsigned big = __ballot_sync(WGM_FULL, np[k] > WGM_LS_LANE_PIECES);
      while (big) {
        const int j = __ffs(big) - 1;
        big &= big - 1;
        const int bs = __shfl_sync(WGM_FULL, rs[k], j), bd = __shfl_sync(WGM_FULL, d[k], j);
        const int bu = __shfl_sync(WGM_FULL, u[k], j), bsl = __shfl_sync(WGM_FULL, sl[k], j);
        const int bn = (bd + P - 1) / P;
        for (int qq = lane; qq < bn; qq += 32) {
          o.o_start[bsl + qq] = bs + qq * P;
          o.o_cnt[bsl + qq] = min(P, bd - qq * P);
          o.o_u[bsl + qq] = bu;
        }
      }
    }
  }
  return ok;
}

/* After a warp's share of a level: relax the locally queued vertices for up
 * to WGM_LQ_ROUNDS rounds (each round's improvements feed the next), then
 * move what is left to the global list for the next level (still claimed). */
template <bool SSSP>
__device__ __forceinline__ bool wgm_ls_local_rounds(const int *row, const int *col,
                                                    const unsigned *wt, unsigned *dist,
                                                    int *stamp, int V, int P, int L,
                                                    const wgm_ls_out &o, wgm_lq *q,
                                                    int rounds) {
  const int lane = wgm_lane();
  bool ok = true;
  int cur = 0;
  for (int round = 0; round < rounds; round++) {
    const int n = q->n[cur];
    if (n == 0) return ok;
    const int nxt = cur ^ 1;
    __syncwarp();
    if (lane == 0) q->n[nxt] = 0;
    __syncwarp();
    const bool have = lane < n;
    const int v = have ? q->v[cur][lane] : 0;
    const int rs = have ? q->rs[cur][lane] : 0;
    const int d = have ? q->d[cur][lane] : 0;
    if (lane == 0) q->n[cur] = 0;
    __syncwarp();
    if (have) wgm_atom_exch_acqrel_gpu(&stamp[v], -1); /* unclaim, then read dist[v] */
    __syncwarp(); /* the lanes that read dist[v] are ordered after the unclaim */
    ok &= wgm_ls_chunk_async<SSSP>(row, col, wt, dist, stamp, V, P, L, rs, have ? d : 0, v, o,
                                   q, nxt);
    cur = nxt;
  }
  /* budget spent: the rest goes to the next level as one piece each */
  const int n = q->n[cur];
  if (n == 0) return ok;
  const bool have = lane < n;
  int base = 0;
  if (lane == 0) base = wgm_out_reserve(o, n);
  base = __shfl_sync(WGM_FULL, base, 0);
  if (base + n > o.cap) return false;
  if (have) {
    o.o_start[base + lane] = q->rs[cur][lane];
    o.o_cnt[base + lane] = q->d[cur][lane];
    o.o_u[base + lane] = q->v[cur][lane];
  }
  __syncwarp();
  if (lane == 0) q->n[cur] = 0;
  __syncwarp();
  return ok;
}

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

/* Near-far schedule for batched SSSP (packed words only).  A level relaxes
 * the near list; an improved vertex whose distance reaches the threshold T
 * is parked in the far list (vertex ids, one list filled while the other
 * is drained).  When a level ends with no near work but a non-empty far
 * list, a split step raises T to max(T, least parked distance) + delta and
 * queues every parked vertex now below T as pieces (one copy per vertex:
 * the first to exchange the word's tag to the split's level), moving the
 * rest to the other far list.  Any order of relaxations that relaxes every
 * improved vertex again reaches the same fixpoint, so the distances are
 * those of the Bellman-Ford worklist; only the work changes: on a 512x512
 * grid with weights U[1,1000] the worklist relaxes every edge ~27 times,
 * near-far with delta = 20 x the mean weight ~3 times, for ~20 % more
 * levels.  A far list that is full sends the vertex to the near list. */
__device__ __forceinline__ bool wgm_nf_split(const int *row, int P, unsigned *dw, int L,
                                             const int *src, int nsrc, unsigned Tn, int gw,
                                             int NW, const wgm_ls_out &o, int *dst,
                                             int *dst_cnt, unsigned *dst_min, int dst_cap) {
  bool ok = true;
  const int lane = wgm_lane();
  for (int b = gw * 32; b < nsrc; b += NW * 32) {
    const int i = b + lane;
    int v = 0;
    unsigned dv = 0;
    bool keep = false;
    if (i < nsrc) {
      v = __ldcg(&src[i]);
      dv = __ldcg(&dw[2 * v + 1]);
      keep = dv >= Tn;
    }
    const unsigned kb = __ballot_sync(WGM_FULL, keep);
    if (kb) {
      int base = 0;
      if (lane == 0) base = atomicAdd(dst_cnt, __popc(kb));
      base = __shfl_sync(WGM_FULL, base, 0);
      const int slot = base + __popc(kb & wgm_lanemask_lt());
      unsigned m = 0xffffffffu;
      if (keep) {
        if (slot < dst_cap) {
          dst[slot] = v;
          m = dv;
        } else {
          keep = false; /* far list full: relax it now */
        }
      }
#pragma unroll
      for (int x = 16; x > 0; x >>= 1) m = min(m, __shfl_xor_sync(WGM_FULL, m, x));
      if (lane == 0 && m != 0xffffffffu) atomicMin(dst_min, m);
    }
    bool mv = false;
    if (i < nsrc && !keep) mv = atomicExch(&dw[2 * v], (unsigned)L) != (unsigned)L;
    ok &= wgm_out_push_vertices(row, P, mv, v, o);
  }
  return ok;
}

/* Near-far bookkeeping shared by the CTA and team level loops.  Every
 * member runs it on the same values, so all take the same steps. */
struct wgm_nf_state {
  unsigned T;
  int fb;   /* far list receiving parked vertices */
  int pend; /* far list drained by the last split: cleared at the next step */
  bool split_last;
  /* heavy-edge deferral: the heavy epoch (heavy steps so far + 1); its
   * parity selects the heavy list being filled */
  int ep = 1;
};

/* Heavy-edge deferral (delta-stepping's light/heavy split on the near-far
 * buckets).  The levels of a bucket relax only light edges (weight < light,
 * light = the bucket width).  A vertex whose first piece a level visits is
 * also appended to the heavy list of the current epoch, unless its settle
 * stamp already names that epoch (it is listed and not yet relaxed).  When
 * the near list runs dry and the heavy list is not empty, a heavy step
 * relaxes the heavy edges of the listed vertices, with their distances as
 * they stand then, and the next epoch begins with the other list.  Any
 * improvement of a vertex is followed by a visit (the near-far schedule
 * visits every improved vertex), which lists it for a heavy step that runs
 * later and reads its distance then; so every improvement is still followed
 * by the relaxation of all its edges and the fixpoint is the same.  With
 * exact buckets a heavy edge from bucket [lo, T) lands at or above T and
 * waits in the far list, so there is one heavy step per bucket and each
 * vertex is relaxed through its heavy edges once; a list holds a vertex at
 * most once, so it fits in cap entries.  On RMAT graphs with weights
 * U[1,1000] the Bellman-Ford bucket reads every edge ~4 times; buckets of
 * 0.2 x the mean weight with deferral read it ~2 times and relax ~1 time. */
struct wgm_heavy_lists {
  int *buf;    /* 2 x 3 x cap: (start, count, vertex) by epoch parity */
  int *settle; /* [V] the epoch whose heavy list holds the vertex */
  int cap;
  __device__ __forceinline__ int *start(int p) const { return buf + (size_t)p * 3 * cap; }
  __device__ __forceinline__ int *cnt(int p) const { return start(p) + cap; }
  __device__ __forceinline__ int *vtx(int p) const { return start(p) + 2 * (size_t)cap; }
};

/* A warp's pieces of one light level: lanes holding a vertex's first piece
 * whose settle stamp was not yet this epoch's append the vertex's pieces to
 * the epoch's heavy list (counter hc). */
__device__ __forceinline__ void wgm_heavy_note(const int *row, int P, bool valid, int start,
                                               int src, const wgm_heavy_lists &H, int ph,
                                               int ep, int *hc) {
  bool first = false;
  if (valid && start == __ldg(&row[src]))
    first = atomicExch(&H.settle[src], ep) != ep;
  wgm_ls_out h;
  h.counter = hc;
  h.o_start = H.start(ph);
  h.o_cnt = H.cnt(ph);
  h.o_u = H.vtx(ph);
  h.cap = H.cap;
  wgm_out_push_vertices(row, P, first, src, h);
}

/* Edges a job walked (relaxations tried, every visit of a vertex counts its
 * edges again): a 64-bit counter at int offset 24 of the job's arrival line,
 * cleared with the control block before each launch.  One atomic per warp
 * when the job ends. */
#define WGM_BATCH_WORK_OFF 24
__device__ __forceinline__ void wgm_batch_add_work(int *arr_line, unsigned long long walked) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) walked += __shfl_xor_sync(WGM_FULL, walked, o);
  if (wgm_lane() == 0 && walked)
    atomicAdd(reinterpret_cast<unsigned long long *>(arr_line + WGM_BATCH_WORK_OFF), walked);
}

/* One job on one CTA.  s_cnt: 3 shared level counters, then (s_cnt[4..7])
 * the two far-list counts and least parked distances, then (s_cnt[8..9])
 * the two heavy-list counts. */
template <bool SSSP, bool ASYNC, bool DEFER = false>
__device__ void wgm_cta_lonestar(const wgm_batch_args &B, const wgm_batch_job &j, int job,
                                 int *s_cnt, wgm_warp_smem *sm, wgm_lq *q) {
  const int V = j.V;
  const int *row = B.rows + j.row_off;
  const int *col = B.cols + j.col_off;
  const unsigned *wt = SSSP ? B.wts + j.col_off : nullptr;
  unsigned *dist = B.dist + j.dist_off;
  int *stamp = B.stamp + j.stamp_off;
  const int cap = j.cap;
  int *wl_start = B.scratch + j.wl_off;
  int *wl_cnt = wl_start + 2 * (size_t)cap;
  int *wl_u = wl_cnt + 2 * (size_t)cap;
  const int lane = wgm_lane(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  /* SSSP without the local queues relaxes packed {tag, distance} words in
   * the stamp scratch and copies the distances out at the end */
  constexpr bool PACK = SSSP && !ASYNC;
  unsigned *dw = PACK ? reinterpret_cast<unsigned *>(stamp) : dist;
  const bool nf = PACK && j.delta > 0;
  const bool defer = DEFER && nf && j.light > 0;
  int *far = wl_u + 2 * (size_t)cap;
  wgm_heavy_lists H;
  H.buf = far + 2 * (size_t)j.far_cap;
  H.settle = H.buf + 6 * (size_t)cap;
  H.cap = cap;
  for (int i = threadIdx.x; i < V; i += blockDim.x) {
    if (PACK) {
      reinterpret_cast<unsigned long long *>(stamp)[i] =
          (i == j.source) ? 0ull : (unsigned long long)WGM_LONESTAR_INF << 32;
      if (defer) H.settle[i] = 0;
    } else {
      dist[i] = (i == j.source) ? 0u : WGM_LONESTAR_INF;
      stamp[i] = 0;
    }
  }
  if (threadIdx.x < WGM_BATCH_SCNT)
    s_cnt[threadIdx.x] = (threadIdx.x == 6 || threadIdx.x == 7) ? (int)0xffffffffu : 0;
  if (lane == 0) q->n[0] = q->n[1] = 0;
  __syncthreads();
  if (threadIdx.x < 32)
    wgm_cta_push(row, j.piece, threadIdx.x == 0, j.source, &s_cnt[1], wl_start + cap,
                 wl_cnt + cap, wl_u ? wl_u + cap : nullptr, sm->acc[0]);
  __syncthreads();
  int *fctl = s_cnt + 4;
  int *hcnt = s_cnt + 8;
  wgm_nf_state ns{nf ? j.delta : 0xffffffffu, 0, -1, false};
  const int Lmax = nf ? (defer ? 8 : 4) * V + 16 : V + 2;
  unsigned long long walked = 0;
  int L = 1;
  for (;;) {
    const int n = s_cnt[L % 3];
    int step = 0, nfar = 0; /* 0: level, 1: split, 2: clear only, 3: heavy */
    const int hn = defer ? hcnt[ns.ep & 1] : 0;
    if (n == 0) {
      if (!nf) break;
      if (hn > 0) {
        step = 3;
      } else {
        nfar = fctl[ns.fb];
        if (nfar == 0) break;
        step = ns.split_last ? 2 : 1;
      }
    }
    if (L > Lmax) break;
    /* the counter of level L-1, read before the previous barrier; the grab
     * counter of level L-1, whose last grab came before that barrier */
    if (threadIdx.x == 0) {
      s_cnt[(L + 2) % 3] = 0;
      s_cnt[10 + (L + 2) % 3] = 0;
      if (ns.pend >= 0) {
        fctl[ns.pend] = 0;
        fctl[2 + ns.pend] = (int)0xffffffffu;
      }
      /* the next epoch's heavy list, last read at the heavy step before */
      if (step == 3) hcnt[(ns.ep + 1) & 1] = 0;
    }
    ns.pend = -1;
    wgm_ls_out o;
    o.counter = &s_cnt[(L + 1) % 3];
    const size_t io = (size_t)(L & 1) * cap, oo = (size_t)((L + 1) & 1) * cap;
    o.o_start = wl_start + oo;
    o.o_cnt = wl_cnt + oo;
    o.o_u = wl_u ? wl_u + oo : nullptr;
    o.cap = cap;
    if (nf) {
      o.far_cnt = &fctl[ns.fb];
      o.far_min = reinterpret_cast<unsigned *>(&fctl[2 + ns.fb]);
      o.far_list = far + (size_t)ns.fb * j.far_cap;
      o.far_cap = j.far_cap;
      o.T = ns.T;
    }
    if (defer) {
      o.wlo = step == 3 ? j.light : 0u;
      o.whi = step == 3 ? 0xffffffffu : j.light;
    }
    if (step == 1) {
      const unsigned fmin = (unsigned)fctl[2 + ns.fb];
      const unsigned Tn =
          (unsigned)min(0xffffffffull, (unsigned long long)max(ns.T, fmin) + j.delta);
      const int nb = ns.fb ^ 1;
      /* the count also holds pushes that found the list full (never stored) */
      wgm_nf_split(row, j.piece, dw, L, far + (size_t)ns.fb * j.far_cap, min(nfar, j.far_cap),
                   Tn, warp, nw, o,
                   far + (size_t)nb * j.far_cap, &fctl[nb],
                   reinterpret_cast<unsigned *>(&fctl[2 + nb]), j.far_cap);
      ns.T = Tn;
      ns.pend = ns.fb;
      ns.fb = nb;
    }
    ns.split_last = step == 1;
    /* the list this level walks: the near list, or the epoch's heavy list */
    const int *ls = wl_start + io, *lc = wl_cnt + io, *lu = wl_u ? wl_u + io : nullptr;
    int m = n;
    if (step == 3) {
      ls = H.start(ns.ep & 1);
      lc = H.cnt(ns.ep & 1);
      lu = H.vtx(ns.ep & 1);
      m = min(hn, cap); /* a list holds a vertex once per epoch: never more */
    }
    const int lb = 0;
    /* pieces per warp: 32, or fewer when the list is short, so a small
     * frontier spreads over every warp instead of queueing on a few */
    const int per = max(1, min(32, (m + nw - 1) / nw));
    /* warps take chunks of `per` pieces from a shared-memory counter as
     * they finish the last, so a warp that drew heavy pieces does not hold
     * the level's barrier while the others wait (level L's counter was
     * cleared at level L-2) */
    int *grab = &s_cnt[10 + L % 3];
    for (;;) {
      int b = 0;
      if (lane == 0) b = atomicAdd(grab, per);
      b = __shfl_sync(WGM_FULL, b, 0);
      if (b >= m) break;
      int i = b + lane, deg = 0, start = 0, src = 0;
      const bool valid = lane < per && i < m;
      if (valid) {
        start = ls[lb + i];
        deg = lc[lb + i];
        src = lu[lb + i];
        walked += deg;
      }
      if (defer && step == 0)
        wgm_heavy_note(row, j.piece, valid, start, src, H, ns.ep & 1, ns.ep, &hcnt[ns.ep & 1]);
      if (ASYNC)
        wgm_ls_chunk_async<SSSP>(row, col, wt, dist, stamp, V, j.piece, L, start, deg, src, o,
                                 q, 0);
      else
        wgm_ls_chunk<SSSP, WGM_BATCH_PRECHECK || SSSP, PACK, WGM_BATCH_LS_K>(
            row, col, wt, dw, stamp, V, j.piece, L, start, deg, src, o);
    }
    if (ASYNC) wgm_ls_local_rounds<SSSP>(row, col, wt, dist, stamp, V, j.piece, L, o, q,
                                         B.lq_rounds);
    if (step == 3) ns.ep++;
    __syncthreads();
    L++;
  }
  if (PACK)
    for (int i = threadIdx.x; i < V; i += blockDim.x) dist[i] = dw[2 * i + 1];
  if (threadIdx.x == 0 && B.levels) B.levels[job] = L;
  wgm_batch_add_work(B.ctl + (size_t)(1 + job * WGM_BATCH_CTL_LINES_PER_JOB + 3) * WGM_LINE,
                     walked);
}

/* Team barrier: a counting barrier on the job's arrival line.  An arrival
 * is one red.release; the waiters poll with ld.acquire, which synchronises
 * with every arrival through the counter's chain of read-modify-writes (a
 * relaxed poll followed by a fence measured several hundred ns slower per
 * barrier on GB300).  `nb` holds the arrivals this member has waited for so
 * far.  Returns false when the
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
    while ((int)((unsigned)wgm_ld_acquire_gpu(arr) - target) < 0) {
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
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

/* End of a team level: one barrier whose poll also returns the next
 * level's size.  The level word packs the pieces queued for the next level
 * (low half, bumped by the pushes) and the team's arrivals (high half);
 * each member arrives with one 64-bit red.release after all its pushes, so
 * the ld.acquire that sees G arrivals reads the final piece count in the
 * same word - no separate counter read after the barrier.  Returns the
 * count, or -1 when the wait ran out (err[0] = WGM_DEV_TIMEOUT) or another
 * CTA already failed. */
__device__ __forceinline__ int wgm_team_level_barrier(int *err, unsigned long long spin_ns,
                                                      unsigned long long *word, int G) {
  __shared__ int s_n;
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(word), "l"(1ull << 32)
                 : "memory");
    const unsigned long long deadline = wgm_globaltimer() + spin_ns;
    unsigned it = 0;
    unsigned long long v;
    int n;
    for (;;) {
      asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(word) : "memory");
      if ((int)(v >> 32) >= G) {
        n = (int)(unsigned)v;
        break;
      }
      if ((++it & 63u) == 0) {
        if (wgm_ld_relaxed_gpu(err) != 0) {
          n = -1;
          break;
        }
        if (wgm_globaltimer() > deadline) {
          if (atomicCAS(err, 0, WGM_DEV_TIMEOUT) == 0) err[1] = WGM_SITE_BARRIER;
          n = -1;
          break;
        }
        if (it > 8192u) __nanosleep(64);
      }
    }
    s_n = n;
  }
  __syncthreads();
  return s_n;
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
  int *cnt;                      /* 3 level-counter lines, first 8 bytes of each zero at start */
  int *arr;                      /* team barrier arrival line, zero at start */
  int lq_rounds;                 /* warp-local continuation rounds (async runs) */
  unsigned delta = 0;            /* packed SSSP: near-far bucket width (0: worklist) */
  int far_cap = 0;               /* entries per far list (after wl_u's 2 x cap) */
  unsigned light = 0;            /* near-far: heavy edges deferred (wgm_batch_job.light) */
};

/* Run a job on a team of G > 1 CTAs.  The level loop is the persistent
 * kernel's (wgm_phase_lonestar): device-side init, then one barrier per
 * level with the level counters triple-buffered in the job's control lines.
 * Returns the number of levels (the Lonestar iteration count), or -1 when a
 * team wait failed. */
template <bool SSSP, bool ASYNC = false, bool DEFER = false>
__device__ int wgm_team_ls_run(const wgm_ls_job &J, wgm_warp_smem *sm, int *err,
                               unsigned long long spin_ns, wgm_lq *q = nullptr) {
  const int V = J.V, G = J.G, rank = J.rank, cap = J.cap;
  const int lane = wgm_lane(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __shared__ int s_grab[3]; /* chunk grab counters by level mod 3 */
  if (threadIdx.x < 3) s_grab[threadIdx.x] = 0;
  unsigned nb = 0;
  const int tid = rank * blockDim.x + threadIdx.x, nth = G * blockDim.x;
  constexpr bool PACK = SSSP && !ASYNC; /* as in wgm_cta_lonestar */
  unsigned *dw = PACK ? reinterpret_cast<unsigned *>(J.stamp) : J.dist;
  const bool nf = PACK && J.delta > 0;
  const bool defer = DEFER && nf && J.light > 0;
  wgm_heavy_lists H;
  H.buf = J.wl_u + 2 * (size_t)cap + 2 * (size_t)J.far_cap;
  H.settle = H.buf + 6 * (size_t)cap;
  H.cap = cap;
  for (int i = tid; i < V; i += nth) {
    if (PACK) {
      reinterpret_cast<unsigned long long *>(J.stamp)[i] =
          (i == J.source) ? 0ull : (unsigned long long)WGM_LONESTAR_INF << 32;
      if (defer) H.settle[i] = 0;
    } else {
      J.dist[i] = (i == J.source) ? 0u : WGM_LONESTAR_INF;
      if (SSSP || ASYNC) J.stamp[i] = 0;
    }
  }
  if (ASYNC && lane == 0) q->n[0] = q->n[1] = 0;
  /* far-list counts [0..1] and least parked distances [2..3], on the
   * arrival line after its counter */
  int *fctl = J.arr + 8;
  if (rank == 0 && threadIdx.x == 0 && nf) fctl[2] = fctl[3] = (int)0xffffffffu;
  if (rank == 0 && threadIdx.x < 32)
    wgm_cta_push(J.row, J.piece, threadIdx.x == 0, J.source, &J.cnt[1 * WGM_LINE],
                 J.wl_start + cap, J.wl_cnt + cap, J.wl_u ? J.wl_u + cap : nullptr, sm->acc[0]);
  if (!wgm_team_barrier(err, spin_ns, J.arr, G, &nb)) return -1;
  const int gw = rank * nw + warp, NW = G * nw;
  /* level words: the first 8 bytes of the three counter lines; level L
   * reads word L%3, pushes into word (L+1)%3 and clears word (L+2)%3, whose
   * last poll (the barrier ending level L-2) every member has passed */
  unsigned long long *lw = reinterpret_cast<unsigned long long *>(J.cnt);
  int n = __ldcg(&J.cnt[1 * WGM_LINE]);
  int *far = nf ? J.wl_u + 2 * (size_t)cap : nullptr;
  /* heavy-list counts [16..17] of the same line (zeroed with the control
   * block before the launch) */
  int *hcnt = J.arr + 16;
  wgm_nf_state ns{nf ? J.delta : 0xffffffffu, 0, -1, false};
  const int Lmax = nf ? (defer ? 8 : 4) * V + 16 : V + 2;
  unsigned long long walked = 0;
  int L = 1;
  for (;;) {
    int step = 0, nfar = 0; /* 0: level, 1: split, 2: clear only, 3: heavy */
    const int hn = defer ? __ldcg(&hcnt[ns.ep & 1]) : 0;
    if (n == 0) {
      if (!nf) break;
      if (hn > 0) {
        step = 3;
      } else {
        nfar = __ldcg(&fctl[ns.fb]);
        if (nfar == 0) break;
        step = ns.split_last ? 2 : 1;
      }
    }
    if (L > Lmax) break;
    if (threadIdx.x == 0) s_grab[(L + 2) % 3] = 0; /* as in wgm_cta_lonestar */
    if (rank == 0 && threadIdx.x == 0) {
      lw[((L + 2) % 3) * (WGM_LINE / 2)] = 0ull;
      /* every member read the drained list's count before the last barrier */
      if (ns.pend >= 0) {
        fctl[ns.pend] = 0;
        fctl[2 + ns.pend] = (int)0xffffffffu;
      }
      /* the next epoch's heavy list: appended to only after this level's
       * barrier, last read at the heavy step before */
      if (step == 3) hcnt[(ns.ep + 1) & 1] = 0;
    }
    ns.pend = -1;
    wgm_ls_out o;
    o.counter = nullptr;
    o.counter64 = &lw[((L + 1) % 3) * (WGM_LINE / 2)];
    const size_t io = (size_t)(L & 1) * cap, oo = (size_t)((L + 1) & 1) * cap;
    o.o_start = J.wl_start + oo;
    o.o_cnt = J.wl_cnt + oo;
    o.o_u = J.wl_u ? J.wl_u + oo : nullptr;
    o.cap = cap;
    if (nf) {
      o.far_cnt = &fctl[ns.fb];
      o.far_min = reinterpret_cast<unsigned *>(&fctl[2 + ns.fb]);
      o.far_list = far + (size_t)ns.fb * J.far_cap;
      o.far_cap = J.far_cap;
      o.T = ns.T;
    }
    if (defer) {
      o.wlo = step == 3 ? J.light : 0u;
      o.whi = step == 3 ? 0xffffffffu : J.light;
    }
    if (step == 1) {
      const unsigned fmin = (unsigned)__ldcg(&fctl[2 + ns.fb]);
      const unsigned Tn =
          (unsigned)min(0xffffffffull, (unsigned long long)max(ns.T, fmin) + J.delta);
      const int nb2 = ns.fb ^ 1;
      /* the count also holds pushes that found the list full (never stored) */
      wgm_nf_split(J.row, J.piece, dw, L, far + (size_t)ns.fb * J.far_cap, min(nfar, J.far_cap),
                   Tn, gw, NW, o,
                   far + (size_t)nb2 * J.far_cap, &fctl[nb2],
                   reinterpret_cast<unsigned *>(&fctl[2 + nb2]), J.far_cap);
      ns.T = Tn;
      ns.pend = ns.fb;
      ns.fb = nb2;
    }
    ns.split_last = step == 1;
    /* the list this level walks: the near list, or the epoch's heavy list */
    const int *ls = J.wl_start + io, *lc = J.wl_cnt + io;
    const int *lu = J.wl_u ? J.wl_u + io : nullptr;
    int m = n;
    if (step == 3) {
      ls = H.start(ns.ep & 1);
      lc = H.cnt(ns.ep & 1);
      lu = H.vtx(ns.ep & 1);
      m = min(hn, cap); /* a list holds a vertex once per epoch: never more */
    }
    const int lb = 0;
    /* pieces per warp: 32, or fewer when the list is short, so a small
     * frontier spreads over every warp instead of queueing on a few */
    const int per = max(1, min(32, (m + NW - 1) / NW));
    /* chunk c of `per` pieces belongs to member c mod G; the member's warps
     * take its chunks from a shared-memory counter as they finish the last */
    for (;;) {
      int t = 0;
      if (lane == 0) t = atomicAdd(&s_grab[L % 3], 1);
      t = __shfl_sync(WGM_FULL, t, 0);
      const long long bc = ((long long)t * G + rank) * per;
      if (bc >= m) break;
      const int b = (int)bc;
      int i = b + lane, deg = 0, start = 0, src = 0;
      const bool valid = lane < per && i < m;
      if (valid) {
        start = __ldcg(&ls[lb + i]);
        deg = __ldcg(&lc[lb + i]);
        if (SSSP || ASYNC) src = __ldcg(&lu[lb + i]);
        walked += deg;
      }
      if (defer && step == 0)
        wgm_heavy_note(J.row, J.piece, valid, start, src, H, ns.ep & 1, ns.ep,
                       &hcnt[ns.ep & 1]);
      if (ASYNC)
        wgm_ls_chunk_async<SSSP>(J.row, J.col, J.wt, J.dist, J.stamp, V, J.piece, L, start, deg,
                                 src, o, q, 0);
      else
        wgm_ls_chunk<SSSP, WGM_BATCH_PRECHECK || SSSP, PACK, WGM_BATCH_LS_K>(
            J.row, J.col, J.wt, dw, J.stamp, V, J.piece, L, start, deg, src, o);
    }
    if (ASYNC)
      wgm_ls_local_rounds<SSSP>(J.row, J.col, J.wt, J.dist, J.stamp, V, J.piece, L, o, q,
                                J.lq_rounds);
    if (step == 3) ns.ep++;
    n = wgm_team_level_barrier(err, spin_ns, o.counter64, G);
    if (n < 0) return -1;
    L++;
  }
  /* every member left at the same level, after a barrier that followed the
   * last relaxation: the words are final, each member copies its share */
  if (PACK)
    for (int i = tid; i < V; i += nth) J.dist[i] = dw[2 * i + 1];
  wgm_batch_add_work(J.arr, walked);
  return L;
}

/* One batch job on a team of G > 1 CTAs; this CTA is member `rank`. */
template <bool SSSP, bool ASYNC, bool DEFER = false>
__device__ void wgm_team_lonestar(const wgm_batch_args &B, const wgm_batch_job &j, int job,
                                  int rank, wgm_warp_smem *sm, wgm_lq *q) {
  wgm_ls_job J;
  J.delta = j.delta;
  J.far_cap = j.far_cap;
  J.light = j.light;
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
  J.stamp = B.stamp + j.stamp_off;
  J.wl_start = B.scratch + j.wl_off;
  J.wl_cnt = J.wl_start + 2 * (size_t)j.cap;
  J.wl_u = J.wl_cnt + 2 * (size_t)j.cap;
  int *ctl = B.ctl + (size_t)(1 + job * WGM_BATCH_CTL_LINES_PER_JOB) * WGM_LINE;
  J.cnt = ctl;
  J.arr = ctl + 3 * WGM_LINE;
  J.lq_rounds = B.lq_rounds;
  const int L = wgm_team_ls_run<SSSP, ASYNC, DEFER>(J, sm, B.err, B.spin_ns, q);
  if (L > 0 && rank == 0 && threadIdx.x == 0 && B.levels) B.levels[job] = L;
}

#endif
