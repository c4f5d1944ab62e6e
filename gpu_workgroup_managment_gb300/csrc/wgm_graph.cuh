/*
 * Persistent graph kernels for sm_103a: Lonestar BFS/SSSP worklists and
 * Pannotia colour/MIS/SSSP frontier loops, plus pull PageRank, all running in
 * one discovery-sized persistent grid synchronised by wgm_barrier.
 *
 * Reference kernels and what changed (outputs are bit-identical; each change
 * is argued where it is made):
 *   lonestar/graph_apps/bfs/device/bfs.cl:104-302   -> wgm_app_lonestar<false>
 *   lonestar/graph_apps/sssp/device/sssp.cl:104-318 -> wgm_app_lonestar<true>
 *   pannotia/graph_apps/color/device/color.cl:3-97  -> wgm_app_color
 *   pannotia/graph_apps/mis/device/mis.cl:5-125     -> wgm_app_mis
 *   pannotia/graph_apps/sssp/device/sssp.cl:10-88   -> wgm_app_pannotia_sssp
 *   (no reference)                                  -> wgm_app_pagerank
 *
 * Edge work is warp-level.  A warp owns up to 32 vertices (one per lane),
 * scans their degrees with shuffles and walks the concatenated adjacency in
 * windows of 32 edges: lane j of a window handles edge slot w+j, its owner is
 * found with one __reduce_or_sync and a clz, so col[] is read coalesced and no
 * CTA-wide __syncthreads is needed inside the edge loop (the reference's
 * block scan is serial in work-item 0, bfs.cl:43-51).  Vertices whose degree
 * exceeds `hub_threshold` ("hubs") skip the warp path; their edges are spread
 * over every warp of the grid so one hub never stalls a level.
 */
#ifndef WGM_GRAPH_CUH
#define WGM_GRAPH_CUH

#include "wgm_device.cuh"

#define WGM_LONESTAR_INF 1000000000u /* bfs.cl:33 */
#define WGM_PANNOTIA_BIG 99999999    /* pannotia sssp.h:3, mis.cl:1 */
#define WGM_MAX_WARPS 32

/* Per-CTA shared scratch of the edge-window walker. */
struct wgm_warp_smem {
  int tab[WGM_MAX_WARPS][32];
  int acc[WGM_MAX_WARPS][32];
};

/* Walk the edge slots [w0, total) of a warp's concatenated adjacency in
 * windows of 32, window stride `wstep`.  Each lane passes its own range as
 * (off = exclusive prefix, deg, base = row start - off).  f(valid, edge,
 * owner_lane) is called by all 32 lanes once per window. */
template <class F>
__device__ __forceinline__ void wgm_for_each_edge(int off, int deg, int base, int total,
                                                  int w0, int wstep, int *tab, F &&f) {
  const int lane = wgm_lane();
  for (int w = w0; w < total; w += wstep) {
    bool in = deg > 0 && off < w + 32 && off + deg > w;
    int pos = in ? max(off - w, 0) : 0;
    unsigned mask = __reduce_or_sync(WGM_FULL, in ? (1u << pos) : 0u);
    if (in) tab[pos] = lane;
    __syncwarp();
    unsigned upto = (lane == 31) ? 0xffffffffu : ((2u << lane) - 1u);
    unsigned mm = mask & upto;
    int owner = tab[mm ? 31 - __clz(mm) : 0] & 31;
    __syncwarp();
    int eb = __shfl_sync(WGM_FULL, base, owner);
    int slot = w + lane;
    f(slot < total, eb + slot, owner);
  }
}

/* Static hub layout (host-built): hub ids, their edge prefix and, for each
 * window of 32 hub-edge slots, a 16-byte record {first hub h0, edge of the
 * window's first slot, slots belonging to h0, first edge of hub h0+1}.  Hubs
 * have degree > 32, so a window touches at most two consecutive hubs, and
 * one load of the record gives every lane its hub and edge. */
struct wgm_hubs {
  const int *ids;    /* [H] */
  const int *prefix; /* [H+1] */
  const int *wmap;   /* [4 * ceil(prefix[H]/32)] window records */
  int H;
  int total;
};

/* Hub and edge of this lane's slot in window k. */
__device__ __forceinline__ void wgm_hub_slot(const int4 &w, int lane, int *h, int *e) {
  const bool first = lane < w.z;
  *h = first ? w.x : w.x + 1;
  *e = first ? w.y + lane : w.w + (lane - w.z);
}

/* Calls f(valid, hub_index, edge) for one window of hub edges. */
template <class F>
__device__ __forceinline__ void wgm_hub_window(const wgm_hubs &hb, const int *row, int k,
                                               F &&f) {
  const int lane = wgm_lane();
  const bool valid = k * 32 + lane < hb.total;
  const int4 w = __ldg(reinterpret_cast<const int4 *>(hb.wmap) + k);
  int h, e;
  wgm_hub_slot(w, lane, &h, &e);
  (void)row;
  f(valid, h, e);
}

/* Reduce `v` over the lanes holding hub h0 and hub h0+1 separately; lane 0
 * receives both results.  op: 0 = max (int bits), 1 = min (int bits), 2 = fp32 sum. */
__device__ __forceinline__ void wgm_two_seg_reduce(bool first, int v, float fv, int op,
                                                   int *r0, int *r1, float *f0,
                                                   float *f1) {
  int a = first ? v : (op == 0 ? INT_MIN : INT_MAX);
  int b = first ? (op == 0 ? INT_MIN : INT_MAX) : v;
  float fa = first ? fv : 0.f, fb = first ? 0.f : fv;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    int ya = __shfl_xor_sync(WGM_FULL, a, o), yb = __shfl_xor_sync(WGM_FULL, b, o);
    float ga = __shfl_xor_sync(WGM_FULL, fa, o), gb = __shfl_xor_sync(WGM_FULL, fb, o);
    if (op == 0) {
      a = max(a, ya);
      b = max(b, yb);
    } else if (op == 1) {
      a = min(a, ya);
      b = min(b, yb);
    }
    fa += ga;
    fb += gb;
  }
  *r0 = a;
  *r1 = b;
  *f0 = fa;
  *f1 = fb;
}

/* ------------------------------------------------------------------------ */
/* Lonestar BFS / SSSP                                                       */
/* ------------------------------------------------------------------------ */

struct wgm_lonestar_args {
  int V;
  const int *row; /* [V+1]; row[V] may be row[V-1]-1 (Lonestar loader quirk) */
  const int *col;
  const unsigned *wt; /* SSSP weights, nullptr for BFS */
  unsigned *dist;     /* [V] output */
  /* Two worklists of `cap` pieces each, structure of arrays: a piece is up
   * to `piece` consecutive edges of one vertex. */
  int *wl_start; /* [2][cap] first edge of the piece */
  int *wl_cnt;   /* [2][cap] number of edges */
  int *wl_u;     /* [2][cap] the vertex (SSSP reads its distance); may be null for BFS */
  int cap;       /* >= V + E/piece, so no level can overflow */
  int piece;     /* edges per piece (>= 32) */
  int *cnt;      /* [3 lines]: pieces queued for each level, by level mod 3 */
  int *stamp;    /* SSSP: level a vertex was last queued at, or (packed) [2V] the
                    64-bit {level tag, distance} words, dist[] written at the end */
  int source;
  int *levels_out; /* number of levels run (written by group 0) */
  int packed = 0;  /* SSSP relaxes packed words (wgm_ls_chunk PACK) */
};

/* Degree as the Lonestar kernel sees it: psrc[nn+1]-psrc[nn] (bfs.cl:165);
 * the loader quirk can make the last vertex -1, which walks no edges. */
__device__ __forceinline__ int wgm_ls_degree(const int *row, int v) {
  return max(__ldg(&row[v + 1]) - __ldg(&row[v]), 0);
}

/* Relaxation rules of one edge from a vertex at distance dsrc, at level L
 * (applied by wgm_ls_chunk):
 * BFS (bfs.cl:115-125): dist[dst]==MYINFINITY -> dist[dst]=level; the
 *   reference's unsynchronised store becomes a CAS so each vertex is queued
 *   exactly once (the stored value is identical: the level).
 * SSSP (sssp.cl:115-131): altdist = dist[src]+wt; if smaller, atomic_min and
 *   queue dst; a per-level stamp queues a vertex at most once per level (its
 *   next visit reads the final dist of the level, so the fixpoint - the
 *   shortest-path vector - is unchanged).
 * Destinations outside [0, V) and weights >= MYINFINITY are skipped
 * (bfs.cl:116, sssp.cl:120). */

/* Queue the flagged lanes' vertices as pieces (warp-aggregated: one atomic
 * per warp, __ballot_sync/__popc/__shfl_sync inside the scan and window
 * walk).  A vertex with no out-edges is not queued: its level or distance is
 * already written and it has nothing to relax.  Pieces are written by the
 * whole warp, one piece per lane per window, so the stores are coalesced. */
__device__ __forceinline__ bool wgm_ls_push(const wgm_lonestar_args &a, bool flag, int u,
                                            int *counter, int *o_start, int *o_cnt, int *o_u,
                                            int *tab) {
  int start = 0, deg = 0, np = 0;
  if (flag) {
    start = __ldg(&a.row[u]);
    deg = wgm_ls_degree(a.row, u);
    np = (deg + a.piece - 1) / a.piece;
  }
  int incl = wgm_warp_incl_scan(np);
  int total = __shfl_sync(WGM_FULL, incl, 31);
  if (total == 0) return true;
  int base = 0;
  if (wgm_lane() == 0) base = atomicAdd(counter, total);
  base = __shfl_sync(WGM_FULL, base, 0);
  if (base + total > a.cap) return false;
  int off = incl - np;
  const int P = a.piece;
  wgm_for_each_edge(off, np, -off, total, 0, 32, tab, [&](bool valid, int k, int owner) {
    /* k: piece index of `owner`'s vertex; slot = its position in the list */
    int s = __shfl_sync(WGM_FULL, start, owner);
    int d = __shfl_sync(WGM_FULL, deg, owner);
    int v = __shfl_sync(WGM_FULL, u, owner);
    int o = __shfl_sync(WGM_FULL, off, owner);
    if (valid) {
      int slot = base + o + k;
      o_start[slot] = s + k * P;
      o_cnt[slot] = min(P, d - k * P);
      if (o_u) o_u[slot] = v;
    }
  });
  return true;
}

/* Owner lane of edge slot s in a warp's concatenated ranges: the last lane
 * whose exclusive offset is <= s, by binary search over shuffles.  A lane with
 * no edges shares its successor's offset, so the search always lands on the
 * lane whose range [off, off+deg) holds s (for 0 <= s < total). */
__device__ __forceinline__ int wgm_owner_of(int off, int s) {
  int j = 0;
#pragma unroll
  for (int step = 16; step > 0; step >>= 1) {
    int o = __shfl_sync(WGM_FULL, off, j + step);
    if (o <= s) j += step;
  }
  return j;
}

/* Worklist a chunk pushes to.  The piece count lives in `counter`, or,
 * when `counter64` is set, in the low half of a 64-bit level word whose
 * high half counts a team's barrier arrivals.  With `far_cnt` set (packed
 * SSSP, near-far schedule) an improved vertex whose new distance is at or
 * above `T` goes to the far list as a vertex id instead of the next level
 * as pieces; `far_min` keeps the least distance stored there. */
struct wgm_ls_out {
  int *counter; /* pieces queued so far (global or shared memory) */
  unsigned long long *counter64 = nullptr;
  int *o_start, *o_cnt, *o_u;
  int cap;
  int *far_cnt = nullptr;
  unsigned *far_min = nullptr;
  int *far_list = nullptr;
  int far_cap = 0;
  unsigned T = 0xffffffffu;
  /* SSSP: relax only edges of weight in [wlo, whi) (batched near-far with
   * heavy edges deferred; the defaults relax every edge) */
  unsigned wlo = 0, whi = 0xffffffffu;
};

/* Store one piece at list slot `slot`. */
__device__ __forceinline__ void wgm_out_put(const wgm_ls_out &o, int slot, int start, int cnt,
                                            int u) {
  o.o_start[slot] = start;
  o.o_cnt[slot] = cnt;
  if (o.o_u) o.o_u[slot] = u;
}

/* Reserve n slots of the output list; returns the first. */
__device__ __forceinline__ int wgm_out_reserve(const wgm_ls_out &o, int n) {
  if (o.counter64) return (int)(unsigned)atomicAdd(o.counter64, (unsigned long long)n);
  return atomicAdd(o.counter, n);
}

/* Queue the flagged lanes' vertices (with out-edges) as pieces of size P
 * (warp-collective; each lane writes its own pieces).  False when the list
 * is full. */
__device__ __forceinline__ bool wgm_out_push_vertices(const int *row, int P, bool flag, int u,
                                                      const wgm_ls_out &o) {
  int rs = 0, dg = 0, np = 0;
  if (flag) {
    rs = __ldg(&row[u]);
    dg = max(__ldg(&row[u + 1]) - rs, 0);
    np = (dg + P - 1) / P;
  }
  const int incl = wgm_warp_incl_scan(np);
  const int total = __shfl_sync(WGM_FULL, incl, 31);
  if (total == 0) return true;
  int base = 0;
  if (wgm_lane() == 31) base = wgm_out_reserve(o, total);
  base = __shfl_sync(WGM_FULL, base, 31);
  if (base + total > o.cap) return false;
  const int s = base + incl - np;
  for (int q = 0; q < np; q++) wgm_out_put(o, s + q, rs + q * P, min(P, dg - q * P), u);
  return true;
}

/* Edges per lane per batch of the chunk walker (its default; callers may
 * pick another): a warp relaxes 32*K edges with every memory step of the K
 * windows issued together, so K chains of loads and atomics are in flight
 * per lane instead of one. */
#ifndef WGM_LS_K
#define WGM_LS_K 4
#endif
/* A pushed vertex with more pieces than this is written by the whole warp. */
#define WGM_LS_LANE_PIECES 4

/* Relax the edges of one chunk (one piece per lane: first edge `start`,
 * `deg` edges, source distance `dv` for SSSP) and queue the improved
 * vertices as pieces of the next level.  Per batch of 32*K edges:
 *   col/wt loads -> dist pre-check -> atomic (CAS for BFS, min for SSSP)
 *   with row[u], row[u+1] fetched beside it -> SSSP stamp exchange ->
 *   one warp scan and one counter atomic for every piece of the batch.
 * The relaxation rules are stated above wgm_ls_push; the order of
 * relaxations inside a level does not change the fixpoint. */
/* PACK (SSSP only): `dist` points at 64-bit words {low: level tag, high:
 * distance} instead of a dist[] / stamp[] pair.  One 64-bit atomicMin of
 * (alt << 32 | L) then both relaxes and deduplicates: it lowered the
 * distance iff the old high half exceeds alt, and a lowering whose old tag
 * is already L found the vertex queued for L+1 by another lane this level
 * (its tag was set by that earlier lowering).  That is the stamp exchange's
 * rule without its dependent round trip; distances read the high halves. */
/* Pieces of a vertex with d edges: ceil(d / P), by a shift when P is a
 * power of two (lg = log2 P; -1 otherwise).  P is uniform across the warp,
 * so the branch is too. */
__device__ __forceinline__ int wgm_pieces(int d, int P, int lg) {
  return lg >= 0 ? (d + P - 1) >> lg : (d + P - 1) / P;
}
__device__ __forceinline__ int wgm_piece_log2(int P) { return (P & (P - 1)) ? -1 : __ffs(P) - 1; }

/* The tail of a relaxation batch, shared by the walkers: lane k-slot holds
 * a destination u[k] whose relaxation succeeded (f[k]), its row start rs[k]
 * and row end d[k] (read beside the atomic), and (SSSP) its new distance
 * alt[k].  Unpacked SSSP exchanges the level stamp (one queueing per level);
 * a vertex without edges is not queued; near-far parks a vertex at or above
 * the threshold in the far list; the rest are queued as pieces with one
 * warp scan and one counter reservation for the whole batch. */
template <int K, bool SSSP, bool PACK>
__device__ __forceinline__ bool wgm_ls_push_batch(const int *row, int *stamp, int P, int lg,
                                                  int L, int (&u)[K], int (&rs)[K], int (&d)[K],
                                                  const unsigned (&alt)[K], bool (&f)[K],
                                                  const wgm_ls_out &o) {
  const int lane = wgm_lane();
  bool ok = true;
  int np[K];
  int mine = 0, fmine = 0;
  bool fr[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    if (SSSP && !PACK && f[k]) f[k] = atomicExch(&stamp[u[k]], L) != L;
    d[k] = f[k] ? max(d[k] - rs[k], 0) : 0; /* a vertex without edges is not queued */
    /* near-far: a distance at or above the threshold waits in the far list */
    fr[k] = PACK && d[k] > 0 && alt[k] >= o.T;
    if (fr[k]) d[k] = 0;
    fmine += fr[k] ? 1 : 0;
    np[k] = wgm_pieces(d[k], P, lg);
    mine += np[k];
  }
  const int pincl = wgm_warp_incl_scan(mine);
  const int ptotal = __shfl_sync(WGM_FULL, pincl, 31);
  int fincl = 0, ftotal = 0;
  if (PACK && __any_sync(WGM_FULL, fmine != 0)) {
    fincl = wgm_warp_incl_scan(fmine);
    ftotal = __shfl_sync(WGM_FULL, fincl, 31);
  }
  if (ptotal == 0 && ftotal == 0) return true;
  /* the piece and far reservations go out together */
  int pbase = 0, fbase = 0;
  if (lane == 31) {
    if (ptotal) pbase = wgm_out_reserve(o, ptotal);
    if (PACK && ftotal) fbase = atomicAdd(o.far_cnt, ftotal);
  }
  pbase = __shfl_sync(WGM_FULL, pbase, 31);
  if (PACK && ftotal) {
    fbase = __shfl_sync(WGM_FULL, fbase, 31);
    int fs = fbase + fincl - fmine;
    unsigned m = 0xffffffffu;
    bool spill[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      spill[k] = false;
      if (fr[k]) {
        if (fs < o.far_cap) {
          o.far_list[fs] = u[k];
          m = min(m, alt[k]);
        } else {
          spill[k] = true; /* far list full: relax it now instead */
        }
        fs++;
      }
    }
#pragma unroll
    for (int x = 16; x > 0; x >>= 1) m = min(m, __shfl_xor_sync(WGM_FULL, m, x));
    if (lane == 0 && m != 0xffffffffu) atomicMin(o.far_min, m);
#pragma unroll
    for (int k = 0; k < K; k++)
      if (__any_sync(WGM_FULL, spill[k]))
        ok &= wgm_out_push_vertices(row, P, spill[k], u[k], o);
  }
  if (ptotal == 0) return ok;
  if (pbase + ptotal > o.cap) return false;
  int slot = pbase + pincl - mine;
  int sl[K];
  bool big = false;
#pragma unroll
  for (int k = 0; k < K; k++) {
    sl[k] = slot;
    if (np[k] <= WGM_LS_LANE_PIECES)
      for (int q = 0; q < np[k]; q++)
        wgm_out_put(o, slot + q, rs[k] + q * P, min(P, d[k] - q * P), u[k]);
    else
      big = true;
    slot += np[k];
  }
  /* high-degree vertices: the whole warp writes their pieces */
  if (__any_sync(WGM_FULL, big)) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      unsigned bb = __ballot_sync(WGM_FULL, np[k] > WGM_LS_LANE_PIECES);
      while (bb) {
        const int j = __ffs(bb) - 1;
        bb &= bb - 1;
        const int bs = __shfl_sync(WGM_FULL, rs[k], j), bd = __shfl_sync(WGM_FULL, d[k], j);
        const int bu = __shfl_sync(WGM_FULL, u[k], j), bsl = __shfl_sync(WGM_FULL, sl[k], j);
        const int bn = wgm_pieces(bd, P, lg);
        for (int q = lane; q < bn; q += 32)
          wgm_out_put(o, bsl + q, bs + q * P, min(P, bd - q * P), bu);
      }
    }
  }
  return ok;
}

/* Relax the edges of one chunk (one piece per lane: first edge `start`,
 * `deg` edges, source distance `dv` for SSSP) and queue the improved
 * vertices as pieces of the next level.  Per batch of 32*K edges:
 *   col/wt loads -> dist pre-check -> atomic (CAS for BFS, min for SSSP)
 *   with row[u], row[u+1] fetched beside it -> SSSP stamp exchange ->
 *   one warp scan and one counter atomic for every piece of the batch.
 * The relaxation rules are stated above wgm_ls_push; the order of
 * relaxations inside a level does not change the fixpoint. */
/* PACK (SSSP only): `dist` points at 64-bit words {low: level tag, high:
 * distance} instead of a dist[] / stamp[] pair.  One 64-bit atomicMin of
 * (alt << 32 | L) then both relaxes and deduplicates: it lowered the
 * distance iff the old high half exceeds alt, and a lowering whose old tag
 * is already L found the vertex queued for L+1 by another lane this level
 * (its tag was set by that earlier lowering).  That is the stamp exchange's
 * rule without its dependent round trip; distances read the high halves. */
template <bool SSSP, bool PRE = true, bool PACK = false, int K = WGM_LS_K>
__device__ __forceinline__ bool wgm_ls_chunk(const int *row, const int *col, const unsigned *wt,
                                             unsigned *dist, int *stamp, int V, int P, int L,
                                             int start, int deg, int src,
                                             const wgm_ls_out &o) {
  static_assert(SSSP || !PACK, "the packed word carries SSSP distances");
  constexpr int DS = PACK ? 2 : 1, DH = PACK ? 1 : 0; /* distance word of v: DS*v+DH */
  const int lane = wgm_lane();
  const int lg = wgm_piece_log2(P);
  const int incl = wgm_warp_incl_scan(deg);
  const int total = __shfl_sync(WGM_FULL, incl, 31);
  const int off = incl - deg;
  const int base = start - off;
  bool ok = true;
  for (int w = 0; w < total; w += 32 * K) {
    int e[K], u[K], rs[K], d[K], sv[K];
    unsigned alt[K];
    bool f[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const int s = w + 32 * k + lane;
      f[k] = s < total;
      const int own = wgm_owner_of(off, min(s, total - 1));
      e[k] = __shfl_sync(WGM_FULL, base, own) + s;
      sv[k] = SSSP ? __shfl_sync(WGM_FULL, src, own) : 0;
    }
    /* the piece vertex's distance is read beside the edge's col and weight
     * (the lanes of one piece read the same word), not before them */
#pragma unroll
    for (int k = 0; k < K; k++) {
      u[k] = f[k] ? __ldg(&col[e[k]]) : -1;
      alt[k] = 0;
      if (SSSP) {
        unsigned wk = f[k] ? __ldg(&wt[e[k]]) : WGM_LONESTAR_INF;
        unsigned dvk = f[k] ? __ldcg(&dist[DS * sv[k] + DH]) : 0u;
        f[k] = f[k] && wk < WGM_LONESTAR_INF /* sssp.cl:120 */ && wk >= o.wlo && wk < o.whi;
        alt[k] = dvk + wk;
      }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      f[k] = f[k] && (unsigned)u[k] < (unsigned)V; /* bfs.cl:116 */
      if (PRE && f[k]) {
        unsigned cur = __ldcg(&dist[DS * u[k] + DH]);
        f[k] = SSSP ? (alt[k] < cur) : (cur == WGM_LONESTAR_INF);
      }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      rs[k] = 0;
      d[k] = 0;
      if (f[k]) {
        if (PACK) {
          const unsigned long long old =
              atomicMin(reinterpret_cast<unsigned long long *>(dist) + u[k],
                        ((unsigned long long)alt[k] << 32) | (unsigned)L);
          f[k] = (unsigned)(old >> 32) > alt[k] && (unsigned)old != (unsigned)L;
        } else if (SSSP)
          f[k] = alt[k] < atomicMin(&dist[u[k]], alt[k]);
        else
          f[k] = atomicCAS(&dist[u[k]], WGM_LONESTAR_INF, (unsigned)L) == WGM_LONESTAR_INF;
        rs[k] = __ldg(&row[u[k]]);
        d[k] = __ldg(&row[u[k] + 1]);
      }
    }
    ok &= wgm_ls_push_batch<K, SSSP, PACK>(row, stamp, P, lg, L, u, rs, d, alt, f, o);
  }
  return ok;
}

/* One level: every warp takes 32 consecutive pieces of the input list (one
 * per lane) and walks their edges with wgm_ls_chunk; a piece holds at most
 * `piece` edges, so no warp ever holds more than 32*piece edges of a level. */
template <bool SSSP>
__device__ __forceinline__ bool wgm_ls_level(const wgm_launch &Lc, wgm_cta *c,
                                             const wgm_lonestar_args &a, int L,
                                             wgm_warp_smem *sm) {
  const int lane = wgm_lane(), warp = threadIdx.x >> 5;
  const int nwarps_cta = blockDim.x >> 5;
  const int gw = c->id * nwarps_cta + warp, NW = c->ngroups * nwarps_cta;
  const int n = __ldcg(&a.cnt[(L % 3) * WGM_LINE]);
  const size_t in_off = (size_t)(L & 1) * a.cap, out_off = (size_t)((L + 1) & 1) * a.cap;
  const int *i_start = a.wl_start + in_off, *i_cnt = a.wl_cnt + in_off;
  const int *i_u = a.wl_u ? a.wl_u + in_off : nullptr;
  wgm_ls_out o;
  o.counter = &a.cnt[((L + 1) % 3) * WGM_LINE];
  o.o_start = a.wl_start + out_off;
  o.o_cnt = a.wl_cnt + out_off;
  o.o_u = a.wl_u ? a.wl_u + out_off : nullptr;
  o.cap = a.cap;
  bool ok = true;
  /* pieces per warp: 32, or fewer when the list is short, so a small
   * frontier spreads over every warp instead of queueing on a few */
  const int per = max(1, min(32, (n + NW - 1) / NW));
  for (int b = gw * per; b < n; b += NW * per) {
    int i = b + lane, deg = 0, start = 0, src = 0;
    if (lane < per && i < n) {
      start = __ldcg(&i_start[i]);
      deg = __ldcg(&i_cnt[i]);
      if (SSSP) src = __ldcg(&i_u[i]);
    }
    if (SSSP && a.packed)
      ok &= wgm_ls_chunk<SSSP, true, SSSP>(a.row, a.col, a.wt,
                                           reinterpret_cast<unsigned *>(a.stamp), a.stamp, a.V,
                                           a.piece, L, start, deg, src, o);
    else
      ok &= wgm_ls_chunk<SSSP>(a.row, a.col, a.wt, a.dist, a.stamp, a.V, a.piece, L, start, deg,
                               src, o);
  }
  (void)sm;
  return ok;
}

/* Lonestar BFS on one CTA (standalone runs of small graphs, bfs_mode 1).
 * A level of a high-diameter graph carries a few hundred vertices, and the
 * grid form pays a chain of dependent L2 round trips per level (counter,
 * worklist pieces, columns, the claiming CAS, the pushed rows, the barrier):
 * ~4 us on the 256x256 grid whether 1 or 152 CTAs run it.  Here the whole
 * traversal lives in one CTA: visited bits in shared memory, claimed with a
 * shared-memory atomicOr; the frontier in shared memory (vertices past its
 * capacity spill to global memory); level counters triple-buffered in shared
 * memory, so a level is one __syncthreads and two global round trips (row
 * pointers, then columns).  Same levels as the Lonestar kernel: the source
 * is level 0, a vertex first reached while level L runs gets L, out-of-range
 * columns are skipped (bfs.cl:116), the loader quirk's negative last degree
 * walks nothing, and the level count is the first level whose frontier
 * walks no edge (the grid form never queues a vertex without edges). */
struct wgm_bfs_cta_smem {
  unsigned *bits; /* [ceil(V/32)] visited */
  int *front;     /* [2][F] frontier buffers */
  int F;
};

__device__ __forceinline__ void wgm_bfs_cta(const wgm_lonestar_args &a, int *spill, int spill_cap,
                                            const wgm_bfs_cta_smem &S, int *s_cnt) {
  const int V = a.V, nw = (V + 31) >> 5;
  for (int i = threadIdx.x; i < nw; i += blockDim.x) S.bits[i] = 0u;
  for (int i = threadIdx.x; i < V; i += blockDim.x)
    a.dist[i] = (i == a.source) ? 0u : WGM_LONESTAR_INF;
  if (threadIdx.x == 0) {
    s_cnt[0] = 0;
    s_cnt[1] = 1;
    s_cnt[2] = 0;
    s_cnt[3] = 0; /* overflow */
    for (int k = 4; k < 7; k++) s_cnt[k] = 0; /* the level walked an edge, by L mod 3 */
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    S.bits[a.source >> 5] = 1u << (a.source & 31);
    S.front[S.F] = a.source; /* level 1 reads buffer 1 */
  }
  __syncthreads();
  int L = 1;
  for (;;) {
    const int n = s_cnt[L % 3];
    if (n == 0) break;
    if (L > V + 1) break;
    const int *in = S.front + (size_t)(L & 1) * S.F;
    int *out = S.front + (size_t)((L + 1) & 1) * S.F;
    const int *in_sp = spill + (size_t)(L & 1) * spill_cap;
    int *out_sp = spill + (size_t)((L + 1) & 1) * spill_cap;
    int *oc = &s_cnt[(L + 1) % 3];
    if (threadIdx.x == 0) {
      s_cnt[(L + 2) % 3] = 0;
      s_cnt[4 + (L + 2) % 3] = 0;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int v = i < S.F ? in[i] : __ldcg(&in_sp[i - S.F]);
      const int s = __ldg(&a.row[v]);
      const int e = s + max(__ldg(&a.row[v + 1]) - s, 0);
      if (e > s) s_cnt[4 + L % 3] = 1;
      for (int j = s; j < e; j++) {
        const int u = __ldg(&a.col[j]);
        if ((unsigned)u >= (unsigned)V) continue;
        const unsigned bit = 1u << (u & 31);
        if (S.bits[u >> 5] & bit) continue;
        if (atomicOr(&S.bits[u >> 5], bit) & bit) continue;
        a.dist[u] = (unsigned)L;
        const int k = atomicAdd(oc, 1);
        if (k < S.F)
          out[k] = u;
        else if (k - S.F < spill_cap)
          out_sp[k - S.F] = u;
        else
          s_cnt[3] = 1;
      }
    }
    __syncthreads();
    /* the grid form queues no vertex without edges (it has no pieces): a
     * level that walked no edge is where its frontier was empty */
    if (!s_cnt[4 + L % 3]) break;
    L++;
  }
  if (threadIdx.x == 0 && a.levels_out) *a.levels_out = L;
}

/* Persistent BFS/SSSP phases: (0) device-side init; (1,L) level L.  One
 * barrier per level (the reference uses two, bfs.cl:282,295): the piece
 * counters are triple-buffered by level, so the counter a level fills was
 * cleared two levels earlier and the swap/reset step needs no barrier. */
template <bool SSSP>
static __device__ int wgm_phase_lonestar(const wgm_launch &Lc, wgm_cta *c,
                                         const wgm_lonestar_args &a, wgm_warp_smem *sm,
                                         int target, int Lv, int *next_target, int *next_round) {
  const int V = a.V;
  if (target == 0) {
    const int tid = c->id * blockDim.x + threadIdx.x, nth = c->ngroups * blockDim.x;
    /* Host init of the plugin (bfs.h:250-262) done on the device. */
    for (int i = tid; i < V; i += nth) {
      if (SSSP && a.packed) {
        reinterpret_cast<unsigned long long *>(a.stamp)[i] =
            (i == a.source) ? 0ull : (unsigned long long)WGM_LONESTAR_INF << 32;
      } else {
        a.dist[i] = (i == a.source) ? 0u : WGM_LONESTAR_INF;
        if (SSSP) a.stamp[i] = 0;
      }
    }
    if (c->id == 0 && threadIdx.x < 32) {
      /* Level 1 processes the source (bfs.cl:235-241 seeds it at iteration 0). */
      if (threadIdx.x == 0)
        for (int k = 0; k < 3; k++) a.cnt[k * WGM_LINE] = 0;
      __syncwarp();
      wgm_ls_push(a, threadIdx.x == 0, a.source, &a.cnt[1 * WGM_LINE], a.wl_start + a.cap,
                  a.wl_cnt + a.cap, a.wl_u ? a.wl_u + a.cap : nullptr, sm->acc[0]);
    }
    *next_target = 1;
    *next_round = 1;
    return 1;
  }
  int n = __ldcg(&a.cnt[(Lv % 3) * WGM_LINE]);
  if (n == 0) {
    if (c->id == 0 && threadIdx.x == 0 && a.levels_out) *a.levels_out = Lv;
    if (SSSP && a.packed) { /* the distances out of the packed words */
      const int tid = c->id * blockDim.x + threadIdx.x, nth = c->ngroups * blockDim.x;
      const unsigned *w = reinterpret_cast<const unsigned *>(a.stamp);
      for (int i = tid; i < V; i += nth) a.dist[i] = __ldcg(&w[2 * i + 1]);
    }
    return 0;
  }
  if (n > a.cap) {
    wgm_fail(Lc, WGM_DEV_OVERFLOW, WGM_SITE_QUEUE, Lv);
    return 0;
  }
  if (Lv > V + 2) { /* Bellman-Ford bound; only a corrupt input gets here */
    wgm_fail(Lc, WGM_DEV_BAD_INPUT, WGM_SITE_QUEUE, Lv);
    return 0;
  }
  if (c->id == 0 && threadIdx.x == 0) a.cnt[((Lv + 2) % 3) * WGM_LINE] = 0;
  if (!wgm_ls_level<SSSP>(Lc, c, a, Lv, sm)) wgm_fail(Lc, WGM_DEV_OVERFLOW, WGM_SITE_QUEUE, Lv);
  *next_target = 1;
  *next_round = Lv + 1;
  return 1;
}

/* ------------------------------------------------------------------------ */
/* Pannotia colour                                                           */
/* ------------------------------------------------------------------------ */

struct wgm_color_args {
  int V;
  const int *row; /* [V+1] */
  const int *col;
  const int *trow; /* in-edges (the transpose; the graph itself when symmetric) */
  const int *tcol;
  const float *node_value;
  int *color;    /* [V] output: 1-based colours */
  int *stop;     /* unused (kept for the argument layout of older callers) */
  int *hub_acc;  /* unused */
  wgm_hubs hubs; /* static layout of out-degree > hub_threshold vertices */
  int hub_threshold;
  int *rounds_out;
  int *pending;  /* [V] larger out-neighbours not yet coloured */
  int *wl_start, *wl_cnt, *wl_u; /* [2][cap] frontier pieces of in-edges; wl_u holds
                                    the value bits of the piece's vertex */
  int cap, piece;
  int *cnt;      /* [3 lines] frontier sizes by round mod 3 */
  int2 *tcv;     /* [in-edges] {in-neighbour, its value bits}, filled at init */
};

/* Pannotia colour (color.cl:3-97) computed as the frontier recurrence it
 * implies.  In the reference a vertex v takes colour r in the first round r
 * in which no out-neighbour with a larger value is uncoloured at the start
 * of r (color.cl:66-83; a vertex coloured in round r still counts as
 * uncoloured during r).  Hence colour(v) = 1 + max colour of its larger
 * out-neighbours (1 if none), degree-1 vertices take colour 1 because they
 * skip their neighbours (color.cl:46), and the reference's round count is
 * the largest colour (its exit test, color.cl:85-87, first fails in the
 * round after the last vertex is coloured).  So: count each vertex's larger
 * out-neighbours once (`pending`), colour the vertices with none in round 1,
 * and in round r let every vertex coloured r decrement its smaller
 * in-neighbours; one that reaches zero takes colour r+1.  Same colours and
 * round count as the reference, each edge looked at twice in all instead of
 * once per round.
 * Phases: (0) init; (3,0) count larger out-neighbours; (4,0) round-1
 * frontier; (1,r) the vertices coloured r release their in-neighbours. */
/* tcv[e] = {in-neighbour w, a word about w} (one 8-byte load per edge).
 * pre(w, word, src, &tag) tests w without side effects and sets the word
 * its queue entry will carry; commit(w) claims it (true: queue it).  The
 * in-edge row bounds of every w that passes `pre` are loaded beside
 * `commit`'s atomic, not after it. */
template <class Pre, class Commit>
__device__ __forceinline__ bool wgm_frontier_chunk(const int *trow, const int2 *tcv, int P,
                                                   int start, int deg, unsigned sv,
                                                   const wgm_ls_out &o, Pre &&pre,
                                                   Commit &&commit) {
  constexpr int K = WGM_LS_K;
  const int lane = wgm_lane();
  const int incl = wgm_warp_incl_scan(deg);
  const int total = __shfl_sync(WGM_FULL, incl, 31);
  const int off = incl - deg;
  const int base = start - off;
  bool ok = true;
  for (int w = 0; w < total; w += 32 * K) {
    int u[K], rs[K], d[K], np[K], tg[K], wv[K];
    unsigned src[K];
    bool f[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const int s = w + 32 * k + lane;
      f[k] = s < total;
      const int own = wgm_owner_of(off, min(s, total - 1));
      const int e = __shfl_sync(WGM_FULL, base, own) + s;
      src[k] = __shfl_sync(WGM_FULL, sv, own);
      const int2 p = f[k] ? __ldg(&tcv[e]) : make_int2(-1, 0);
      u[k] = p.x;
      wv[k] = p.y;
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      tg[k] = 0;
      f[k] = f[k] && pre(u[k], wv[k], src[k], &tg[k]);
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      rs[k] = 0;
      d[k] = 0;
      if (f[k]) {
        rs[k] = __ldg(&trow[u[k]]);
        d[k] = __ldg(&trow[u[k] + 1]);
        f[k] = commit(u[k]);
      }
    }
    int mine = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
      d[k] = f[k] ? max(d[k] - rs[k], 0) : 0;
      np[k] = (d[k] + P - 1) / P;
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
        for (int q = 0; q < np[k]; q++) {
          o.o_start[slot + q] = rs[k] + q * P;
          o.o_cnt[slot + q] = min(P, d[k] - q * P);
          o.o_u[slot + q] = tg[k];
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
        const int bu = __shfl_sync(WGM_FULL, tg[k], j), bsl = __shfl_sync(WGM_FULL, sl[k], j);
        const int bn = (bd + P - 1) / P;
        for (int q = lane; q < bn; q += 32) {
          o.o_start[bsl + q] = bs + q * P;
          o.o_cnt[bsl + q] = min(P, bd - q * P);
          o.o_u[bsl + q] = bu;
        }
      }
    }
  }
  return ok;
}

/* Queue the in-edge pieces of the lanes' flagged vertices (one vertex per
 * lane, the whole warp writes); the entries carry `tag`. */
__device__ __forceinline__ bool wgm_frontier_push(const int *trow, int P, bool flag, int v,
                                                  int tag, const wgm_ls_out &o, int *tab) {
  int start = 0, deg = 0, np = 0;
  if (flag) {
    start = __ldg(&trow[v]);
    deg = max(__ldg(&trow[v + 1]) - start, 0);
    np = (deg + P - 1) / P;
  }
  int incl = wgm_warp_incl_scan(np);
  int total = __shfl_sync(WGM_FULL, incl, 31);
  if (total == 0) return true;
  int base = 0;
  if (wgm_lane() == 0) base = wgm_out_reserve(o, total);
  base = __shfl_sync(WGM_FULL, base, 0);
  if (base + total > o.cap) return false;
  int off = incl - np;
  wgm_for_each_edge(off, np, -off, total, 0, 32, tab, [&](bool valid, int k, int owner) {
    int s = __shfl_sync(WGM_FULL, start, owner);
    int d = __shfl_sync(WGM_FULL, deg, owner);
    int x = __shfl_sync(WGM_FULL, tag, owner);
    int oo = __shfl_sync(WGM_FULL, off, owner);
    if (valid) {
      int slot = base + oo + k;
      o.o_start[slot] = s + k * P;
      o.o_cnt[slot] = min(P, d - k * P);
      o.o_u[slot] = x;
    }
  });
  return true;
}

static __device__ int wgm_phase_color(const wgm_launch &Lc, wgm_cta *c, const wgm_color_args &a,
                                      wgm_warp_smem *sm, wgm_step cur, wgm_step *nxt) {
  const wgm_split s(c);
  const int V = a.V;
  const int lane = s.lane, warp = s.warp;
  if (cur.target == 0) {
    for (int i = s.tid; i < V; i += s.nth) {
      a.color[i] = -1; /* color.h:50 */
      a.pending[i] = 0;
    }
    /* every in-edge beside its neighbour's value: a release reads both at once */
    const int ET = __ldg(&a.trow[V]);
    for (int e = s.tid; e < ET; e += s.nth) {
      const int w = __ldg(&a.tcol[e]);
      a.tcv[e] = make_int2(w, __float_as_int(__ldg(&a.node_value[w])));
    }
    if (c->id == 0 && threadIdx.x < 3) a.cnt[threadIdx.x * WGM_LINE] = 0;
    *nxt = {3, 0};
    return WGM_PHASE_NEXT;
  }
  if (cur.target == 3) {
    /* larger out-neighbours of every vertex; a degree-1 vertex has none
     * (color.cl:46) */
    for (int b = s.gw * 32; b < V; b += s.NW * 32) {
      const int i = b + lane;
      int deg = 0, start = 0;
      float vi = 0.f;
      if (i < V) {
        start = __ldg(&a.row[i]);
        const int d = __ldg(&a.row[i + 1]) - start;
        deg = (d == 1 || d > a.hub_threshold) ? 0 : d;
        vi = __ldg(&a.node_value[i]);
      }
      sm->acc[warp][lane] = 0;
      int incl = wgm_warp_incl_scan(deg);
      int total = __shfl_sync(WGM_FULL, incl, 31);
      int off = incl - deg;
      __syncwarp();
      wgm_for_each_edge(off, deg, start - off, total, 0, 32, sm->tab[warp],
                        [&](bool valid, int e, int owner) {
                          const float vo = __shfl_sync(WGM_FULL, vi, owner);
                          if (valid && __ldg(&a.node_value[__ldg(&a.col[e])]) > vo)
                            atomicAdd(&sm->acc[warp][owner], 1);
                        });
      __syncwarp();
      if (i < V && deg > 0) a.pending[i] = sm->acc[warp][lane];
    }
    const int nwin = (a.hubs.total + 31) >> 5;
    for (int k = s.gw; k < nwin; k += s.NW) {
      wgm_hub_window(a.hubs, a.row, k, [&](bool valid, int h, int e) {
        int h0 = __shfl_sync(WGM_FULL, h, 0);
        int cntv = 0;
        if (valid) {
          const int v = __ldg(&a.hubs.ids[h]);
          cntv = __ldg(&a.node_value[__ldg(&a.col[e])]) > __ldg(&a.node_value[v]) ? 1 : 0;
        }
        int m0, m1;
        float f0, f1;
        wgm_two_seg_reduce(h == h0, 0, (float)cntv, 2, &m0, &m1, &f0, &f1);
        if (lane == 0) {
          if (f0 > 0.f) atomicAdd(&a.pending[__ldg(&a.hubs.ids[h0])], (int)f0);
          if (f1 > 0.f && h0 + 1 < a.hubs.H)
            atomicAdd(&a.pending[__ldg(&a.hubs.ids[h0 + 1])], (int)f1);
        }
      });
    }
    *nxt = {4, 0};
    return WGM_PHASE_NEXT;
  }
  wgm_ls_out o;
  o.cap = a.cap;
  if (cur.target == 4) {
    /* round 1: every vertex without a larger out-neighbour */
    o.counter = &a.cnt[1 * WGM_LINE];
    o.o_start = a.wl_start + a.cap;
    o.o_cnt = a.wl_cnt + a.cap;
    o.o_u = a.wl_u + a.cap;
    bool ok = true;
    for (int b = s.gw * 32; b < V; b += s.NW * 32) {
      const int i = b + lane;
      const bool f = i < V && __ldcg(&a.pending[i]) == 0;
      int tag = 0;
      if (f) {
        a.color[i] = 1;
        tag = __float_as_int(__ldg(&a.node_value[i]));
      }
      ok &= wgm_frontier_push(a.trow, a.piece, f, i, tag, o, sm->tab[warp]);
    }
    if (!ok) wgm_fail(Lc, WGM_DEV_OVERFLOW, WGM_SITE_QUEUE, 1);
    *nxt = {1, 1};
    return WGM_PHASE_NEXT;
  }
  const int r = cur.round;
  const int n = __ldcg(&a.cnt[(r % 3) * WGM_LINE]);
  if (n == 0) {
    if (c->id == 0 && threadIdx.x == 0 && a.rounds_out) *a.rounds_out = r - 1;
    return WGM_PHASE_DONE;
  }
  if (n > a.cap || r > V + 2) {
    wgm_fail(Lc, WGM_DEV_BAD_INPUT, WGM_SITE_QUEUE, r);
    return WGM_PHASE_DONE;
  }
  if (c->id == 0 && threadIdx.x == 0) a.cnt[((r + 2) % 3) * WGM_LINE] = 0;
  const size_t io = (size_t)(r & 1) * a.cap, oo = (size_t)((r + 1) & 1) * a.cap;
  o.counter = &a.cnt[((r + 1) % 3) * WGM_LINE];
  o.o_start = a.wl_start + oo;
  o.o_cnt = a.wl_cnt + oo;
  o.o_u = a.wl_u + oo;
  const int next_colour = r + 1;
  bool ok = true;
  /* pieces per warp: 32, or fewer when the frontier is short */
  const int per = max(1, min(32, (n + s.NW - 1) / s.NW));
  for (int b = s.gw * per; b < n; b += s.NW * per) {
    int i = b + lane, deg = 0, start = 0;
    unsigned sv = 0;
    if (lane < per && i < n) {
      start = __ldcg(&a.wl_start[io + i]);
      deg = __ldcg(&a.wl_cnt[io + i]);
      sv = (unsigned)__ldcg(&a.wl_u[io + i]); /* the coloured vertex's value bits */
    }
    ok &= wgm_frontier_chunk(
        a.trow, a.tcv, a.piece, start, deg, sv, o,
        [&](int w, int wbits, unsigned src, int *tag) {
          /* w has the coloured vertex as a larger out-neighbour */
          (void)w;
          *tag = wbits;
          return __int_as_float(wbits) < __uint_as_float(src);
        },
        [&](int w) {
          if (atomicSub(&a.pending[w], 1) != 1) return false;
          a.color[w] = next_colour;
          return true;
        });
  }
  if (!ok) wgm_fail(Lc, WGM_DEV_OVERFLOW, WGM_SITE_QUEUE, r);
  *nxt = {1, r + 1};
  return WGM_PHASE_NEXT;
}

/* ------------------------------------------------------------------------ */
/* Pannotia colour without rounds (standalone runs)                          */
/* ------------------------------------------------------------------------ */

/* colour(v) = 1 + the largest colour among v's larger out-neighbours (1 if
 * none; degree-1 vertices 1), the recurrence wgm_phase_color computes a
 * round at a time.  Nothing forces rounds: a vertex can take its colour the
 * moment its last larger out-neighbour has one.  So after the same counts
 * (wgm_phase_color's target 3) every warp works from a queue of release
 * pieces - up to 32 in-edges of a coloured vertex with its value and colour
 * - and, for every in-neighbour w smaller than it, raises cmax[w] to
 * colour + 1 and takes one off pending[w] with an acq_rel atomic; the lane
 * that takes the last one (it reads every raise of cmax[w], ordered before
 * the other decrements) colours w with cmax[w] and queues w's in-edges.  A
 * vertex of at most 32 in-edges goes to its warp's own stack in shared
 * memory and is released by that warp next; larger ones go to the global
 * queue in pieces.  Measured against the round form it loses: on RMAT-20
 * 16 ms against 8.3 ms (1629 colours, ~10 us per link of the longest chain
 * against ~5 us per round), because that chain runs through high-degree
 * vertices whose releases pass the global queue (a reservation, the piece
 * written and seen, its fields read) where a round spreads them over every
 * warp behind one barrier.  So rounds stay the default.  Degree-1 vertices start at
 * pending 0 (coloured 1) and releases only take them below 0, so they are
 * never coloured again - the reference's quirk (color.cl:46).  Colours are
 * the round-based form's, bit for bit; the run reports the largest colour
 * as its round count. */
#define WGM_CA_STACK 64
/* vertices of at most this many in-edges stay on their warp's stack;
 * larger ones go to the global queue in pieces.  Keeping up to 1024 on the
 * stack (32 edges a step) made RMAT-20 5x slower: the longest colour chains
 * run through high-degree vertices, whose releases must spread over many
 * warps at once. */
#define WGM_CA_LOCAL_MAX 32
struct wgm_color_async_args {
  int4 *tcv4;   /* [in-edges] {in-neighbour w, bits of w's value, w's first
                   in-edge, w's in-degree} */
  int *cmax;    /* [V] 1 + the largest releaser colour so far */
  int *q_start, *q_cnt, *q_val, *q_col; /* [qcap] release pieces (q_cnt -1 until
                                           written, with release) */
  int qcap;
  int *ctl;     /* lines: 0 queue head, 1 tail, 2 pieces done, 3 pieces in all,
                   4 largest colour */
};
struct wgm_ca_stack { /* per warp, shared memory: pieces of one edge window */
  int start[WGM_CA_STACK], cnt[WGM_CA_STACK], val[WGM_CA_STACK], col[WGM_CA_STACK];
  int n;
};

/* Init (between barriers): colours, pending counts, cmax, the in-edge
 * records, the queue's ready words and the control lines. */
__device__ __forceinline__ void wgm_color_async_init(const wgm_cta *c, const wgm_color_args &a,
                                                     const wgm_color_async_args &q) {
  const wgm_split s(c);
  const int V = a.V;
  for (int i = s.tid; i < V; i += s.nth) {
    a.color[i] = -1;
    a.pending[i] = 0;
    q.cmax[i] = 0;
  }
  const int ET = __ldg(&a.trow[V]);
  for (int e = s.tid; e < ET; e += s.nth) {
    const int w = __ldg(&a.tcol[e]);
    const int t0 = __ldg(&a.trow[w]);
    q.tcv4[e] = make_int4(w, __float_as_int(__ldg(&a.node_value[w])), t0,
                          __ldg(&a.trow[w + 1]) - t0);
  }
  for (int i = s.tid; i < q.qcap; i += s.nth) q.q_cnt[i] = -1;
  if (c->id == 0 && threadIdx.x < 5) q.ctl[threadIdx.x * WGM_LINE] = 0;
}

/* Queue the release pieces of the flagged lanes' vertices (vertex record
 * rec = tcv4-style {w, value bits, first in-edge, in-degree}, colour cw):
 * one-piece vertices onto the warp's stack while it has room, the rest onto
 * the global queue.  Warp-collective.  Returns false on a full queue. */
__device__ __forceinline__ bool wgm_ca_push(bool flag, int4 rec, int cw,
                                            const wgm_color_async_args &q, wgm_ca_stack *st) {
  const int lane = wgm_lane();
  const int deg = flag ? rec.w : 0;
  bool local = deg > 0 && deg <= WGM_CA_LOCAL_MAX;
  const unsigned lm = __ballot_sync(WGM_FULL, local);
  const int nloc = __popc(lm);
  int n0 = 0;
  if (lane == 0) n0 = st->n;
  n0 = __shfl_sync(WGM_FULL, n0, 0);
  if (n0 + nloc > WGM_CA_STACK) local = false;
  if (local) {
    const int k = n0 + __popc(lm & wgm_lanemask_lt());
    st->start[k] = rec.z;
    st->cnt[k] = deg;
    st->val[k] = rec.y;
    st->col[k] = cw;
  }
  __syncwarp();
  if (lane == 0 && n0 + nloc <= WGM_CA_STACK) st->n = n0 + nloc;
  __syncwarp();
  const int np = (deg > 0 && !local) ? (deg + 31) >> 5 : 0;
  const int incl = wgm_warp_incl_scan(np);
  const int total = __shfl_sync(WGM_FULL, incl, 31);
  if (total == 0) return true;
  int base = 0;
  if (lane == 31) base = atomicAdd(&q.ctl[1 * WGM_LINE], total);
  base = __shfl_sync(WGM_FULL, base, 31);
  if (base + total > q.qcap) return false;
  const int first = base + incl - np;
  /* a few pieces per lane, else the whole warp writes one vertex's pieces */
  if (np <= 4) {
    for (int k = 0; k < np; k++) {
      const int slot = first + k;
      q.q_start[slot] = rec.z + 32 * k;
      q.q_val[slot] = rec.y;
      q.q_col[slot] = cw;
      wgm_st_release_gpu(&q.q_cnt[slot], min(32, deg - 32 * k));
    }
  }
  unsigned big = __ballot_sync(WGM_FULL, np > 4);
  while (big) {
    const int j = __ffs(big) - 1;
    big &= big - 1;
    const int bz = __shfl_sync(WGM_FULL, rec.z, j), by = __shfl_sync(WGM_FULL, rec.y, j);
    const int bd = __shfl_sync(WGM_FULL, deg, j), bf = __shfl_sync(WGM_FULL, first, j);
    const int bc = __shfl_sync(WGM_FULL, cw, j);
    for (int k = lane; k < (bd + 31) >> 5; k += 32) {
      q.q_start[bf + k] = bz + 32 * k;
      q.q_val[bf + k] = by;
      q.q_col[bf + k] = bc;
      wgm_st_release_gpu(&q.q_cnt[bf + k], min(32, bd - 32 * k));
    }
  }
  return true;
}

/* Seeding (between barriers, after the counts): every vertex without a
 * larger out-neighbour takes colour 1 and is queued; the pieces of every
 * vertex's in-edges are counted (each vertex is coloured exactly once). */
__device__ __forceinline__ bool wgm_color_async_seed(const wgm_cta *c, const wgm_color_args &a,
                                                     const wgm_color_async_args &q,
                                                     wgm_ca_stack *st) {
  const wgm_split s(c);
  const int V = a.V, lane = s.lane;
  bool ok = true;
  int pieces = 0;
  for (int b = s.gw * 32; b < V; b += s.NW * 32) {
    const int i = b + lane;
    int4 rec = make_int4(0, 0, 0, 0);
    bool f = false;
    if (i < V) {
      const int t0 = __ldg(&a.trow[i]);
      rec = make_int4(i, __float_as_int(__ldg(&a.node_value[i])), t0, __ldg(&a.trow[i + 1]) - t0);
      pieces += (rec.w + 31) >> 5;
      f = __ldcg(&a.pending[i]) == 0;
      if (f) a.color[i] = 1;
    }
    /* seeds go to the global queue: any warp may take them */
    if (lane == 0) st->n = WGM_CA_STACK;
    __syncwarp();
    ok &= wgm_ca_push(f, rec, 1, q, st);
    __syncwarp();
  }
  if (lane == 0) st->n = 0;
  for (int o = 16; o > 0; o >>= 1) pieces += __shfl_xor_sync(WGM_FULL, pieces, o);
  if (lane == 0 && pieces) atomicAdd(&q.ctl[3 * WGM_LINE], pieces);
  if (lane == 0 && V > 0) atomicMax(&q.ctl[4 * WGM_LINE], 1);
  return ok;
}

/* The release loop (no barrier): returns false when a wait gave up or the
 * queue overflowed. */
__device__ __forceinline__ bool wgm_color_async_run(const wgm_launch &L, const wgm_color_args &a,
                                                    const wgm_color_async_args &q,
                                                    wgm_ca_stack *st) {
  const int lane = wgm_lane();
  const int T = __ldcg(&q.ctl[3 * WGM_LINE]);
  bool ok = true;
  int cmax_seen = 0;
  int mydone = 0; /* 32-edge steps released by this warp, not yet counted */
  for (;;) {
    int start = 0, cnt = 0, val = 0, col = 0, have = 0;
    if (lane == 0) {
      if (st->n > 0) {
        const int k = st->n - 1;
        start = st->start[k];
        cnt = st->cnt[k];
        val = st->val[k];
        col = st->col[k];
        have = 1;
        if (cnt > 32) { /* the rest of its in-edges stays on the stack */
          st->start[k] = start + 32;
          st->cnt[k] = cnt - 32;
          cnt = 32;
        } else {
          st->n = k;
        }
      } else {
        /* the steps this warp released count before it waits */
        if (mydone) wgm_red_add_release_gpu(&q.ctl[2 * WGM_LINE], mydone);
        mydone = 0;
        const int i = atomicAdd(&q.ctl[0], 1);
        if (i < T && i < q.qcap) {
          wgm_spin sp = wgm_spin_start(L);
          for (;;) {
            cnt = wgm_ld_acquire_gpu(&q.q_cnt[i]);
            if (cnt >= 0) {
              have = 1;
              break;
            }
            /* every piece was released elsewhere: slot i stays empty */
            if ((sp.n & 7u) == 7u && wgm_ld_relaxed_gpu(&q.ctl[2 * WGM_LINE]) >= T) break;
            if (wgm_spin_giveup(L, sp, WGM_SITE_QUEUE)) {
              ok = false;
              break;
            }
            /* a waiting warp polls gently: the releasing ones need the L2 */
            if (sp.n > 4) __nanosleep(100);
          }
          if (have) {
            start = __ldcg(&q.q_start[i]);
            val = __ldcg(&q.q_val[i]);
            col = __ldcg(&q.q_col[i]);
          }
        }
      }
    }
    have = __shfl_sync(WGM_FULL, have, 0);
    if (!have) break;
    start = __shfl_sync(WGM_FULL, start, 0);
    cnt = __shfl_sync(WGM_FULL, cnt, 0);
    val = __shfl_sync(WGM_FULL, val, 0);
    col = __shfl_sync(WGM_FULL, col, 0);
    bool ready = false;
    int4 rec = make_int4(0, 0, 0, 0);
    int cw = 0;
    if (lane < cnt) {
      rec = __ldcg(&q.tcv4[start + lane]); /* written by this launch's init */
      /* w has the released vertex as a larger out-neighbour */
      if (__int_as_float(rec.y) < __int_as_float(val)) {
        atomicMax(&q.cmax[rec.x], col + 1);
        ready = wgm_atom_add_acqrel_gpu(&a.pending[rec.x], -1) == 1;
        if (ready) {
          cw = __ldcg(&q.cmax[rec.x]);
          a.color[rec.x] = cw;
          cmax_seen = max(cmax_seen, cw);
        }
      }
    }
    ok &= wgm_ca_push(ready, rec, cw, q, st);
    mydone++;
  }
  if (lane == 0 && mydone) wgm_red_add_release_gpu(&q.ctl[2 * WGM_LINE], mydone);
  for (int o = 16; o > 0; o >>= 1) cmax_seen = max(cmax_seen, __shfl_xor_sync(WGM_FULL, cmax_seen, o));
  if (lane == 0 && cmax_seen) atomicMax(&q.ctl[4 * WGM_LINE], cmax_seen);
  return ok;
}

/* ------------------------------------------------------------------------ */
/* Pannotia MIS                                                              */
/* ------------------------------------------------------------------------ */

struct wgm_mis_args {
  int V;
  const int *row;
  const int *col;
  const float *node_value;
  int *s_array; /* [V] output: 2 = member, 0 = not */
  int *status;  /* [V]: -1 active, 2r removed in round r, 2r+1 joined in r */
  int *stop;    /* [3 lines] */
  int *hub_acc; /* [2][H] running min (float bits), by round parity */
  wgm_hubs hubs;
  int hub_threshold;
  int *rounds_out;
};

/* The reference's c_array/cu_array pair (mis.cl:73-118) becomes one status
 * word stamped with the round: a vertex is "active at the start of round r"
 * iff status == -1 or status>>1 == r, which is exactly what mis1/mis2 of round
 * r see in the reference (cu is only committed to c in mis3, after the
 * barrier).  That lets mis1+mis2+mis3 run between two barriers instead of
 * three; s_array, the only output the reference checks (mis.h:199-202), is
 * identical. */
__device__ __forceinline__ bool wgm_active_at(int st, int r) {
  return st == -1 || (st >> 1) == r;
}

/* Phases: (0) init; (1,r) mis1+mis2 for non-hub vertices and hub minima over
 * the grid; (2,r) mis2 for hubs.  (1,r) first applies the reference's exit
 * test to round r-1 (mis.cl:106-108). */
static __device__ int wgm_phase_mis(const wgm_launch &Lc, wgm_cta *c, const wgm_mis_args &a,
                                    wgm_warp_smem *sm, wgm_step cur, wgm_step *nxt) {
  const wgm_split s(c);
  const int V = a.V;
  const int BIG = __float_as_int((float)WGM_PANNOTIA_BIG);
  if (cur.target == 0) {
    for (int i = s.tid; i < V; i += s.nth) {
      a.s_array[i] = 0; /* mis.h:58-92 */
      a.status[i] = -1;
    }
    for (int h = s.tid; h < 2 * a.hubs.H; h += s.nth) a.hub_acc[h] = BIG;
    if (c->id == 0 && threadIdx.x == 0)
      for (int k = 0; k < 3; k++) a.stop[k * WGM_LINE] = 0;
    *nxt = {1, 1};
    return WGM_PHASE_NEXT;
  }
  const int r = cur.round;
  int *hacc = a.hub_acc + (size_t)(r & 1) * a.hubs.H;
  const int nwin = (a.hubs.total + 31) >> 5;
  if (cur.target == 2) {
    /* mis2 for hubs.  The join test is a pure function of the final hub
     * minimum and the round-start status (a joined hub reads 2r+1, still
     * "active at r"), so every warp re-derives it while marking neighbours
     * and one thread per hub records the join.  The other parity's minima
     * are reset here for the next round. */
    int *hnext = a.hub_acc + (size_t)((r + 1) & 1) * a.hubs.H;
    for (int h = s.tid; h < a.hubs.H; h += s.nth) {
      int v = __ldg(&a.hubs.ids[h]);
      if (__ldcg(&a.status[v]) == -1 &&
          __ldg(&a.node_value[v]) < __int_as_float(__ldcg(&hacc[h]))) {
        a.s_array[v] = 2;
        a.status[v] = 2 * r + 1;
      }
      hnext[h] = BIG;
    }
    for (int k = s.gw; k < nwin; k += s.NW) {
      wgm_hub_window(a.hubs, a.row, k, [&](bool valid, int h, int e) {
        if (!valid) return;
        int v = __ldg(&a.hubs.ids[h]);
        int stv = __ldcg(&a.status[v]);
        if (wgm_active_at(stv, r) && stv != 2 * r &&
            __ldg(&a.node_value[v]) < __int_as_float(__ldcg(&hacc[h]))) {
          int j = __ldg(&a.col[e]);
          if (wgm_active_at(__ldcg(&a.status[j]), r) && j != v) a.status[j] = 2 * r;
        }
      });
    }
    *nxt = {1, r + 1};
    return WGM_PHASE_NEXT;
  }
  if (r > 1 && __ldcg(&a.stop[((r - 1) % 3) * WGM_LINE]) == 0) {
    if (c->id == 0 && threadIdx.x == 0 && a.rounds_out) *a.rounds_out = r - 1;
    return WGM_PHASE_DONE;
  }
  if (r > V + 2) {
    wgm_fail(Lc, WGM_DEV_BAD_INPUT, WGM_SITE_QUEUE, r);
    return WGM_PHASE_DONE;
  }
  if (c->id == 0 && threadIdx.x == 0) a.stop[((r + 1) % 3) * WGM_LINE] = 0;
  bool any = false;
  const int lane = s.lane, warp = s.warp;
  for (int b = s.gw * 32; b < V; b += s.NW * 32) {
    int i = b + lane;
    int deg = 0, start = 0;
    bool act = false;
    if (i < V) {
      act = __ldcg(&a.status[i]) == -1; /* active: nothing else can stamp it yet */
      start = __ldg(&a.row[i]);
      int d = __ldg(&a.row[i + 1]) - start;
      if (act) any = true; /* mis.cl:33 */
      if (d > a.hub_threshold)
        act = false;
      else if (act)
        deg = d;
    }
    sm->acc[warp][lane] = BIG;
    int incl = wgm_warp_incl_scan(deg);
    int total = __shfl_sync(WGM_FULL, incl, 31);
    int off = incl - deg;
    __syncwarp();
    /* mis1: min over neighbours active at round start (mis.cl:44-51).  (A
     * four-window version of this walk measured slower here: 8.6 against
     * 6.9 ms on RMAT-22, the status gathers of idle windows cost more than
     * the latency they hide.) */
    wgm_for_each_edge(off, deg, start - off, total, 0, 32, sm->tab[warp],
                      [&](bool valid, int e, int owner) {
                        if (valid) {
                          int j = __ldg(&a.col[e]);
                          if (wgm_active_at(__ldcg(&a.status[j]), r))
                            atomicMin(&sm->acc[warp][owner],
                                      __float_as_int(__ldg(&a.node_value[j])));
                        }
                      });
    __syncwarp();
    /* mis2: join, then mark the neighbours removed (mis.cl:68-95). */
    bool join = act && __ldg(&a.node_value[i]) < __int_as_float(sm->acc[warp][lane]);
    if (join) {
      a.s_array[i] = 2;
      a.status[i] = 2 * r + 1;
    }
    int jdeg = join ? deg : 0;
    int jincl = wgm_warp_incl_scan(jdeg);
    int jtotal = __shfl_sync(WGM_FULL, jincl, 31);
    int joff = jincl - jdeg;
    wgm_for_each_edge(joff, jdeg, start - joff, jtotal, 0, 32, sm->tab[warp],
                      [&](bool valid, int e, int owner) {
                        if (valid) {
                          int j = __ldg(&a.col[e]);
                          if (wgm_active_at(__ldcg(&a.status[j]), r)) a.status[j] = 2 * r;
                        }
                      });
  }
  /* Hub minima across the grid (mis1 for hubs). */
  for (int k = s.gw; k < nwin; k += s.NW) {
    wgm_hub_window(a.hubs, a.row, k, [&](bool valid, int h, int e) {
      int h0 = __shfl_sync(WGM_FULL, h, 0);
      int val = INT_MAX;
      if (valid && wgm_active_at(__ldcg(&a.status[__ldg(&a.hubs.ids[h])]), r)) {
        int j = __ldg(&a.col[e]);
        if (wgm_active_at(__ldcg(&a.status[j]), r)) val = __float_as_int(__ldg(&a.node_value[j]));
      }
      int m0, m1;
      float f0, f1;
      wgm_two_seg_reduce(h == h0, val, 0.f, 1, &m0, &m1, &f0, &f1);
      if (lane == 0) {
        if (m0 != INT_MAX) atomicMin(&hacc[h0], m0);
        if (m1 != INT_MAX && h0 + 1 < a.hubs.H) atomicMin(&hacc[h0 + 1], m1);
      }
    });
  }
  if (__any_sync(WGM_FULL, any) && lane == 0) a.stop[(r % 3) * WGM_LINE] = 1;
  *nxt = (a.hubs.H > 0) ? wgm_step{2, r} : wgm_step{1, r + 1};
  return WGM_PHASE_NEXT;
}

/* ------------------------------------------------------------------------ */
/* Pannotia SSSP (pull min-plus)                                             */
/* ------------------------------------------------------------------------ */

struct wgm_psssp_args {
  int V;
  const int *row;
  const int *col;
  const int *data;
  int *x;    /* [V] output cost (sssp.h:168 reads x) */
  int *stop; /* [3 lines] */
  wgm_hubs hubs;
  int hub_threshold;
  int source;
  int *rounds_out;
};

/* sssp.cl's vector_assign / spmv_min_dot_plus / vector_diff (three barriers
 * per round) become one in-place relaxation pass per round:
 * x[v] = min(x[v], min_j data[j] + x[col[j]]).  The reference's Jacobi
 * iteration and this chaotic (in-place) iteration both stop at the fixpoint
 * of the min-plus system started from x = BIG_NUM except x[source] = 0, which
 * is unique (the shortest-path distances, BIG_NUM where unreachable), so the
 * returned vector is identical; only the round count can be smaller.
 * Phases: (0) init; (1,r) one relaxation pass (after the exit test of r-1). */
static __device__ int wgm_phase_pannotia_sssp(const wgm_launch &Lc, wgm_cta *c,
                                              const wgm_psssp_args &a, wgm_warp_smem *sm,
                                              wgm_step cur, wgm_step *nxt) {
  const wgm_split s(c);
  const int V = a.V;
  if (cur.target == 0) {
    for (int i = s.tid; i < V; i += s.nth) a.x[i] = (i == a.source) ? 0 : WGM_PANNOTIA_BIG;
    if (c->id == 0 && threadIdx.x == 0)
      for (int k = 0; k < 3; k++) a.stop[k * WGM_LINE] = 0;
    *nxt = {1, 1};
    return WGM_PHASE_NEXT;
  }
  const int r = cur.round;
  if (r > 1 && __ldcg(&a.stop[((r - 1) % 3) * WGM_LINE]) == 0) {
    if (c->id == 0 && threadIdx.x == 0 && a.rounds_out) *a.rounds_out = r - 1;
    return WGM_PHASE_DONE;
  }
  if (r > V + 2) {
    wgm_fail(Lc, WGM_DEV_BAD_INPUT, WGM_SITE_QUEUE, r);
    return WGM_PHASE_DONE;
  }
  if (c->id == 0 && threadIdx.x == 0) a.stop[((r + 1) % 3) * WGM_LINE] = 0;
  bool changed = false;
  const int lane = s.lane, warp = s.warp;
  for (int b = s.gw * 32; b < V; b += s.NW * 32) {
    int i = b + lane, deg = 0, start = 0;
    if (i < V) {
      start = __ldg(&a.row[i]);
      int d = __ldg(&a.row[i + 1]) - start;
      deg = d > a.hub_threshold ? 0 : d;
    }
    sm->acc[warp][lane] = INT_MAX;
    int incl = wgm_warp_incl_scan(deg);
    int total = __shfl_sync(WGM_FULL, incl, 31);
    int off = incl - deg;
    __syncwarp();
    /* four 32-edge windows per step: their col and weight loads, then their
     * x gathers, in flight together (a min is exact in any order) */
    const int ebase = start - off;
    for (int w = 0; w < total; w += 128) {
      int own[4], j[4], wt[4], xj[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int sl = w + 32 * q + lane;
        const int o = wgm_owner_of(off, min(sl, total - 1));
        own[q] = sl < total ? o : -1;
        const int e = __shfl_sync(WGM_FULL, ebase, o) + sl;
        j[q] = own[q] >= 0 ? __ldg(&a.col[e]) : 0;
        wt[q] = own[q] >= 0 ? __ldg(&a.data[e]) : 0;
      }
#pragma unroll
      for (int q = 0; q < 4; q++) xj[q] = own[q] >= 0 ? __ldcg(&a.x[j[q]]) : 0;
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (own[q] >= 0) atomicMin(&sm->acc[warp][own[q]], wt[q] + xj[q]);
    }
    __syncwarp();
    if (deg > 0) {
      int cand = sm->acc[warp][lane];
      if (cand < __ldcg(&a.x[i])) {
        atomicMin(&a.x[i], cand);
        changed = true;
      }
    }
  }
  /* hub edges: four windows per warp step, their records, col and weight
   * loads, and x gathers in flight together */
  const int nwin = (a.hubs.total + 31) >> 5;
  const int4 *wrec = reinterpret_cast<const int4 *>(a.hubs.wmap);
  for (int k0 = s.gw * 4; k0 < nwin; k0 += s.NW * 4) {
    int4 w[4];
    int hh[4], j[4], wt[4], xj[4];
    bool val[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int k = min(k0 + q, nwin - 1);
      w[q] = __ldg(wrec + k);
      val[q] = k0 + q < nwin && (k0 + q) * 32 + lane < a.hubs.total;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int e;
      wgm_hub_slot(w[q], lane, &hh[q], &e);
      j[q] = val[q] ? __ldg(&a.col[e]) : 0;
      wt[q] = val[q] ? __ldg(&a.data[e]) : 0;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) xj[q] = val[q] ? __ldcg(&a.x[j[q]]) : 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (k0 + q >= nwin) break; /* warp-uniform */
      const int h0 = w[q].x;
      int m0, m1;
      float f0, f1;
      wgm_two_seg_reduce(hh[q] == h0, val[q] ? wt[q] + xj[q] : INT_MAX, 0.f, 1, &m0, &m1,
                         &f0, &f1);
      if (lane == 0) {
        const int v0 = __ldg(&a.hubs.ids[h0]);
        if (m0 < __ldcg(&a.x[v0]) && atomicMin(&a.x[v0], m0) > m0) changed = true;
        if (h0 + 1 < a.hubs.H && m1 != INT_MAX) {
          const int v1 = __ldg(&a.hubs.ids[h0 + 1]);
          if (m1 < __ldcg(&a.x[v1]) && atomicMin(&a.x[v1], m1) > m1) changed = true;
        }
      }
    }
  }
  if (__any_sync(WGM_FULL, changed) && lane == 0) a.stop[(r % 3) * WGM_LINE] = 1;
  *nxt = {1, r + 1};
  return WGM_PHASE_NEXT;
}

/* ------------------------------------------------------------------------ */
/* Pull PageRank (FP32; no reference implementation)                          */
/* ------------------------------------------------------------------------ */

struct wgm_pr_args {
  int V;
  const int *row;
  const int *col;
  float *pr;       /* [V] output */
  float *contrib;  /* [2][V] pr/deg of the previous iteration */
  float *dang;     /* [3 lines] dangling mass by iteration */
  float *hub_sum;  /* [H] */
  wgm_hubs hubs;
  int hub_threshold;
  int iterations;
  float damping;
  float dang0;     /* initial dangling mass: (zero-degree vertices)/V */
};

/* First stage of a PageRank hub step: the records of windows k0..k0+3
 * (first hub of each in hx), this lane's hub in each (hh) and the col
 * value of its slot (u; -1 past the end). */
__device__ __forceinline__ void wgm_pr_hub_stage(const int4 *wrec, const int *col, int total,
                                                 int nwin, int k0, int lane, int *hx, int *hh,
                                                 int *u) {
  int4 w[4];
#pragma unroll
  for (int q = 0; q < 4; q++) w[q] = __ldg(wrec + min(k0 + q, nwin - 1));
#pragma unroll
  for (int q = 0; q < 4; q++) {
    int e;
    wgm_hub_slot(w[q], lane, &hh[q], &e);
    hx[q] = w[q].x;
    u[q] = (k0 + q < nwin && (k0 + q) * 32 + lane < total) ? __ldg(&col[e]) : -1;
  }
}

/* Hub sums of four windows of PageRank hub edges (values v, hub hh per
 * lane, first hub of each window hx), in groups of M consecutive windows.  A group's 32*M slots span at
 * most two hubs when every hub has at least 32*M edges (hub threshold >=
 * 32*M - 1): the group's first hub h0 and h0 + 1.  Each lane sums its M
 * values into those two, then one two-sum warp reduction and at most two
 * atomics serve the group.  Windows past the end hold zeros. */
template <int M>
__device__ __forceinline__ void wgm_pr_hub_sums(const int *hx, const int *hh, const float *v,
                                                int k0, int nwin, int H, float *hub_sum) {
#pragma unroll
  for (int g = 0; g < 4; g += M) {
    if (k0 + g >= nwin) break; /* warp-uniform */
    const int h0 = hx[g];
    float f0 = 0.f, f1 = 0.f;
#pragma unroll
    for (int q = g; q < g + M; q++) {
      if (hh[q] == h0) f0 += v[q];
      else f1 += v[q];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      f0 += __shfl_xor_sync(WGM_FULL, f0, o);
      f1 += __shfl_xor_sync(WGM_FULL, f1, o);
    }
    if (wgm_lane() == 0) {
      atomicAdd(&hub_sum[h0], f0);
      if (h0 + 1 < H && f1 != 0.f) atomicAdd(&hub_sum[h0 + 1], f1);
    }
  }
}

/* pr' = (1-d)/V + d*(sum_{u in N(v)} pr[u]/deg(u) + dangling/V).  Phases:
 * (0) init; (1,t) iteration t for non-hub vertices, hub sums accumulated over
 * the grid; (2,t) hub finalisation.  Per-vertex sums run in a fixed order (a
 * segmented warp scan per window), so only the dangling mass and hub sums
 * depend on atomic order. */
static __device__ int wgm_phase_pagerank(const wgm_launch &Lc, wgm_cta *c, const wgm_pr_args &a,
                                         wgm_warp_smem *sm, wgm_step cur, wgm_step *nxt) {
  const wgm_split s(c);
  const int V = a.V;
  const float d = a.damping;
  if (cur.target == 0) {
    for (int i = s.tid; i < V; i += s.nth) {
      int deg = __ldg(&a.row[i + 1]) - __ldg(&a.row[i]);
      float p = 1.0f / (float)V;
      a.pr[i] = p;
      a.contrib[i] = deg > 0 ? p / (float)deg : 0.f;
    }
    for (int h = s.tid; h < a.hubs.H; h += s.nth) a.hub_sum[h] = 0.f;
    if (c->id == 0 && threadIdx.x == 0) {
      a.dang[0] = a.dang0;
      a.dang[1 * WGM_LINE] = 0.f;
      a.dang[2 * WGM_LINE] = 0.f;
    }
    *nxt = {1, 0};
    return WGM_PHASE_NEXT;
  }
  const int t = cur.round;
  const float *cin = a.contrib + (size_t)(t & 1) * V;
  float *cout = a.contrib + (size_t)((t + 1) & 1) * V;
  const float base = (1.0f - d) / (float)V + d * __ldcg(&a.dang[(t % 3) * WGM_LINE]) / (float)V;
  if (cur.target == 2) {
    for (int h = s.tid; h < a.hubs.H; h += s.nth) {
      int v = __ldg(&a.hubs.ids[h]);
      int dg = __ldg(&a.row[v + 1]) - __ldg(&a.row[v]);
      float p = base + d * __ldcg(&a.hub_sum[h]);
      a.pr[v] = p;
      cout[v] = p / (float)dg;
      a.hub_sum[h] = 0.f;
    }
    *nxt = {1, t + 1};
    return WGM_PHASE_NEXT;
  }
  if (t >= a.iterations) return WGM_PHASE_DONE;
  if (c->id == 0 && threadIdx.x == 0) a.dang[((t + 2) % 3) * WGM_LINE] = 0.f;
  const int lane = s.lane, warp = s.warp;
  float *acc = reinterpret_cast<float *>(sm->acc[warp]);
  float dl = 0.f;
  for (int b = s.gw * 32; b < V; b += s.NW * 32) {
    int i = b + lane, deg = 0, start = 0, dfull = 0;
    if (i < V) {
      start = __ldg(&a.row[i]);
      dfull = __ldg(&a.row[i + 1]) - start;
      deg = dfull > a.hub_threshold ? 0 : dfull;
    }
    acc[lane] = 0.f;
    const int incl = wgm_warp_incl_scan(deg);
    const int total = __shfl_sync(WGM_FULL, incl, 31);
    const int off = incl - deg;
    const int ebase = start - off;
    __syncwarp();
    /* windows of 32 edge slots, four at a time: the col loads of the four
     * windows, then their gathers, are in flight together; each window's
     * contributions are then summed per owner by a segmented scan, windows
     * in order, so a vertex's sum has a fixed order */
    for (int w = 0; w < total; w += 128) {
      int own[4], u[4];
      float v[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int sl = w + 32 * q + lane;
        const int o = wgm_owner_of(off, min(sl, total - 1));
        own[q] = sl < total ? o : -1;
        const int e = __shfl_sync(WGM_FULL, ebase, o) + sl;
        u[q] = own[q] >= 0 ? __ldg(&a.col[e]) : 0;
      }
#pragma unroll
      for (int q = 0; q < 4; q++) v[q] = own[q] >= 0 ? __ldcg(&cin[u[q]]) : 0.f;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        float x = v[q];
        const int ow = own[q];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          float y = __shfl_up_sync(WGM_FULL, x, o);
          int oy = __shfl_up_sync(WGM_FULL, ow, o);
          if (lane >= o && oy == ow) x += y;
        }
        int nx = __shfl_down_sync(WGM_FULL, ow, 1);
        if (ow >= 0 && (lane == 31 || nx != ow)) acc[ow] += x;
        __syncwarp();
      }
    }
    __syncwarp();
    if (i < V && dfull <= a.hub_threshold) {
      float p = base + d * acc[lane];
      a.pr[i] = p;
      cout[i] = dfull > 0 ? p / (float)dfull : 0.f;
      if (dfull == 0) dl += p;
    }
  }
  /* hub edges: four windows per warp step, summed in groups of M windows,
   * in a two-stage pipeline: the next step's window records and col loads
   * (two dependent round trips) are issued before this step's gathers are
   * summed, so each step waits for about one round trip instead of three */
  const int nwin = (a.hubs.total + 31) >> 5;
  const int4 *wrec = reinterpret_cast<const int4 *>(a.hubs.wmap);
  const int kstep = s.NW * 4;
  int k0 = s.gw * 4;
  int hx[4], hh[4], u[4];
  if (k0 < nwin) wgm_pr_hub_stage(wrec, a.col, a.hubs.total, nwin, k0, lane, hx, hh, u);
  for (; k0 < nwin; k0 += kstep) {
    float v[4];
#pragma unroll
    for (int q = 0; q < 4; q++) v[q] = u[q] >= 0 ? __ldcg(&cin[u[q]]) : 0.f;
    int cx[4], ch[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      cx[q] = hx[q];
      ch[q] = hh[q];
    }
    if (k0 + kstep < nwin)
      wgm_pr_hub_stage(wrec, a.col, a.hubs.total, nwin, k0 + kstep, lane, hx, hh, u);
    if (a.hub_threshold >= 127)
      wgm_pr_hub_sums<4>(cx, ch, v, k0, nwin, a.hubs.H, a.hub_sum);
    else if (a.hub_threshold >= 63)
      wgm_pr_hub_sums<2>(cx, ch, v, k0, nwin, a.hubs.H, a.hub_sum);
    else
      wgm_pr_hub_sums<1>(cx, ch, v, k0, nwin, a.hubs.H, a.hub_sum);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) dl += __shfl_xor_sync(WGM_FULL, dl, o);
  if (lane == 0 && dl != 0.f) atomicAdd(&a.dang[((t + 1) % 3) * WGM_LINE], dl);
  *nxt = (a.hubs.H > 0) ? wgm_step{2, t} : wgm_step{1, t + 1};
  return WGM_PHASE_NEXT;
}

/* ------------------------------------------------------------------------ */
/* Pannotia betweenness centrality                                           */
/* ------------------------------------------------------------------------ */

struct wgm_bc_args {
  int V;
  const int *row, *col;   /* out-edges */
  const int *trow, *tcol; /* in-edges (the transpose; the graph when symmetric) */
  float *bc;              /* [V] output */
  int *dist;              /* [V] BFS level from the current source, -1 unreached */
  float *rho;             /* [V] shortest-path counts x 10000 */
  float *sigma;           /* [V] dependencies x 10000 */
  int *order;             /* [V] reached vertices, level by level */
  int *level_start;       /* [V + 2] first position of each level in order[] */
  int *cnt;               /* [3 lines] vertices found for a level, by level mod 3 */
  int num_sources;        /* sources 0 .. num_sources-1 (the reference: all V) */
  int *rounds_out;
};

#define WGM_BC_SCALE 10000.0f /* bc.cl:230 and :131: "scaling by 10000" */

/* bc.cl:1-235 (bc_combined: for every source s, clear, BFS with path
 * counts, backtrack with dependencies).  The reference scans every vertex
 * at every level for d[i] == level; here each level is a frontier list:
 * BFS level L relaxes the out-edges of order[level_start[L] ..] and appends
 * the vertices it discovers (one CAS each) as level L+1, so the backtrack
 * walks the same lists in reverse.  Arithmetic is the reference's: rho in
 * float scaled by 10000, rho[w] += rho[i] for every edge from level L to
 * L+1 (bc.cl:52-56), sigma[w] += rho[w] / rho[i] * (10000 + sigma[i]) for
 * every in-edge from level L-1 (bc.cl:122-124), bc[i] += sigma[i] / 10000
 * for every vertex but the source (bc.cl:131); only the order of the float
 * atomic adds differs (as between two runs of the reference).
 * Phases: target = kind | level << 2, round = source: kind 0 clears bc,
 * 1 clears the per-source state, 2 is a BFS level, 3 a backtrack level. */
static __device__ int wgm_phase_bc(const wgm_launch &Lc, wgm_cta *c, const wgm_bc_args &a,
                                   wgm_warp_smem *sm, wgm_step cur, wgm_step *nxt) {
  const wgm_split s(c);
  const int V = a.V, kind = cur.target & 3, L = cur.target >> 2, src = cur.round;
  const int lane = s.lane, warp = s.warp;
  if (kind == 0) {
    for (int i = s.tid; i < V; i += s.nth) a.bc[i] = 0.f;
    if (a.num_sources <= 0) {
      if (c->id == 0 && threadIdx.x == 0 && a.rounds_out) *a.rounds_out = 0;
      return WGM_PHASE_DONE;
    }
    *nxt = {1, 0};
    return WGM_PHASE_NEXT;
  }
  if (kind == 1) {
    /* clean_1d_array (bc.cl:165-181) */
    for (int i = s.tid; i < V; i += s.nth) {
      a.sigma[i] = 0.f;
      a.rho[i] = i == src ? WGM_BC_SCALE : 0.f;
      a.dist[i] = i == src ? 0 : -1;
    }
    if (c->id == 0 && threadIdx.x == 0) {
      a.order[0] = src;
      a.level_start[0] = 0;
      a.level_start[1] = 1;
      a.cnt[0] = 1;
      a.cnt[1 * WGM_LINE] = 0;
      a.cnt[2 * WGM_LINE] = 0;
    }
    *nxt = {2, src};
    return WGM_PHASE_NEXT;
  }
  if (kind == 2) {
    /* BFS level L (mega_bfs_kernel_func, bc.cl:16-92) */
    const int n = __ldcg(&a.cnt[(L % 3) * WGM_LINE]);
    const int S = __ldcg(&a.level_start[L]);
    if (n == 0) {
      /* no level L: the deepest is L-1, backtrack from it */
      *nxt = {3 | ((L - 1) << 2), src};
      return WGM_PHASE_NEXT;
    }
    if (L + 2 > V + 1) {
      wgm_fail(Lc, WGM_DEV_BAD_INPUT, WGM_SITE_QUEUE, L);
      return WGM_PHASE_DONE;
    }
    const int S1 = S + n;
    if (c->id == 0 && threadIdx.x == 0) {
      a.level_start[L + 1] = S1;
      a.cnt[((L + 2) % 3) * WGM_LINE] = 0;
    }
    int *ncnt = &a.cnt[((L + 1) % 3) * WGM_LINE];
    for (int b = s.gw * 32; b < n; b += s.NW * 32) {
      const int k = b + lane;
      int v = 0, start = 0, deg = 0;
      float rv = 0.f;
      if (k < n) {
        v = __ldcg(&a.order[S + k]);
        start = __ldg(&a.row[v]);
        deg = __ldg(&a.row[v + 1]) - start;
        rv = __ldcg(&a.rho[v]);
      }
      const int incl = wgm_warp_incl_scan(deg);
      const int total = __shfl_sync(WGM_FULL, incl, 31);
      const int off = incl - deg;
      wgm_for_each_edge(off, deg, start - off, total, 0, 32, sm->tab[warp],
                        [&](bool valid, int e, int owner) {
                          const float ro = __shfl_sync(WGM_FULL, rv, owner);
                          bool found = false;
                          int w = 0;
                          if (valid) {
                            w = __ldg(&a.col[e]);
                            int d = __ldcg(&a.dist[w]);
                            if (d < 0) {
                              d = atomicCAS(&a.dist[w], -1, L + 1);
                              found = d == -1;
                              if (found) d = L + 1;
                            }
                            if (d == L + 1) atomicAdd(&a.rho[w], ro);
                          }
                          wgm_warp_push(found, w, ncnt, a.order + S1, V - S1, false);
                        });
    }
    *nxt = {2 | ((L + 1) << 2), src};
    return WGM_PHASE_NEXT;
  }
  /* backtrack level L (mega_backtrack_kernel_func, bc.cl:96-140) */
  const int S = __ldcg(&a.level_start[L]), E = __ldcg(&a.level_start[L + 1]);
  for (int b = S + s.gw * 32; b < E; b += s.NW * 32) {
    const int k = b + lane;
    int v = 0, start = 0, deg = 0;
    float rv = 1.f, sv = 0.f;
    if (k < E) {
      v = __ldcg(&a.order[k]);
      start = __ldg(&a.trow[v]);
      deg = L > 0 ? __ldg(&a.trow[v + 1]) - start : 0;
      rv = __ldcg(&a.rho[v]);
      sv = __ldcg(&a.sigma[v]);
    }
    const int incl = wgm_warp_incl_scan(deg);
    const int total = __shfl_sync(WGM_FULL, incl, 31);
    const int off = incl - deg;
    wgm_for_each_edge(off, deg, start - off, total, 0, 32, sm->tab[warp],
                      [&](bool valid, int e, int owner) {
                        const float ri = __shfl_sync(WGM_FULL, rv, owner);
                        const float si = __shfl_sync(WGM_FULL, sv, owner);
                        if (valid) {
                          const int w = __ldg(&a.tcol[e]);
                          if (__ldcg(&a.dist[w]) == L - 1)
                            atomicAdd(&a.sigma[w], __ldcg(&a.rho[w]) / ri * (WGM_BC_SCALE + si));
                        }
                      });
    if (k < E && v != src) a.bc[v] = a.bc[v] + sv / WGM_BC_SCALE;
  }
  if (L > 0) {
    *nxt = {3 | ((L - 1) << 2), src};
    return WGM_PHASE_NEXT;
  }
  if (src + 1 >= a.num_sources) {
    if (c->id == 0 && threadIdx.x == 0 && a.rounds_out) *a.rounds_out = src + 1;
    return WGM_PHASE_DONE;
  }
  *nxt = {1, src + 1};
  return WGM_PHASE_NEXT;
}

/* Betweenness centrality with the sources spread over CTAs: a CTA takes a
 * source from a queue and runs its BFS and backtrack alone, with dist, rho,
 * sigma, the level lists and their starts in shared memory (20 bytes per
 * vertex) and __syncthreads as the level barrier; bc gathers the
 * dependencies with global float atomics.  Same arithmetic as wgm_phase_bc,
 * no grid barrier at all: sources, not levels, are the parallel units.  For
 * graphs of at most WGM_BC_CTA_MAX_V vertices. */
#define WGM_BC_CTA_MAX_V 10240


static __device__ void wgm_bc_cta_source(const wgm_bc_args &a, int src, int *dist, float *rho,
                                  float *sig, int *order, int *ls, int *s_cnt, int *tab) {
  const int V = a.V, lane = wgm_lane(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = threadIdx.x; i < V; i += blockDim.x) {
    dist[i] = i == src ? 0 : -1;
    rho[i] = i == src ? WGM_BC_SCALE : 0.f;
    sig[i] = 0.f;
  }
  if (threadIdx.x == 0) {
    order[0] = src;
    ls[0] = 0;
    ls[1] = 1;
    *s_cnt = 0;
  }
  __syncthreads();
  int L = 0, S = 0, n = 1;
  for (;;) {
    const int S1 = S + n;
    for (int b = warp * 32; b < n; b += nw * 32) {
      const int k = b + lane;
      int v = 0, start = 0, deg = 0;
      float rv = 0.f;
      if (k < n) {
        v = order[S + k];
        start = __ldg(&a.row[v]);
        deg = __ldg(&a.row[v + 1]) - start;
        rv = rho[v];
      }
      const int incl = wgm_warp_incl_scan(deg);
      const int total = __shfl_sync(WGM_FULL, incl, 31);
      const int off = incl - deg;
      wgm_for_each_edge(off, deg, start - off, total, 0, 32, tab + warp * 32,
                        [&](bool valid, int e, int owner) {
                          const float ro = __shfl_sync(WGM_FULL, rv, owner);
                          bool found = false;
                          int w = 0;
                          if (valid) {
                            w = __ldg(&a.col[e]);
                            int d = dist[w];
                            if (d < 0) {
                              d = atomicCAS(&dist[w], -1, L + 1);
                              found = d == -1;
                              if (found) d = L + 1;
                            }
                            if (d == L + 1) atomicAdd(&rho[w], ro);
                          }
                          wgm_warp_push(found, w, s_cnt, order + S1, V - S1, false);
                        });
    }
    __syncthreads();
    const int n2 = *s_cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
      *s_cnt = 0;
      ls[L + 2] = S1 + n2;
    }
    if (n2 == 0) break;
    S = S1;
    n = n2;
    L++;
  }
  __syncthreads();
  for (int l = L; l >= 0; l--) {
    const int B = ls[l], E = ls[l + 1];
    for (int b = B + warp * 32; b < E; b += nw * 32) {
      const int k = b + lane;
      int v = 0, start = 0, deg = 0;
      float rv = 1.f, sv = 0.f;
      if (k < E) {
        v = order[k];
        start = __ldg(&a.trow[v]);
        deg = l > 0 ? __ldg(&a.trow[v + 1]) - start : 0;
        rv = rho[v];
        sv = sig[v];
      }
      const int incl = wgm_warp_incl_scan(deg);
      const int total = __shfl_sync(WGM_FULL, incl, 31);
      const int off = incl - deg;
      wgm_for_each_edge(off, deg, start - off, total, 0, 32, tab + warp * 32,
                        [&](bool valid, int e, int owner) {
                          const float ri = __shfl_sync(WGM_FULL, rv, owner);
                          const float si = __shfl_sync(WGM_FULL, sv, owner);
                          if (valid) {
                            const int w = __ldg(&a.tcol[e]);
                            if (dist[w] == l - 1)
                              atomicAdd(&sig[w], rho[w] / ri * (WGM_BC_SCALE + si));
                          }
                        });
      if (k < E && v != src && sv != 0.f) atomicAdd(&a.bc[v], sv / WGM_BC_SCALE);
    }
    __syncthreads();
  }
}

#endif
