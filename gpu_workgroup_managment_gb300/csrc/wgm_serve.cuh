/*
 * Served form: one megakernel launch hosts a resident persistent job (Pannotia
 * colour then Lonestar BFS on one graph, repeated) and, beside it, a stream
 * of requests - BFS queries on resident graphs, FP32 reductions, FP32 matrix
 * products - that arrive while it runs.  Discovered group 0 is the
 * scheduler: it reads request descriptors from a host ring (mapped memory),
 * gives each request a team of free groups, and when too few are free asks
 * the persistent job for groups; the persistent job cedes them at its next
 * resizing barrier (offer_kill, the highest persistent ids leave) and takes
 * free groups back (offer_fork) when no request is waiting.  Several
 * requests run at once on different teams (continuous batching); each team's
 * last group posts the completion to a host ring.
 *
 * Reference counterparts (paths relative to the reference):
 *   src/scheduler_rt/rt_device/cl_scheduler.cl:191-308  scheduler loop -> wgm_serve_scheduler
 *   src/scheduler_rt/rt_device/scheduler_1.cl:10-81     offer_fork/kill -> wgm_serve_fork,
 *                                                       wgm_offer_kill
 *   src/scheduler_rt/rt_device/iw_barrier.cl:165-227    resizing barrier -> wgm_serve_barrier
 *   src/scheduler_rt/rt_device/main_device_body.cl:1-93 worker loop -> wgm_k_serve
 * The reference serves one non-persistent task at a time from a host flag
 * handshake; here requests queue on the device and run concurrently, and the
 * free groups are tracked in a bitmap, so a team can take any free slots.
 */
#ifndef WGM_SERVE_CUH
#define WGM_SERVE_CUH

#include "wgm_batch.cuh"
#include "wgm_mega.cuh"

/* Request kinds (wgm_req.kind). */
#define WGM_REQ_BFS 1    /* Lonestar BFS on resident graph arg0 from source arg1 */
#define WGM_REQ_REDUCE 2 /* FP32 min over resident vector arg0 */
#define WGM_REQ_MATMUL 3 /* FP32 n x n product of resident operand pair arg0 */
#define WGM_REQ_REDUCE_I32 4 /* reduce.cl: int32 min over resident int vector arg0 */
#define WGM_REQ_MATMUL_I32 5 /* matmult.cl: int32 product of int pair arg0 + diagonal hash */

#define WGM_TASK_REQ 3 /* task_array value: run request slot_req[slot] */

/* Request descriptor, written by the host into the mapped request ring. */
struct wgm_req {
  int kind;
  int groups; /* team size */
  int arg0, arg1;
  long long state_off; /* byte offset of the request's state in the arena */
  int id;              /* completion record value - 1 */
  int pad[9];
};

/* Resident BFS graph of the request stream. */
struct wgm_serve_graph {
  int V, piece, cap, pad;
  long long row_off, col_off;
};

/* Request state layout (arena, 256-byte aligned; lines of WGM_LINE ints):
 * line 0: done counter; lines 1-3: BFS level counters; line 4: team barrier
 * arrivals; line 5: result word (reduce); then the payload (BFS: dist[V],
 * wl_start[2][cap], wl_cnt[2][cap]; matmul: C[n*n]). */
#define WGM_REQ_CTL_LINES 6
#define WGM_REQ_CTL_BYTES (WGM_REQ_CTL_LINES * WGM_LINE * 4)

/* Device words of the serving loop (device memory, zeroed before launch). */
struct wgm_serve_dev {
  int free_bits[WGM_MAX_GROUPS / 32]; /* bit s: slot s is free and unclaimed */
  int slot_req[WGM_MAX_GROUPS];       /* request ring index of the slot's task */
  int slot_rank[WGM_MAX_GROUPS];      /* rank in that request's team */
  int pending;                        /* requests seen but not yet given groups */
  int pad0[WGM_LINE - 1];
  int pad1[WGM_LINE];
  int persist_done;                   /* persistent repetitions completed */
  int pad2[WGM_LINE - 1];
  int kills;                          /* groups ceded by the persistent job */
  int forks;                          /* groups taken back */
  int pad3[WGM_LINE - 2];
  int completed;                      /* requests finished */
  int pad4[WGM_LINE - 1];
  /* the persistent job's barrier (wgm_serve_barrier): the released
   * generation in the low half, 1 in the high half when the next barrier
   * resizes; and the arrivals of the current barrier, plus
   * WGM_SERVE_RESIZE_FLAG for every request of a resizing barrier */
  unsigned long long gate;
  int pad5[WGM_LINE - 2];
  int arrive;
  int pad6[WGM_LINE - 1];
};

#define WGM_SERVE_RESIZE_FLAG (1 << 16)
#define WGM_SERVE_ARRIVALS 0xffff
/* restoration record word: the group's next barrier resizes */
#define WGM_RC_SERVE_SLOW 4
/* free groups beyond the reserve that make the scheduler ask for a fork */
#define WGM_SERVE_FORK_MIN 16

/* Host-visible words of the serving loop (mapped pinned memory). */
struct wgm_serve_host {
  int head;      /* requests written by the host (ring index, grows) */
  int quit;      /* host: no more requests; end when everything drained */
  int pad0[WGM_LINE - 2];
  int seen;      /* scheduler: requests read from the ring */
  int started;   /* scheduler: requests given a team */
  int persist_reps; /* persistent repetitions completed */
  int persist_groups; /* groups of the persistent job, as of its last resize */
  int pad1[WGM_LINE - 4];
};

struct wgm_serve_args {
  /* persistent job: colour, then Lonestar BFS, `reps` times */
  wgm_color_args color;
  wgm_lonestar_args ls;
  int reps;
  int persist_groups; /* groups given to the persistent job at start (0: none) */
  /* request stream */
  const wgm_req *ring; /* mapped host ring of `ring_size` descriptors */
  int ring_size;
  int *completions;    /* mapped host ring: id + 1 when request id finished */
  wgm_serve_host *hs;  /* mapped */
  wgm_serve_dev *sd;   /* device */
  wgm_req *dreq;       /* device copy of the ring */
  char *arena;         /* request state */
  const int *g_rows, *g_cols;
  const wgm_serve_graph *graphs;
  const float *vecs; /* reduce inputs, vec_len floats each */
  int vec_len;
  const float *mats; /* matmul operand pairs: A then B, mat_n^2 floats each */
  int mat_n;
  const int *ivecs;  /* int32 reduce inputs, ivec_len each */
  int ivec_len;
  const int *imats;  /* int32 operand pairs, imat_n^2 each */
  int imat_n;
  int *err;          /* team waits: first error, site */
  unsigned long long *rtimes; /* per request id: start, end (%globaltimer ns) */
  int max_requests;           /* entries of rtimes */
  int reserve;       /* free groups the fork leaves for requests */
  int persist_max;   /* most groups the persistent job forks up to */
  unsigned long long idle_ns;
};

/* ---- pool of free groups: a bitmap, claimed under the pool lock ---------- */

/* A group enters the pool: WAIT first, then its bit (release), then the
 * count.  Whoever claims the bit sees the WAIT and overwrites it. */
__device__ __forceinline__ void wgm_pool_enter(const wgm_launch &L, wgm_serve_dev *sd, int slot) {
  wgm_st_relaxed_gpu(&L.st->task_array[slot], WGM_TASK_WAIT);
  asm volatile("red.release.gpu.global.or.b32 [%0], %1;" ::"l"(&sd->free_bits[slot >> 5]),
               "r"(1u << (slot & 31))
               : "memory");
  wgm_atom_add_acqrel_gpu(&L.st->available_workgroups, 1);
}

/* Claim up to `want` free slots into out[] (shared memory); warp-wide, the
 * caller's warp holds the pool lock.  Slots are scanned from the top down, so
 * requests and the persistent job mostly keep to separate ends.  Returns the
 * number claimed (warp-uniform). */
__device__ __forceinline__ int wgm_pool_claim(wgm_serve_dev *sd, int nslots, int want, int *out) {
  const int lane = wgm_lane();
  const int nwords = (nslots + 31) >> 5;
  int got = 0;
  for (int w0 = nwords - 1; w0 >= 0 && got < want; w0 -= 32) {
    const int w = w0 - lane;
    unsigned bits = 0;
    if (w >= 0) bits = (unsigned)wgm_ld_acquire_gpu(&sd->free_bits[w]);
    /* slots beyond nslots never have bits; take the highest bits first */
    int cnt = __popc(bits);
    int incl = wgm_warp_incl_scan(cnt);
    int excl = incl - cnt;
    int total = __shfl_sync(WGM_FULL, incl, 31);
    int take = max(0, min(cnt, want - got - excl));
    unsigned mine = 0;
    for (int k = 0; k < take; k++) {
      int b = 31 - __clz(bits);
      bits &= ~(1u << b);
      mine |= 1u << b;
      out[got + excl + k] = w * 32 + b;
    }
    if (mine) atomicAnd(&sd->free_bits[w], ~(int)mine);
    got += min(total, want - got);
    __syncwarp();
  }
  return got;
}


/* ---- requests (run by the groups of their team) -------------------------- */

__device__ __forceinline__ int *wgm_req_ctl(const wgm_serve_args &A, const wgm_req &r) {
  return (int *)(A.arena + r.state_off);
}

/* BFS query: the batched form's team Lonestar BFS on a resident graph. */
__device__ void wgm_req_bfs(const wgm_serve_args &A, const wgm_req &r, int rank,
                            wgm_warp_smem *sm) {
  const wgm_serve_graph g = A.graphs[r.arg0];
  int *ctl = wgm_req_ctl(A, r);
  wgm_ls_job J;
  J.V = g.V;
  J.source = r.arg1;
  J.piece = g.piece;
  J.cap = g.cap;
  J.G = r.groups;
  J.rank = rank;
  J.row = A.g_rows + g.row_off;
  J.col = A.g_cols + g.col_off;
  J.wt = nullptr;
  J.dist = (unsigned *)(ctl + WGM_REQ_CTL_LINES * WGM_LINE);
  J.stamp = nullptr;
  J.wl_start = (int *)(J.dist + ((g.V + 63) & ~63));
  J.wl_cnt = J.wl_start + 2 * (size_t)g.cap;
  J.wl_u = nullptr;
  J.cnt = ctl + 1 * WGM_LINE;
  J.arr = ctl + 4 * WGM_LINE;
  wgm_team_ls_run<false>(J, sm, A.err, A.idle_ns);
}

/* FP32 min over a resident vector (reduce.cl:3-39 on floats): block min,
 * then one atomicMin on the int bits (inputs are non-negative). */
__device__ void wgm_req_reduce(const wgm_serve_args &A, const wgm_req &r, int rank) {
  __shared__ int red[32];
  const float *x = A.vecs + (size_t)r.arg0 * A.vec_len;
  const int gid = rank * blockDim.x + threadIdx.x, nth = r.groups * blockDim.x;
  int m = INT_MAX;
  const int len = A.vec_len;
  /* vectors start wherever vec_len puts them: scalar loads up to the first
   * 16-byte boundary, float4 loads for the body, scalar loads for the tail */
  const int pre = min(len, (int)(((16u - ((unsigned)(uintptr_t)x & 15u)) & 15u) >> 2));
  const int n4 = (len - pre) >> 2;
  const float4 *x4 = reinterpret_cast<const float4 *>(x + pre);
  for (int i = gid; i < pre; i += nth) m = min(m, __float_as_int(__ldg(&x[i])));
  for (int i = gid; i < n4; i += nth) {
    float4 v = __ldg(x4 + i);
    m = min(m, min(min(__float_as_int(v.x), __float_as_int(v.y)),
                   min(__float_as_int(v.z), __float_as_int(v.w))));
  }
  for (int i = pre + (n4 << 2) + gid; i < len; i += nth) m = min(m, __float_as_int(__ldg(&x[i])));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(WGM_FULL, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    int v = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : INT_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(WGM_FULL, v, o));
    if (threadIdx.x == 0) atomicMin(wgm_req_ctl(A, r) + 5 * WGM_LINE, v);
  }
  __syncthreads();
}

/* int32 min over a resident vector (reduce.cl:3-39): block min, one
 * atomicMin per group on the result word. */
__device__ void wgm_req_reduce_i32(const wgm_serve_args &A, const wgm_req &r, int rank) {
  __shared__ int red[32];
  const int *x = A.ivecs + (size_t)r.arg0 * A.ivec_len;
  const int gid = rank * blockDim.x + threadIdx.x, nth = r.groups * blockDim.x;
  const int len = A.ivec_len;
  const int pre = min(len, (int)(((16u - ((unsigned)(uintptr_t)x & 15u)) & 15u) >> 2));
  const int n4 = (len - pre) >> 2;
  const int4 *x4 = reinterpret_cast<const int4 *>(x + pre);
  int m = INT_MAX;
  for (int i = gid; i < pre; i += nth) m = min(m, __ldg(&x[i]));
  for (int i = gid; i < n4; i += nth) {
    int4 v = __ldg(x4 + i);
    m = min(m, min(min(v.x, v.y), min(v.z, v.w)));
  }
  for (int i = pre + (n4 << 2) + gid; i < len; i += nth) m = min(m, __ldg(&x[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(WGM_FULL, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    int v = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : INT_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(WGM_FULL, v, o));
    if (threadIdx.x == 0) atomicMin(wgm_req_ctl(A, r) + 5 * WGM_LINE, v);
  }
  __syncthreads();
}

/* int32 C = A * B with wrapping arithmetic (matmult.cl:26-67), tiles over
 * the team; the group that finishes last hashes the diagonal (djb2,
 * matmult.cl:64, wrapping int32) into the result word. */
__device__ void wgm_req_matmul_i32(const wgm_serve_args &A, const wgm_req &r, int rank) {
  __shared__ int ta[32][33], tb[32][33];
  const int n = A.imat_n, nt = n >> 5;
  const int *Am = A.imats + (size_t)r.arg0 * 2 * n * n, *Bm = Am + (size_t)n * n;
  int *ctl = wgm_req_ctl(A, r);
  int *C = ctl + WGM_REQ_CTL_LINES * WGM_LINE;
  for (int t = rank; t < nt * nt; t += r.groups) {
    const int ti = t / nt, tj = t % nt;
    unsigned acc[4] = {0u, 0u, 0u, 0u};
    for (int k0 = 0; k0 < n; k0 += 32) {
      __syncthreads();
      for (int e = threadIdx.x; e < 1024; e += blockDim.x) {
        const int y = e >> 5, x = e & 31;
        ta[y][x] = __ldg(&Am[(size_t)(ti * 32 + y) * n + k0 + x]);
        tb[y][x] = __ldg(&Bm[(size_t)(k0 + y) * n + tj * 32 + x]);
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int e = threadIdx.x + q * blockDim.x;
        if (e < 1024) {
          const int y = e >> 5, x = e & 31;
          unsigned a = acc[q];
#pragma unroll 8
          for (int k = 0; k < 32; k++) a += (unsigned)ta[y][k] * (unsigned)tb[k][x];
          acc[q] = a;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int e = threadIdx.x + q * blockDim.x;
      if (e < 1024) C[(size_t)(ti * 32 + (e >> 5)) * n + tj * 32 + (e & 31)] = (int)acc[q];
    }
  }
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    /* the done counter of line 0 is the completion's; count the products
     * on line 1 (unused by this kind) */
    s_last = wgm_atom_add_acqrel_gpu(ctl + 1 * WGM_LINE, 1) == r.groups - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x < 32) {
    /* djb2 over the diagonal in order: the warp loads it, lane 0 folds */
    unsigned h = 5381;
    for (int i0 = 0; i0 < n; i0 += 32) {
      const int i = i0 + (int)threadIdx.x;
      const unsigned v = i < n ? (unsigned)__ldcg(&C[(size_t)i * n + i]) : 0u;
      for (int k = 0; k < 32 && i0 + k < n; k++) h = h * 33u + __shfl_sync(WGM_FULL, v, k);
    }
    if (threadIdx.x == 0) {
      ctl[5 * WGM_LINE] = (int)h;
      __threadfence();
    }
  }
  __syncthreads();
}

/* FP32 C = A * B, n x n (n a multiple of 32): 32x32 tiles of C over the
 * team, k in steps of 32 through shared memory; every element sums its k
 * terms in increasing k with fmaf, so the result does not depend on the team
 * size or the block size. */
__device__ void wgm_req_matmul(const wgm_serve_args &A, const wgm_req &r, int rank) {
  __shared__ float ta[32][33], tb[32][33];
  const int n = A.mat_n, nt = n >> 5;
  const float *Am = A.mats + (size_t)r.arg0 * 2 * n * n, *Bm = Am + (size_t)n * n;
  float *C = (float *)(wgm_req_ctl(A, r) + WGM_REQ_CTL_LINES * WGM_LINE);
  for (int t = rank; t < nt * nt; t += r.groups) {
    const int ti = t / nt, tj = t % nt;
    float acc[4] = {0.f, 0.f, 0.f, 0.f}; /* elements threadIdx.x + q*blockDim.x */
    for (int k0 = 0; k0 < n; k0 += 32) {
      __syncthreads();
      for (int e = threadIdx.x; e < 1024; e += blockDim.x) {
        const int y = e >> 5, x = e & 31;
        ta[y][x] = __ldg(&Am[(size_t)(ti * 32 + y) * n + k0 + x]);
        tb[y][x] = __ldg(&Bm[(size_t)(k0 + y) * n + tj * 32 + x]);
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int e = threadIdx.x + q * blockDim.x;
        if (e < 1024) {
          const int y = e >> 5, x = e & 31;
          float a = acc[q];
#pragma unroll 8
          for (int k = 0; k < 32; k++) a = fmaf(ta[y][k], tb[k][x], a);
          acc[q] = a;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int e = threadIdx.x + q * blockDim.x;
      if (e < 1024) C[(size_t)(ti * 32 + (e >> 5)) * n + tj * 32 + (e & 31)] = acc[q];
    }
  }
  __syncthreads();
}


/* ---- the resident persistent job ---------------------------------------- */

/* (colour, then Lonestar BFS) x reps as one phase sequence, so a forked group
 * resumes it from (target, round) alone.  target = rep << 9 | app << 8 | the
 * app's own target (colour 0-2, Lonestar 0-1). */
__device__ int wgm_phase_combo(const wgm_launch &L, wgm_cta *c, const wgm_serve_args &A,
                               wgm_warp_smem *sm, wgm_step cur, wgm_step *nxt) {
  const int rep = cur.target >> 9, app = (cur.target >> 8) & 1, t = cur.target & 255;
  if (rep >= A.reps) return WGM_PHASE_DONE;
  if (app == 0) {
    wgm_step sc = {t, cur.round}, sn = sc;
    if (wgm_phase_color(L, c, A.color, sm, sc, &sn) == WGM_PHASE_NEXT) {
      *nxt = {(rep << 9) | sn.target, sn.round};
    } else {
      *nxt = {(rep << 9) | (1 << 8), 0}; /* this repetition's BFS, init phase */
    }
    return WGM_PHASE_NEXT;
  }
  int nt = 0, nr = 0;
  if (wgm_phase_lonestar<false>(L, c, A.ls, sm, t, cur.round, &nt, &nr)) {
    *nxt = {(rep << 9) | (1 << 8) | nt, nr};
    return WGM_PHASE_NEXT;
  }
  if (c->id == 0 && threadIdx.x == 0) {
    atomicAdd(&A.sd->persist_done, 1);
    wgm_st_release_sys(&A.hs->persist_reps, rep + 1);
  }
  *nxt = {(rep + 1) << 9, 0};
  return rep + 1 < A.reps ? WGM_PHASE_NEXT : WGM_PHASE_DONE;
}

__device__ __forceinline__ unsigned long long wgm_ld_acquire_gpu_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void wgm_st_release_gpu_u64(unsigned long long *p,
                                                       unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ int wgm_atom_exch_acqrel_gpu_s(int *p, int v) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;"
               : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

/* Wait until the job's gate releases generation g + 1; returns its resize
 * bit, or -1 when the wait gave up. */
__device__ __forceinline__ int wgm_serve_gate_wait(const wgm_launch &L, wgm_serve_dev *sd, int g) {
  wgm_spin s = wgm_spin_start(L);
  for (;;) {
    const unsigned long long v = wgm_ld_acquire_gpu_u64(&sd->gate);
    if ((int)((unsigned)v - (unsigned)(g + 1)) >= 0) return (int)(v >> 32);
    if (wgm_spin_giveup(L, s, WGM_SITE_RESIZE_BARRIER)) return -1;
  }
}

/* Barrier of the served form's persistent job.  Most barriers are plain:
 * every group adds one arrival, the last one releases the next generation
 * (a sense barrier, two dependent L2 round trips).  A barrier resizes only
 * when the one before it said so, in the high half of the generation word
 * it released: the scheduler asks for that by adding WGM_SERVE_RESIZE_FLAG
 * to the arrival word when a request waits for groups (or free groups could
 * be taken back), and the last arriver, resetting the word, sees the flag.
 * Every group reads the bit with the generation it waits for, so all agree
 * on the next barrier's kind without another round trip.
 *
 * A resizing barrier is global_barrier_resize (iw_barrier.cl:165-227) as in
 * the megakernel - a slave first offers to die, the master waits for every
 * live slave - with a fork that takes free groups from the bitmap (any
 * slots) and only when no request is waiting, leaving `reserve` groups free
 * for the next requests.  Warp 0 of the master scans the bitmap.  The master
 * keeps the next barrier resizing while a request still wants groups.  So
 * the reference's kill on arrival happens within two barriers of the
 * request, and the plain barriers the job runs otherwise cost what its
 * standalone barrier costs.  Returns 1 to continue, 0 if this group was
 * killed, -1 on a failed wait. */
#define WGM_SERVE_FORK_MAX 256
static __device__ int wgm_serve_barrier(const wgm_launch &L, wgm_cta *c, wgm_step nxt,
                                        const wgm_serve_args &A, int nslots, int *s_claim) {
  __shared__ int s_want;
  wgm_dev_state *st = L.st;
  wgm_serve_dev *sd = A.sd;
  int *kng = &st->k_num_groups[1][0];
  __syncthreads();
  if (threadIdx.x < 32) {
    const int g = c->gen;
    int res = 1, slow = 0;
    const bool resize = c->tmp[3] != 0;
    if (!resize) {
      if (threadIdx.x == 0) {
        const int r = wgm_atom_add_acqrel_gpu(&sd->arrive, 1);
        if ((r & WGM_SERVE_ARRIVALS) + 1 == c->ngroups) {
          const unsigned old = (unsigned)wgm_atom_exch_acqrel_gpu_s(&sd->arrive, 0);
          slow = (old >> 16) != 0 ? 1 : 0;
          wgm_st_release_gpu_u64(&sd->gate,
                                 (unsigned)(g + 1) | ((unsigned long long)slow << 32));
        } else {
          slow = wgm_serve_gate_wait(L, sd, g);
          if (slow < 0) res = -1;
        }
      }
    } else if (c->id != 0) {
      if (threadIdx.x == 0) {
        if (wgm_offer_kill(L, c->id)) {
          res = 0;
          atomicAdd(&sd->kills, 1);
        } else {
          wgm_atom_add_acqrel_gpu(&sd->arrive, 1);
          slow = wgm_serve_gate_wait(L, sd, g);
          if (slow < 0) res = -1;
        }
      }
    } else {
      int n = 0;
      if (threadIdx.x == 0) {
        wgm_spin s = wgm_spin_start(L);
        for (;;) {
          int arrived = wgm_ld_acquire_gpu(&sd->arrive) & WGM_SERVE_ARRIVALS;
          n = wgm_ld_acquire_gpu(kng);
          if (arrived == n - 1) break;
          if (wgm_spin_giveup(L, s, WGM_SITE_RESIZE_BARRIER)) {
            res = -1;
            break;
          }
        }
        int want = 0;
        if (res == 1) {
          const unsigned old = (unsigned)wgm_atom_exch_acqrel_gpu_s(&sd->arrive, 0);
          n = wgm_ld_acquire_gpu(kng);
          slow = ((old >> 16) != 0 || wgm_ld_acquire_gpu(&st->groups_to_kill) > 0) ? 1 : 0;
          if (wgm_ld_acquire_gpu(&sd->pending) == 0) {
            int spare = wgm_ld_acquire_gpu(&st->available_workgroups) - A.reserve;
            want = min(min(spare, WGM_SERVE_FORK_MAX), A.persist_max - n);
            if (want > 0 && !wgm_try_lock(&st->pool_lock)) want = 0;
          }
        }
        s_want = want;
      }
      __syncwarp();
      const int want = s_want;
      int got = 0;
      if (want > 0) got = wgm_pool_claim(sd, nslots, want, s_claim);
      __syncwarp();
      if (threadIdx.x == 0 && res == 1) {
        if (want > 0) {
          wgm_rctx rc;
          for (int k = 0; k < WGM_RCTX_WORDS; k++) rc.w[k] = 0;
          rc.w[WGM_RC_TARGET] = nxt.target;
          rc.w[WGM_RC_ROUND] = nxt.round;
          rc.w[WGM_RC_GEN] = g + 1;
          rc.w[WGM_RC_NGROUPS] = n + got;
          rc.w[WGM_RC_SERVE_SLOW] = slow;
          for (int k = 0; k < got; k++) {
            const int slot = s_claim[k];
            st->k_group_ids[1][slot] = n + k;
            st->r_ctx_arr[slot] = rc;
          }
          if (got > 0) {
            wgm_atom_add_acqrel_gpu(kng, got);
            atomicAdd(&st->k_executing[1][0], got);
            wgm_atom_add_acqrel_sys(&L.hf->persistent_flag, got);
            atomicAdd(&st->available_workgroups, -got);
            atomicAdd(&sd->forks, got);
            for (int k = 0; k < got; k++)
              wgm_st_release_gpu(&st->task_array[s_claim[k]], WGM_TASK_PERSIST);
          }
          wgm_unlock(&st->pool_lock);
          n += got;
        }
        wgm_st_relaxed_gpu(&st->bar_num_groups, n);
        wgm_st_relaxed_sys(&A.hs->persist_groups, n); /* the host's groups-over-time trace */
        wgm_st_release_gpu_u64(&sd->gate, (unsigned)(g + 1) | ((unsigned long long)slow << 32));
      }
    }
    if (threadIdx.x == 0) {
      c->gen = g + 1;
      /* the group count changes only at resizing barriers; after one it is
       * the count the master published with the release */
      if (res == 1 && resize) c->ngroups = wgm_ld_acquire_gpu(&st->bar_num_groups);
      if (res == -1) c->ok = 0;
      c->tmp[1] = res;
      c->tmp[3] = slow > 0 ? 1 : 0;
    }
  }
  __syncthreads();
  return c->tmp[1];
}


/* ---- scheduler (warp 0 of discovered group 0) ---------------------------- */

__device__ __forceinline__ int wgm_bcast(int v) { return __shfl_sync(WGM_FULL, v, 0); }

/* Lock the pool from lane 0 of the scheduler warp; warp-uniform result. */
__device__ __forceinline__ bool wgm_warp_lock(const wgm_launch &L, int *m) {
  int ok = 1;
  if (wgm_lane() == 0) ok = wgm_lock(L, m, WGM_SITE_SCHEDULER) ? 1 : 0;
  return wgm_bcast(ok) != 0;
}

/* Give `G` claimed slots (s_claim) a task: the persistent job (ids from
 * first_id, restoration record rc) or request ring index ri (ranks 0..G-1). */
__device__ __forceinline__ void wgm_assign(const wgm_launch &L, const wgm_serve_args &A, int G,
                                           const int *s_claim, int task, int ri, int first_id,
                                           const wgm_rctx &rc) {
  wgm_dev_state *st = L.st;
  for (int k = wgm_lane(); k < G; k += 32) {
    const int slot = s_claim[k];
    if (task == WGM_TASK_PERSIST) {
      st->k_group_ids[1][slot] = first_id + k;
      st->r_ctx_arr[slot] = rc;
    } else {
      A.sd->slot_req[slot] = ri;
      A.sd->slot_rank[slot] = k;
    }
    wgm_st_release_gpu(&st->task_array[slot], task);
  }
  __syncwarp();
}

/* The serving loop: start the persistent job on persist_groups groups, then
 * move request descriptors from the host ring to the device, give each
 * request (in arrival order) a team as soon as enough groups are free - if
 * not, ask the persistent job for the difference through groups_to_kill -
 * and, once the host has set quit and every request and the persistent job
 * are done, send every group QUIT.  Returns false when a wait gave up. */
static __device__ bool wgm_serve_scheduler(const wgm_launch &L, const wgm_serve_args &A, int lpg,
                                           int *s_claim) {
  wgm_dev_state *st = L.st;
  wgm_serve_dev *sd = A.sd;
  const int lane = wgm_lane();
  const int nslots = lpg + 1; /* worker slots 1..lpg; slot 0 (the scheduler) has no bit */
  wgm_rctx rc;
  for (int k = 0; k < WGM_RCTX_WORDS; k++) rc.w[k] = 0;
  if (lane == 0) {
    wgm_st_relaxed_gpu(&st->k_executing[1][0], 0);
    wgm_st_relaxed_gpu(&st->k_num_groups[1][0], 0);
    wgm_st_relaxed_gpu(&st->groups_to_kill, 0);
  }
  /* every worker enters the pool first */
  int ok = 1;
  if (lane == 0)
    ok = wgm_wait_geq(L, A.idle_ns, &st->available_workgroups, lpg, WGM_SITE_SCHEDULER) ? 1 : 0;
  if (!wgm_bcast(ok)) return false;
  const int P = min(A.persist_groups, lpg);
  if (P > 0) {
    if (!wgm_warp_lock(L, &st->pool_lock)) return false;
    if (lane == 0) {
      wgm_st_relaxed_gpu(&st->k_num_groups[1][0], P);
      wgm_st_relaxed_gpu(&st->bar_num_groups, P);
      wgm_st_relaxed_gpu(&st->k_executing[1][0], P);
      wgm_st_relaxed_gpu(&st->groups_to_kill, 0);
      wgm_st_relaxed_gpu(&sd->arrive, 0);
      wgm_st_relaxed_sys(&A.hs->persist_groups, P);
      wgm_st_release_sys(&L.hf->persistent_flag, P);
    }
    rc.w[WGM_RC_GEN] =
        wgm_bcast(lane == 0 ? (int)(unsigned)wgm_ld_acquire_gpu_u64(&sd->gate) : 0);
    rc.w[WGM_RC_NGROUPS] = P;
    rc.w[WGM_RC_SERVE_SLOW] = 1; /* the job's first barrier resizes */
    for (int done = 0; done < P;) {
      const int want = min(P - done, WGM_SERVE_FORK_MAX);
      const int got = wgm_pool_claim(sd, nslots, want, s_claim);
      if (got == 0) break;
      wgm_assign(L, A, got, s_claim, WGM_TASK_PERSIST, 0, done, rc);
      if (lane == 0) atomicAdd(&st->available_workgroups, -got);
      done += got;
    }
    if (lane == 0) wgm_unlock(&st->pool_lock);
  }
  int seen = 0, started = 0;
  unsigned fork_gen = 0xffffffffu; /* gate generation of the last fork request */
  wgm_spin idle = wgm_idle_start(L, A.idle_ns);
  for (;;) {
    bool progress = false;
    /* new descriptors: host ring (mapped) -> device ring.  Every lane takes
     * the head with its own acquire load (and the warp the smallest value),
     * so each lane's reads of the descriptor words are ordered after the
     * host's writes of them. */
    const int head = (int)__reduce_min_sync(
        WGM_FULL, (unsigned)wgm_ld_acquire_sys(&A.hs->head));
    if (head != seen) {
      for (int idx = seen; idx != head; idx++) {
        const int ri = idx % A.ring_size;
        const int *src = reinterpret_cast<const int *>(&A.ring[ri]);
        int *dst = reinterpret_cast<int *>(&A.dreq[ri]);
        if (lane < (int)(sizeof(wgm_req) / 4)) dst[lane] = wgm_ld_relaxed_sys(src + lane);
      }
      __threadfence();
      __syncwarp();
      if (lane == 0) {
        atomicAdd(&sd->pending, head - seen);
        wgm_st_relaxed_sys(&A.hs->seen, head);
      }
      seen = head;
      progress = true;
    }
    /* start waiting requests in arrival order */
    while (started != seen) {
      const int ri = started % A.ring_size;
      const int G = __ldcg(&A.dreq[ri].groups);
      if (!wgm_warp_lock(L, &st->pool_lock)) return false;
      const int avail = wgm_bcast(lane == 0 ? wgm_ld_acquire_gpu(&st->available_workgroups) : 0);
      if (avail < G) {
        if (lane == 0) {
          int tk = wgm_ld_relaxed_gpu(&st->groups_to_kill);
          if (tk < G - avail) {
            wgm_st_release_gpu(&st->groups_to_kill, G - avail);
            /* the job's next barrier resizes */
            atomicAdd(&sd->arrive, WGM_SERVE_RESIZE_FLAG);
          }
          wgm_unlock(&st->pool_lock);
        }
        __syncwarp();
        break;
      }
      const int got = wgm_pool_claim(sd, nslots, G, s_claim);
      if (got < G) {
        /* a bit not yet visible although counted: give the claims back, retry */
        for (int k = lane; k < got; k += 32)
          atomicOr(&sd->free_bits[s_claim[k] >> 5], 1 << (s_claim[k] & 31));
        __syncwarp();
        if (lane == 0) wgm_unlock(&st->pool_lock);
        __syncwarp();
        break;
      }
      if (lane == 0) {
        int *ctl = (int *)(A.arena + __ldcg(&A.dreq[ri].state_off));
        /* first 8 bytes of every line: the team Lonestar run keeps 64-bit
         * level words there */
        for (int l = 0; l < WGM_REQ_CTL_LINES; l++) {
          ctl[l * WGM_LINE] = 0;
          ctl[l * WGM_LINE + 1] = 0;
        }
        ctl[5 * WGM_LINE] = INT_MAX; /* reduce result */
        const int id = __ldcg(&A.dreq[ri].id);
        if (A.rtimes && id < A.max_requests) A.rtimes[2 * (size_t)id] = wgm_globaltimer();
        __threadfence();
      }
      __syncwarp();
      wgm_assign(L, A, got, s_claim, WGM_TASK_REQ, ri, 0, rc);
      if (lane == 0) {
        atomicAdd(&st->available_workgroups, -got);
        if (atomicAdd(&sd->pending, -1) == 1) wgm_st_relaxed_gpu(&st->groups_to_kill, 0);
        wgm_unlock(&st->pool_lock);
        wgm_st_relaxed_sys(&A.hs->started, started + 1);
      }
      started++;
      progress = true;
    }
    /* free groups the job could take back: ask for a resizing barrier, at
     * most once per barrier generation */
    if (lane == 0 && started == seen &&
        wgm_ld_acquire_gpu(&st->k_executing[1][0]) > 0 &&
        wgm_ld_acquire_gpu(&st->k_executing[1][0]) < A.persist_max &&
        wgm_ld_acquire_gpu(&st->available_workgroups) - A.reserve >= WGM_SERVE_FORK_MIN) {
      const unsigned gen = (unsigned)wgm_ld_acquire_gpu_u64(&sd->gate);
      if (gen != fork_gen) {
        fork_gen = gen;
        atomicAdd(&sd->arrive, WGM_SERVE_RESIZE_FLAG);
      }
    }
    /* end: host done, every request finished, the persistent job left */
    int fin = 0;
    if (lane == 0)
      fin = wgm_ld_acquire_sys(&A.hs->quit) != 0 && started == seen &&
            wgm_ld_acquire_sys(&A.hs->head) == seen &&
            wgm_ld_acquire_gpu(&sd->completed) == started &&
            wgm_ld_acquire_gpu(&st->k_executing[1][0]) == 0 &&
            wgm_ld_acquire_gpu(&st->available_workgroups) == lpg;
    if (wgm_bcast(fin)) {
      if (!wgm_warp_lock(L, &st->pool_lock)) return false;
      for (int done = 0; done < lpg;) {
        const int got = wgm_pool_claim(sd, nslots, min(lpg - done, WGM_SERVE_FORK_MAX), s_claim);
        if (got == 0) break;
        wgm_assign(L, A, got, s_claim, WGM_TASK_QUIT, 0, 0, rc);
        if (lane == 0) atomicAdd(&st->available_workgroups, -got);
        done += got;
      }
      if (lane == 0) wgm_unlock(&st->pool_lock);
      return true;
    }
    if (progress) {
      idle = wgm_idle_start(L, A.idle_ns);
    } else {
      int give = 0;
      if (lane == 0) give = wgm_spin_giveup(L, idle, WGM_SITE_SCHEDULER) ? 1 : 0;
      if (wgm_bcast(give)) return false;
    }
  }
}

/* ---- the kernel ----------------------------------------------------------- */

/* Read a request descriptor the scheduler copied (L2, never a stale L1 line:
 * ring entries are reused). */
__device__ __forceinline__ wgm_req wgm_load_req(const wgm_req *p) {
  wgm_req r;
  const int *s = reinterpret_cast<const int *>(p);
  int *d = reinterpret_cast<int *>(&r);
#pragma unroll
  for (int k = 0; k < (int)(sizeof(wgm_req) / 4); k++) d[k] = __ldcg(s + k);
  return r;
}

#endif
