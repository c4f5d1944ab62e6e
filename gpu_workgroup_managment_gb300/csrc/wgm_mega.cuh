/*
 * The hand-written megakernel: one persistent launch in which discovered
 * group 0 runs the device-side scheduler and every other group loops
 * "announce free -> get a task -> run it", where a task is either a slice of
 * the resident persistent app (resizable at every barrier) or a
 * non-persistent task.
 *
 * GB300 counterparts of the reference (paths relative to the reference):
 *   src/scheduler_rt/rt_device/main_device_body.cl:1-93  -> wgm_k_mega worker loop
 *   src/scheduler_rt/rt_device/cl_scheduler.cl:168-308  -> wgm_get_task, wgm_scheduler_loop
 *   src/scheduler_rt/rt_device/scheduler_1.cl:10-135    -> wgm_offer_fork, wgm_offer_kill,
 *                                                          the two task-assignment loops
 *   src/scheduler_rt/rt_device/iw_barrier.cl:165-305    -> wgm_resize_barrier (and the
 *                                                          query variant)
 *   src/non_persistent_kernels/{matmult,reduce}/device  -> wgm_np_* tasks
 * The host drives the scheduler through the mapped wgm_host_flags words with
 * the reference's state machine (DEVICE_WAITING, DEVICE_TO_TASK, ...).
 */
#ifndef WGM_MEGA_CUH
#define WGM_MEGA_CUH

#include "wgm_graph.cuh"
#include "wgm_octree.cuh"
#include "wgm_c4.cuh"
#include "wgm_protocol.h"

/* Non-persistent task kinds. */
#define WGM_NP_MATMULT_I32 1 /* matmult.cl: int32 C = A*B, djb2 hash of the diagonal */
#define WGM_NP_REDUCE_I32 2  /* reduce.cl: int32 min */
#define WGM_NP_MATMULT_F32 3 /* FP32 C = A*B */
#define WGM_NP_REDUCE_F32 4  /* FP32 min (non-negative inputs) */

struct wgm_np_args {
  int kind;
  int n;           /* matmult: n x n matrices */
  const int *A, *B;
  int *C;
  const float *Af, *Bf;
  float *Cf;
  int *hash;       /* matmult.cl:64 result word */
  const int *buf;  /* reduce input */
  const float *buff;
  int len;
  int *result;     /* reduce result (int bits for FP32) */
};

/* Persistent app hosted by the megakernel. */
struct wgm_mega_args {
  int app; /* WGM_K_* of the persistent app */
  wgm_lonestar_args ls;
  wgm_color_args color;
  wgm_mis_args mis;
  wgm_psssp_args psssp;
  wgm_pr_args pr;
  wgm_bc_args bc;
  wgm_octree_args oct;
  wgm_c4_args c4;
  wgm_np_args np;
  unsigned long long idle_ns; /* budget of host-driven waits */
  int use_query_barrier;
};

/* Restoration record layout (wgm_rctx.w). */
#define WGM_RC_TARGET 0
#define WGM_RC_ROUND 1
#define WGM_RC_GEN 2     /* barrier generation the group completes next */
#define WGM_RC_NGROUPS 3 /* persistent group count after the fork */

/* A long wait that the host paces (the scheduler's flag polls, idle groups
 * waiting for a task): deadline idle_ns, same abort/error checks. */
__device__ __forceinline__ wgm_spin wgm_idle_start(const wgm_launch &L,
                                                   unsigned long long idle_ns) {
  wgm_spin s;
  s.deadline = wgm_globaltimer() + idle_ns;
  s.n = 0;
  return s;
}

__device__ __forceinline__ bool wgm_try_lock(int *m) {
  return wgm_atom_exch_acquire_gpu(m, 1) == 0; /* cl_scheduler.cl:145-147 */
}
__device__ __forceinline__ void wgm_unlock(int *m) { wgm_st_release_gpu(m, 0); }
__device__ __forceinline__ bool wgm_lock(const wgm_launch &L, int *m, int site) {
  wgm_spin s = wgm_spin_start(L);
  while (!wgm_try_lock(m)) {
    if (wgm_spin_giveup(L, s, site)) return false;
  }
  return true;
}

/* ------------------------------------------------------------------------ */
/* Non-persistent tasks (run by the groups the scheduler assigned)            */
/* ------------------------------------------------------------------------ */

/* matmult (matmult.cl:26-67): grid-stride over C, then the last group to
 * finish hashes the diagonal (djb2, wrapping int32).  FP32 variant without
 * the hash.  kid/kn: this group's id and the task's group count. */
static __device__ void wgm_np_matmult(const wgm_launch &L, const wgm_np_args &a, int kid, int kn) {
  const int n = a.n;
  const int gid = kid * blockDim.x + threadIdx.x, nth = kn * blockDim.x;
  if (a.kind == WGM_NP_MATMULT_I32) {
    for (int i = gid; i < n * n; i += nth) {
      int r = i / n, c = i % n;
      unsigned acc = 0;
      for (int j = 0; j < n; j++)
        acc += (unsigned)__ldg(&a.A[r * n + j]) * (unsigned)__ldg(&a.B[j * n + c]);
      a.C[i] = (int)acc;
    }
  } else {
    for (int i = gid; i < n * n; i += nth) {
      int r = i / n, c = i % n;
      float acc = 0.f;
      for (int j = 0; j < n; j++) acc = fmaf(__ldg(&a.Af[r * n + j]), __ldg(&a.Bf[j * n + c]), acc);
      a.Cf[i] = acc;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && a.kind == WGM_NP_MATMULT_I32) {
    int finished = wgm_atom_add_acqrel_gpu(&L.st->np_counter, 1);
    if (finished == kn - 1) {
      unsigned h = 5381;
      for (int i = 0; i < n; i++) h = h * 33u + (unsigned)__ldcg(&a.C[i * n + i]);
      wgm_st_release_sys(a.hash, (int)h); /* host-visible word */
    }
  }
}

/* MY_reduce (reduce.cl:3-39): block min, then one atomic per group. */
static __device__ void wgm_np_reduce(const wgm_np_args &a, int kid, int kn) {
  __shared__ int red[32];
  const int gid = kid * blockDim.x + threadIdx.x, nth = kn * blockDim.x;
  int m = INT_MAX;
  if (a.kind == WGM_NP_REDUCE_I32) {
    for (int i = gid; i < a.len; i += nth) m = min(m, __ldg(&a.buf[i]));
  } else {
    for (int i = gid; i < a.len; i += nth) m = min(m, __float_as_int(__ldg(&a.buff[i])));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(WGM_FULL, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    int v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : INT_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(WGM_FULL, v, o));
    if (threadIdx.x == 0) atomicMin_system(a.result, v); /* host-visible word */
  }
  __syncthreads();
}

/* ------------------------------------------------------------------------ */
/* offer_kill / offer_fork and the resizing barrier                           */
/* ------------------------------------------------------------------------ */

/* The protocol steps of wgm_protocol.h on the GPU: gpu-scope acquire loads
 * and acq_rel read-modify-writes. */
struct wgm_gpu_ops {
  static __device__ __forceinline__ int ld_acquire(int *p) { return wgm_ld_acquire_gpu(p); }
  static __device__ __forceinline__ int cas(int *p, int cmp, int v) {
    return wgm_atom_cas_acqrel_gpu(p, cmp, v);
  }
  static __device__ __forceinline__ int add(int *p, int v) { return wgm_atom_add_acqrel_gpu(p, v); }
  static __device__ __forceinline__ void between() {}
};

/* __offer_kill (scheduler_1.cl:59-81), thread 0 only: the group with the
 * highest persistent id leaves when the scheduler wants groups; being the
 * highest id is the lock, and the decrement of num_groups releases it.  The
 * decrement of groups_to_kill is a compare-and-swap, because the scheduler
 * may clear the word at any time (wgm_proto_offer_kill). */
__device__ __forceinline__ bool wgm_offer_kill(const wgm_launch &L, int kid) {
  return wgm_proto_offer_kill<wgm_gpu_ops>(&L.st->k_num_groups[1][0], &L.st->groups_to_kill,
                                           kid);
}

/* offer_fork (scheduler_1.cl:10-57), master thread 0 only, after every live
 * group arrived: take every free group, give each the restoration record
 * `rc` (the next phase, the barrier generation and the new group count),
 * then grow the persistent group count.  n < 0: read the group count under
 * the pool lock (a task loop without barriers that keeps kills out while it
 * forks). */
__device__ __forceinline__ int wgm_offer_fork(const wgm_launch &L, int n, wgm_rctx rc) {
  wgm_dev_state *st = L.st;
  if (wgm_ld_acquire_gpu(&st->available_workgroups) <= 0) return n;
  if (!wgm_try_lock(&st->pool_lock)) return n;
  if (n < 0) n = wgm_ld_acquire_gpu(&st->k_num_groups[1][0]);
  int snap = wgm_ld_acquire_gpu(&st->available_workgroups);
  int got = 0;
  rc.w[WGM_RC_NGROUPS] = n + snap;
  for (int i = n; i < n + snap; i++) {
    int slot = i + 1;
    if (slot >= WGM_MAX_GROUPS) break;
    /* "two phase check": available and task_array can be out of step */
    wgm_spin s = wgm_spin_start(L);
    bool ok = true;
    while (wgm_ld_acquire_gpu(&st->task_array[slot]) != WGM_TASK_WAIT) {
      if (wgm_spin_giveup(L, s, WGM_SITE_FORK)) {
        ok = false;
        break;
      }
    }
    if (!ok) break;
    st->k_group_ids[1][slot] = i;
    st->r_ctx_arr[slot] = rc;
    got++;
  }
  if (got > 0) {
    rc.w[WGM_RC_NGROUPS] = n + got;
    for (int i = n; i < n + got; i++) st->r_ctx_arr[i + 1].w[WGM_RC_NGROUPS] = n + got;
    /* grow the group count before the new groups can run */
    wgm_atom_add_acqrel_gpu(&st->k_num_groups[1][0], got);
    atomicAdd(&st->k_executing[1][0], got);
    wgm_atom_add_acqrel_sys(&L.hf->persistent_flag, got);
    atomicAdd(&st->available_workgroups, -got);
    for (int i = n; i < n + got; i++) wgm_st_release_gpu(&st->task_array[i + 1], WGM_TASK_PERSIST);
  }
  wgm_unlock(&st->pool_lock);
  return n + got;
}

/* global_barrier_resize (iw_barrier.cl:165-227) on a counter instead of the
 * reference's per-group flags.  A slave first offers to die; the master waits
 * until every live slave arrived (reading the arrival count before the group
 * count, so a concurrent kill can never make it leave early), resets the
 * count, offers the free groups a fork into the next phase and releases.
 * Returns 1 to continue, 0 if this group was killed, -1 on a failed wait.
 * Query variant (iw_barrier.cl:229-305): the master reads groups_to_kill and
 * the chosen highest ids leave after the release instead of on arrival. */
static __device__ int wgm_resize_barrier(const wgm_launch &L, wgm_cta *c, wgm_step nxt, bool query) {
  wgm_dev_state *st = L.st;
  int *kng = &st->k_num_groups[1][0];
  __syncthreads();
  if (threadIdx.x == 0) {
    const int g = c->gen;
    int res = 1;
    if (c->id != 0) {
      if (!query && wgm_offer_kill(L, c->id)) {
        res = 0;
      } else {
        wgm_atom_add_acqrel_gpu(&st->bar_count, 1);
        wgm_spin s = wgm_spin_start(L);
        /* Wait for generation g+1 or later, not for "anything but g": a group
         * forked at barrier g-1 starts its phase before the master releases
         * g, so it can arrive here while bar_gen still reads g-1. */
        while ((int)((unsigned)wgm_ld_acquire_gpu(&st->bar_gen) - (unsigned)(g + 1)) < 0) {
          if (wgm_spin_giveup(L, s, WGM_SITE_RESIZE_BARRIER)) {
            res = -1;
            break;
          }
        }
        if (res == 1 && query && c->id >= wgm_ld_acquire_gpu(&st->bar_num_groups)) res = 0;
      }
    } else {
      wgm_spin s = wgm_spin_start(L);
      for (;;) {
        int arrived = wgm_ld_acquire_gpu(&st->bar_count);
        int n = wgm_ld_acquire_gpu(kng);
        if (arrived == n - 1) break;
        if (wgm_spin_giveup(L, s, WGM_SITE_RESIZE_BARRIER)) {
          res = -1;
          break;
        }
      }
      if (res == 1) {
        wgm_st_relaxed_gpu(&st->bar_count, 0);
        int n = wgm_ld_acquire_gpu(kng);
        const int tk = query ? wgm_ld_acquire_gpu(&st->groups_to_kill) : 0;
        if (tk > 0) {
          /* query barrier: shrink by min(to_kill, n-1) from the top; no fork
           * while the scheduler wants groups */
          const int k = wgm_proto_take_kills<wgm_gpu_ops>(&st->groups_to_kill, n - 1);
          wgm_atom_add_acqrel_gpu(kng, -k);
          n -= k;
        } else {
          wgm_rctx rc;
          for (int k = 0; k < WGM_RCTX_WORDS; k++) rc.w[k] = 0;
          rc.w[WGM_RC_TARGET] = nxt.target;
          rc.w[WGM_RC_ROUND] = nxt.round;
          rc.w[WGM_RC_GEN] = g + 1;
          n = wgm_offer_fork(L, n, rc);
        }
        wgm_st_relaxed_gpu(&st->bar_num_groups, n);
        wgm_st_release_gpu(&st->bar_gen, g + 1);
      }
    }
    c->gen = g + 1;
    /* The group count of the next phase is the one the master published with
     * the release; num_groups itself can already be lower again, when a
     * group that finished the next phase early killed itself at the barrier
     * after it. */
    if (res == 1) c->ngroups = wgm_ld_acquire_gpu(&st->bar_num_groups);
    if (res == -1) c->ok = 0;
    c->tmp[1] = res;
  }
  __syncthreads();
  return c->tmp[1];
}

/* ------------------------------------------------------------------------ */
/* Device-side scheduler (discovered group 0, thread 0)                       */
/* ------------------------------------------------------------------------ */

/* Wait until the host sets the scheduler flag to one of the states the
 * scheduler acts on; returns -1 when the wait gives up. */
__device__ __forceinline__ int wgm_wait_flag(const wgm_launch &L, unsigned long long idle_ns,
                                             int want, int site) {
  wgm_spin s = wgm_idle_start(L, idle_ns);
  for (;;) {
    int f = wgm_ld_acquire_sys(&L.hf->scheduler_flag);
    if (want >= 0 ? (f == want)
                  : (f == WGM_DEVICE_TO_QUIT || f == WGM_DEVICE_TO_TASK ||
                     f == WGM_DEVICE_TO_PERSISTENT_TASK))
      return f;
    if (wgm_spin_giveup(L, s, site)) return -1;
  }
}

__device__ __forceinline__ bool wgm_wait_geq(const wgm_launch &L, unsigned long long ns,
                                             const int *p, int v, int site) {
  wgm_spin s = wgm_idle_start(L, ns);
  while (wgm_ld_acquire_gpu(p) < v) {
    if (wgm_spin_giveup(L, s, site)) return false;
  }
  return true;
}
__device__ __forceinline__ bool wgm_wait_eq(const wgm_launch &L, unsigned long long ns,
                                            const int *p, int v, int site) {
  wgm_spin s = wgm_idle_start(L, ns);
  while (wgm_ld_acquire_gpu(p) != v) {
    if (wgm_spin_giveup(L, s, site)) return false;
  }
  return true;
}

/* scheduler_init + scheduler_loop (cl_scheduler.cl:191-308) with the two
 * assignment loops of scheduler_1.cl:83-135.  lpg = participating groups
 * (discovered groups minus the scheduler's). */
static __device__ void wgm_scheduler(const wgm_launch &L, const wgm_mega_args &A, int lpg) {
  wgm_dev_state *st = L.st;
  const unsigned long long idle = A.idle_ns;
  wgm_st_relaxed_sys(&L.hf->participating_groups, lpg);
  wgm_st_relaxed_gpu(&st->pool_lock, 0);
  wgm_st_relaxed_gpu(&st->groups_to_kill, 0);
  wgm_st_relaxed_gpu(&st->k_executing[0][0], 0);
  wgm_st_relaxed_gpu(&st->k_executing[1][0], 0);
  wgm_st_release_sys(&L.hf->persistent_flag, 0);
  wgm_st_release_sys(&L.hf->scheduler_flag, WGM_DEVICE_WAITING);
  for (;;) {
    int flag = wgm_wait_flag(L, idle, -1, WGM_SITE_SCHEDULER);
    if (flag < 0) return;
    if (flag == WGM_DEVICE_TO_QUIT) {
      if (!wgm_wait_eq(L, idle, &st->k_executing[0][0], 0, WGM_SITE_SCHEDULER) ||
          !wgm_wait_eq(L, idle, &st->k_executing[1][0], 0, WGM_SITE_SCHEDULER) ||
          !wgm_lock(L, &st->pool_lock, WGM_SITE_SCHEDULER))
        return;
      for (int i = 1; i <= lpg; i++) {
        if (!wgm_wait_eq(L, L.spin_ns, &st->task_array[i], WGM_TASK_WAIT, WGM_SITE_SCHEDULER))
          break;
        wgm_st_release_gpu(&st->task_array[i], WGM_TASK_QUIT);
        atomicAdd(&st->available_workgroups, -1);
      }
      wgm_unlock(&st->pool_lock);
      return;
    }
    const int ts = wgm_ld_acquire_sys(&L.hf->task_size);
    if (flag == WGM_DEVICE_TO_TASK) {
      /* cl_scheduler.cl:239-269 */
      wgm_st_relaxed_gpu(&st->k_num_groups[0][0], ts);
      wgm_st_relaxed_gpu(&st->k_executing[0][0], ts);
      wgm_st_relaxed_gpu(&st->np_counter, 0);
      if (!wgm_lock(L, &st->pool_lock, WGM_SITE_SCHEDULER)) return;
      int to_kill = ts - wgm_ld_acquire_gpu(&st->available_workgroups);
      wgm_st_release_gpu(&st->groups_to_kill, to_kill);
      /* response time: the persistent groups leave at their next barrier */
      if (!wgm_wait_geq(L, idle, &st->available_workgroups, ts, WGM_SITE_SCHEDULER)) return;
      wgm_st_release_sys(&L.hf->scheduler_flag, WGM_DEVICE_GOT_GROUPS);
      if (wgm_wait_flag(L, idle, WGM_DEVICE_TO_EXECUTE, WGM_SITE_SCHEDULER) < 0) return;
      for (int i = 0; i < ts; i++) { /* scheduler_assign_tasks_graphics */
        int slot = lpg - i;
        st->k_group_ids[0][slot] = i;
        if (!wgm_wait_eq(L, L.spin_ns, &st->task_array[slot], WGM_TASK_WAIT, WGM_SITE_SCHEDULER))
          return;
        wgm_st_release_gpu(&st->task_array[slot], WGM_TASK_MULT);
        atomicAdd(&st->available_workgroups, -1);
      }
      wgm_unlock(&st->pool_lock);
      if (!wgm_wait_eq(L, idle, &st->k_executing[0][0], 0, WGM_SITE_SCHEDULER)) return;
      wgm_st_release_sys(&L.hf->scheduler_flag, WGM_DEVICE_WAITING);
    } else { /* WGM_DEVICE_TO_PERSISTENT_TASK, cl_scheduler.cl:273-306 */
      wgm_st_relaxed_gpu(&st->k_num_groups[1][0], ts);
      wgm_st_relaxed_gpu(&st->bar_num_groups, ts);
      wgm_st_relaxed_gpu(&st->k_executing[1][0], ts);
      wgm_st_relaxed_gpu(&st->groups_to_kill, 0);
      wgm_st_release_sys(&L.hf->persistent_flag, ts);
      if (!wgm_lock(L, &st->pool_lock, WGM_SITE_SCHEDULER)) return;
      if (!wgm_wait_geq(L, idle, &st->available_workgroups, ts, WGM_SITE_SCHEDULER)) return;
      wgm_st_release_sys(&L.hf->scheduler_flag, WGM_DEVICE_GOT_GROUPS);
      if (wgm_wait_flag(L, idle, WGM_DEVICE_TO_EXECUTE, WGM_SITE_SCHEDULER) < 0) return;
      const int g = wgm_ld_acquire_gpu(&st->bar_gen);
      for (int i = 0; i < ts; i++) { /* scheduler_assign_tasks_persistent */
        int slot = i + 1;
        st->k_group_ids[1][slot] = i;
        if (!wgm_wait_eq(L, L.spin_ns, &st->task_array[slot], WGM_TASK_WAIT, WGM_SITE_SCHEDULER))
          return;
        wgm_rctx rc;
        for (int k = 0; k < WGM_RCTX_WORDS; k++) rc.w[k] = 0;
        rc.w[WGM_RC_GEN] = g;
        rc.w[WGM_RC_NGROUPS] = ts;
        st->r_ctx_arr[slot] = rc;
        wgm_st_release_gpu(&st->task_array[slot], WGM_TASK_PERSIST);
        atomicAdd(&st->available_workgroups, -1);
      }
      wgm_unlock(&st->pool_lock);
      wgm_st_release_sys(&L.hf->scheduler_flag, WGM_DEVICE_WAITING);
    }
  }
}

#endif
