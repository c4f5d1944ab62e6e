/*
 * Device runtime of the cooperative-kernel framework for sm_103a.
 *
 * GB300 counterpart of the reference's scheduler_rt/rt_device:
 *   ticket_lock.cl:5-26      -> wgm_tl_lock / wgm_tl_unlock
 *   discovery.cl:10-72       -> wgm_discover (ticket or reference mode)
 *   iw_barrier.cl:63-109     -> wgm_barrier_xf (master/slave flags)
 *   iw_barrier.cl:315-351    -> wgm_barrier_sense (counter + generation)
 *                               and wgm_barrier_tree (two-level counters)
 * Memory-order choices: every cross-CTA hand-off is an explicit .gpu-scope
 * release (writer) / acquire (reader) pair; host-visible words use .sys scope.
 * Every wait is bounded by a %globaltimer deadline and by the device error
 * word, so a lost CTA turns into a recorded WGM_DEV_TIMEOUT, never a hang.
 */
#ifndef WGM_DEVICE_CUH
#define WGM_DEVICE_CUH

#include <stdint.h>

#include "wgm_common.h"

/* ------------------------------------------------------------------------ */
/* Scoped memory operations                                                  */
/* ------------------------------------------------------------------------ */

__device__ __forceinline__ int wgm_ld_acquire_gpu(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int wgm_ld_relaxed_gpu(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void wgm_st_release_gpu(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void wgm_st_relaxed_gpu(int *p, int v) {
  asm volatile("st.relaxed.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int wgm_atom_add_acqrel_gpu(int *p, int v) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;"
               : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ int wgm_atom_add_relaxed_gpu(int *p, int v) {
  int old;
  asm volatile("atom.relaxed.gpu.global.add.s32 %0, [%1], %2;"
               : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ int wgm_atom_or_acqrel_gpu(int *p, int v) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.or.b32 %0, [%1], %2;"
               : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ int wgm_atom_exch_acquire_gpu(int *p, int v) {
  int old;
  asm volatile("atom.acquire.gpu.global.exch.b32 %0, [%1], %2;"
               : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ int wgm_atom_cas_acqrel_gpu(int *p, int cmp, int v) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.cas.b32 %0, [%1], %2, %3;"
               : "=r"(old) : "l"(p), "r"(cmp), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ void wgm_red_add_release_gpu(int *p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void wgm_fence_acqrel_gpu() {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
}
/* System scope: words in mapped pinned host memory. */
__device__ __forceinline__ int wgm_ld_acquire_sys(const int *p) {
  int v;
  asm volatile("ld.acquire.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int wgm_ld_relaxed_sys(const int *p) {
  int v;
  asm volatile("ld.relaxed.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void wgm_st_release_sys(int *p, int v) {
  asm volatile("st.release.sys.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void wgm_st_relaxed_sys(int *p, int v) {
  asm volatile("st.relaxed.sys.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int wgm_atom_add_acqrel_sys(int *p, int v) {
  int old;
  asm volatile("atom.acq_rel.sys.global.add.s32 %0, [%1], %2;"
               : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ int wgm_atom_cas_acqrel_sys(int *p, int cmp, int v) {
  int old;
  asm volatile("atom.acq_rel.sys.global.cas.b32 %0, [%1], %2, %3;"
               : "=r"(old) : "l"(p), "r"(cmp), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ unsigned long long wgm_globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int wgm_smid() {
  unsigned s;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(s));
  return (int)s;
}

/* ------------------------------------------------------------------------ */
/* Launch parameters and per-CTA state                                        */
/* ------------------------------------------------------------------------ */

struct wgm_launch {
  wgm_dev_state *st;
  wgm_host_flags *hf; /* device alias of the mapped host flags */
  unsigned long long spin_ns;
  unsigned long long window_ns; /* discovery closing window */
  int gen;          /* launch generation (selects discovery slot gen&1) */
  int expected;     /* ticket discovery closes once this many arrived */
  int disc_mode;    /* WGM_DISCOVERY_* */
  int extra_rounds; /* reference discovery: lock rounds before closing */
  int im_exit;      /* occupancy-only launch */
  int barrier_kind; /* WGM_BARRIER_* */
  int handshake;    /* standalone host handshake (standalone.cl:277-289) */
  int tree_fanin;   /* groups per leaf of the tree barrier */
};

struct wgm_cta {
  int id;      /* discovered group id (p_get_group_id) */
  int ngroups; /* discovered groups (p_get_num_groups) */
  int gen;     /* barrier generation this CTA will complete next */
  int ok;      /* cleared when a wait gave up */
  int tmp[4];
};

/* Record the first failure of this launch, device side and host side. */
static __device__ __noinline__ void wgm_fail(const wgm_launch &L, int code, int site,
                                      int detail) {
  if (atomicCAS(&L.st->dev_error, 0, code) == 0) {
    wgm_st_relaxed_sys(&L.hf->status_site, site);
    wgm_st_relaxed_sys(&L.hf->status_detail, detail);
    wgm_st_release_sys(&L.hf->status, code);
  }
}

struct wgm_spin {
  unsigned long long deadline;
  unsigned n;
};
__device__ __forceinline__ wgm_spin wgm_spin_start(const wgm_launch &L) {
  wgm_spin s;
  s.deadline = wgm_globaltimer() + L.spin_ns;
  s.n = 0;
  return s;
}
/* True when the wait must be abandoned: a deadline passed, the host raised
 * abort_flag, or another CTA already failed. */
__device__ __forceinline__ bool wgm_spin_giveup(const wgm_launch &L, wgm_spin &s,
                                                int site) {
  ++s.n;
  if ((s.n & 31u) != 0) return false;
  if (wgm_ld_relaxed_gpu(&L.st->dev_error) != 0) return true;
  if ((s.n & 2047u) == 0 && wgm_ld_relaxed_sys(&L.hf->abort_flag) != 0) {
    wgm_fail(L, WGM_DEV_ABORTED, site, 0);
    return true;
  }
  if (wgm_globaltimer() > s.deadline) {
    wgm_fail(L, WGM_DEV_TIMEOUT, site, (int)blockIdx.x);
    return true;
  }
  if (s.n > 4096u) __nanosleep(64);
  return false;
}

/* ------------------------------------------------------------------------ */
/* Ticket lock (ticket_lock.cl:5-26), bounded                                */
/* ------------------------------------------------------------------------ */

__device__ __forceinline__ bool wgm_tl_lock(const wgm_launch &L) {
  int ticket = wgm_atom_add_acqrel_gpu(&L.st->tl_counter, 1);
  wgm_spin s = wgm_spin_start(L);
  while (wgm_ld_acquire_gpu(&L.st->tl_now_serving) != ticket) {
    if (wgm_spin_giveup(L, s, WGM_SITE_TICKET_LOCK)) return false;
  }
  return true;
}
__device__ __forceinline__ void wgm_tl_unlock(const wgm_launch &L) {
  int t = wgm_ld_relaxed_gpu(&L.st->tl_now_serving);
  wgm_st_release_gpu(&L.st->tl_now_serving, t + 1);
}

/* ------------------------------------------------------------------------ */
/* Occupancy discovery                                                       */
/* ------------------------------------------------------------------------ */

/* Ticket mode (the GB300 protocol).  Each CTA takes one ticket with a
 * fetch-add on the poll word of its launch generation; a ticket taken after
 * the CLOSED bit was set means "not co-resident in time", the CTA leaves.
 * Ticket 0 closes the poll once `expected` tickets are out or the closing
 * window has passed since it arrived, publishes the count and clears the
 * other generation's slot for the next launch.  One atomic per CTA replaces
 * the reference's 12 serialised ticket-lock rounds per CTA, which on a GB300
 * with >1000 CTAs would cost milliseconds. */
__device__ __forceinline__ bool wgm_discover_ticket(const wgm_launch &L, int *id,
                                                    int *n) {
  const int slot = L.gen & 1;
  int t = wgm_atom_add_acqrel_gpu(&L.st->poll_word[slot], 1);
  if (t & WGM_POLL_CLOSED) return false;
  *id = t;
  if (t == 0) {
    unsigned long long close_at = wgm_globaltimer() + L.window_ns;
    wgm_spin s = wgm_spin_start(L);
    while ((wgm_ld_relaxed_gpu(&L.st->poll_word[slot]) & (WGM_POLL_CLOSED - 1)) <
               L.expected &&
           wgm_globaltimer() < close_at) {
      if (wgm_spin_giveup(L, s, WGM_SITE_DISCOVERY)) break;
    }
    int old = wgm_atom_or_acqrel_gpu(&L.st->poll_word[slot], WGM_POLL_CLOSED);
    int cnt = old & (WGM_POLL_CLOSED - 1);
    wgm_st_relaxed_gpu(&L.st->poll_word[slot ^ 1], 0);
    wgm_st_relaxed_gpu(&L.st->bar_arrivals[(slot ^ 1) * WGM_LINE], 0);
    wgm_st_relaxed_gpu(&L.st->count[slot], cnt);
    wgm_st_release_gpu(&L.st->published, L.gen);
    *n = cnt;
    return true;
  }
  wgm_spin s = wgm_spin_start(L);
  while (wgm_ld_acquire_gpu(&L.st->published) != L.gen) {
    if (wgm_spin_giveup(L, s, WGM_SITE_DISCOVERY)) return false;
  }
  *n = wgm_ld_relaxed_gpu(&L.st->count[slot]);
  return true;
}

/* Reference mode: discovery_protocol_rep (discovery.cl:26-57) with bounded
 * waits.  Poll: under the ticket lock, take id = count++ if the poll is open;
 * then `extra_rounds` lock/unlock rounds; then close the poll. */
__device__ __forceinline__ bool wgm_discover_reference(const wgm_launch &L, int *id,
                                                       int *n) {
  const int slot = L.gen & 1;
  if (!wgm_tl_lock(L)) return false;
  bool open = wgm_ld_relaxed_gpu(&L.st->closed_gen) != L.gen;
  if (open) {
    *id = wgm_ld_relaxed_gpu(&L.st->count[slot]);
    if (*id == 0) {
      wgm_st_relaxed_gpu(&L.st->count[slot ^ 1], 0);
      wgm_st_relaxed_gpu(&L.st->bar_arrivals[(slot ^ 1) * WGM_LINE], 0);
    }
    wgm_st_relaxed_gpu(&L.st->count[slot], *id + 1);
  }
  wgm_tl_unlock(L);
  if (!open) return false;
  for (int i = 0; i < L.extra_rounds; i++) {
    if (!wgm_tl_lock(L)) return false;
    wgm_tl_unlock(L);
  }
  if (!wgm_tl_lock(L)) return false;
  if (wgm_ld_relaxed_gpu(&L.st->closed_gen) != L.gen) {
    wgm_st_relaxed_gpu(&L.st->closed_gen, L.gen);
    wgm_st_release_gpu(&L.st->published, L.gen);
  }
  wgm_tl_unlock(L);
  *n = wgm_ld_acquire_gpu(&L.st->count[slot]);
  return true;
}

/* DISCOVERY_PROTOCOL (discovery.cl:59-72): returns false for CTAs that must
 * leave (not discovered, occupancy-only launch, or a wait gave up). */
__device__ __forceinline__ bool wgm_discover(const wgm_launch &L, wgm_cta *c) {
  if (threadIdx.x == 0) {
    int id = -1, n = 0;
    bool part = (L.disc_mode == WGM_DISCOVERY_REFERENCE)
                    ? wgm_discover_reference(L, &id, &n)
                    : wgm_discover_ticket(L, &id, &n);
    c->id = id;
    c->ngroups = n;
    c->ok = part ? 1 : 0;
    if (part) {
      L.st->p_group_ids[blockIdx.x] = id;
      L.st->group_smid[id] = wgm_smid();
      if (id == 0) wgm_st_relaxed_sys(&L.hf->discovered, n);
    }
    /* Generation of the next barrier, read before this CTA's first arrival
     * (no barrier can complete before every CTA has arrived). */
    c->gen = wgm_ld_relaxed_gpu(&L.st->bar_gen);
    c->tmp[0] = 0;
    c->tmp[2] = 0; /* counting barrier: arrivals expected so far */
  }
  __syncthreads();
  if (!c->ok) return false;
  if (L.im_exit) return false;
  /* Discovered ids are dense but ngroups may still be unpublished for ids
   * >= count when a wait gave up; never run with an out-of-range id. */
  if (c->id >= c->ngroups || c->ngroups > WGM_MAX_GROUPS) return false;
  return true;
}

/* ------------------------------------------------------------------------ */
/* Inter-CTA barriers                                                        */
/* ------------------------------------------------------------------------ */

/* Sense-reversal barrier with a generation word: one acq_rel fetch-add per
 * CTA; the last arriver resets the counter and releases the generation. */
__device__ __forceinline__ bool wgm_barrier_sense(const wgm_launch &L, wgm_cta *c,
                                                  int ngroups) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int g = c->gen;
    int arrived = wgm_atom_add_acqrel_gpu(&L.st->bar_count, 1) + 1;
    if (arrived == ngroups) {
      wgm_st_relaxed_gpu(&L.st->bar_count, 0);
      wgm_st_release_gpu(&L.st->bar_gen, g + 1);
    } else {
      /* the deadline clock starts only once the wait has polled a while:
       * most barriers complete within a few polls */
      unsigned quick = 0;
      while (wgm_ld_acquire_gpu(&L.st->bar_gen) == g && ++quick < 64) {
      }
      if (quick >= 64) {
        wgm_spin s = wgm_spin_start(L);
        while (wgm_ld_acquire_gpu(&L.st->bar_gen) == g) {
          if (wgm_spin_giveup(L, s, WGM_SITE_BARRIER)) {
            c->ok = 0;
            break;
          }
        }
      }
    }
    c->gen = g + 1;
  }
  __syncthreads();
  return c->ok;
}

/* Counting barrier.  The launch's arrival counter (zeroed by the previous
 * launch's discovery closer, so it starts at 0) only grows: barrier k of the
 * launch completes when it reaches (k+1)*ngroups.  An arrival is one
 * fire-and-forget red.release (this CTA's writes before the barrier are
 * published by it); the waiters poll the counter itself with ld.acquire
 * (a relaxed poll plus a trailing fence is slower on GB300), so
 * the last arriver needs neither a returned value nor a second store - one
 * L2 hop shorter than the generation barrier.  Differences are taken modulo
 * 2^32, which keeps the test right across wrap-around. */
__device__ __forceinline__ bool wgm_barrier_count(const wgm_launch &L, wgm_cta *c,
                                                  int ngroups) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int *ctr = &L.st->bar_arrivals[(L.gen & 1) * WGM_LINE];
    const unsigned target = (unsigned)c->tmp[2] + (unsigned)ngroups;
    c->tmp[2] = (int)target;
    wgm_red_add_release_gpu(ctr, 1);
    wgm_spin s = wgm_spin_start(L);
    while ((int)((unsigned)wgm_ld_acquire_gpu(ctr) - target) < 0) {
      if (wgm_spin_giveup(L, s, WGM_SITE_BARRIER)) {
        c->ok = 0;
        break;
      }
    }
  }
  __syncthreads();
  return c->ok;
}

/* Spread barrier: the sense barrier's counter, but the last arriver releases
 * the new generation on 16 lines and CTA i polls line i % 16, so no line has
 * more than ngroups/16 pollers queued on it.  Arrival is the sense
 * barrier's acq_rel fetch-add; waiters poll their line with ld.acquire. */
__device__ __forceinline__ bool wgm_barrier_spread(const wgm_launch &L, wgm_cta *c,
                                                   int ngroups) {
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int g = c->gen;
    int last = 0;
    if (lane == 0) last = wgm_atom_add_acqrel_gpu(&L.st->bar_count, 1) + 1 == ngroups;
    last = __shfl_sync(0xffffffffu, last, 0);
    if (last) {
      if (lane == 0) {
        wgm_st_relaxed_gpu(&L.st->bar_count, 0);
        wgm_st_release_gpu(&L.st->bar_gen, g + 1);
      }
      __syncwarp();
      if (lane < 16) wgm_st_release_gpu(&L.st->bar_gen_spread[lane * WGM_LINE], g + 1);
    } else if (lane == 0) {
      const int *line = &L.st->bar_gen_spread[(c->id & 15) * WGM_LINE];
      wgm_spin s = wgm_spin_start(L);
      while ((int)((unsigned)wgm_ld_acquire_gpu(line) - (unsigned)(g + 1)) < 0) {
        if (wgm_spin_giveup(L, s, WGM_SITE_BARRIER)) {
          c->ok = 0;
          break;
        }
      }
    }
    if (lane == 0) c->gen = g + 1;
  }
  __syncthreads();
  return c->ok;
}

/* Two-level barrier: groups arrive on a per-leaf counter (tree_fanin groups
 * per leaf, each leaf on its own line); the last of a leaf arrives at the
 * root; the last at the root releases the generation every CTA polls. */
__device__ __forceinline__ bool wgm_barrier_tree(const wgm_launch &L, wgm_cta *c,
                                                 int ngroups) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int g = c->gen;
    /* At most 128 leaves (tree_count has 128 lines). */
    int fan = max(max(L.tree_fanin, 1), (ngroups + 127) / 128);
    int leaf = c->id / fan;
    int nleaves = (ngroups + fan - 1) / fan;
    int leaf_size = min(fan, ngroups - leaf * fan);
    int *lc = &L.st->tree_count[leaf * WGM_LINE];
    bool released = false;
    if (wgm_atom_add_acqrel_gpu(lc, 1) + 1 == leaf_size) {
      wgm_st_relaxed_gpu(lc, 0);
      if (wgm_atom_add_acqrel_gpu(&L.st->bar_count, 1) + 1 == nleaves) {
        wgm_st_relaxed_gpu(&L.st->bar_count, 0);
        wgm_st_release_gpu(&L.st->bar_gen, g + 1);
        released = true;
      }
    }
    if (!released) {
      wgm_spin s = wgm_spin_start(L);
      while (wgm_ld_acquire_gpu(&L.st->bar_gen) == g) {
        if (wgm_spin_giveup(L, s, WGM_SITE_BARRIER)) {
          c->ok = 0;
          break;
        }
      }
    }
    c->gen = g + 1;
  }
  __syncthreads();
  return c->ok;
}

/* XF master/slave barrier (iw_barrier.cl:63-109, global_barrier_disc). */
__device__ __forceinline__ bool wgm_barrier_xf(const wgm_launch &L, wgm_cta *c,
                                               int ngroups) {
  int *flags = L.st->xf_flags;
  if (c->id == 0) {
    for (int peer = threadIdx.x + 1; peer < ngroups; peer += blockDim.x) {
      wgm_spin s = wgm_spin_start(L);
      while (wgm_ld_acquire_gpu(&flags[peer]) == 0) {
        if (wgm_spin_giveup(L, s, WGM_SITE_XF_BARRIER)) {
          c->ok = 0;
          break;
        }
      }
    }
    __syncthreads();
    for (int peer = threadIdx.x + 1; peer < ngroups; peer += blockDim.x)
      wgm_st_release_gpu(&flags[peer], 0);
  } else {
    __syncthreads();
    if (threadIdx.x == 0) {
      wgm_st_release_gpu(&flags[c->id], 1);
      wgm_spin s = wgm_spin_start(L);
      while (wgm_ld_acquire_gpu(&flags[c->id]) == 1) {
        if (wgm_spin_giveup(L, s, WGM_SITE_XF_BARRIER)) {
          c->ok = 0;
          break;
        }
      }
    }
  }
  __syncthreads();
  return c->ok && wgm_ld_relaxed_gpu(&L.st->dev_error) == 0;
}

__device__ __forceinline__ bool wgm_barrier(const wgm_launch &L, wgm_cta *c) {
  /* Every 1024 barriers each CTA looks at the host abort word once (a few
   * ms of barriers), so a run the host gives up on ends soon even when no
   * wait spins long (the other CTAs then see dev_error in their next wait). */
  if (threadIdx.x == 0 && ((++c->tmp[0]) & 1023) == 0 &&
      wgm_ld_relaxed_sys(&L.hf->abort_flag) != 0) {
    wgm_fail(L, WGM_DEV_ABORTED, WGM_SITE_BARRIER, c->id);
    c->ok = 0;
  }
  switch (L.barrier_kind) {
    case WGM_BARRIER_XF:
      return wgm_barrier_xf(L, c, c->ngroups);
    case WGM_BARRIER_TREE:
      return wgm_barrier_tree(L, c, c->ngroups);
    case WGM_BARRIER_COUNT:
      return wgm_barrier_count(L, c, c->ngroups);
    case WGM_BARRIER_SPREAD:
      return wgm_barrier_spread(L, c, c->ngroups);
    case WGM_BARRIER_AUTO:
      if (c->ngroups <= WGM_BARRIER_AUTO_COUNT_MAX) return wgm_barrier_count(L, c, c->ngroups);
      return wgm_barrier_sense(L, c, c->ngroups);
    default:
      return wgm_barrier_sense(L, c, c->ngroups);
  }
}

/* Standalone host handshake (lonestar/graph_apps/bfs/device/standalone.cl:
 * 277-289): discovered group 0 publishes persistent_flag = count and
 * DEVICE_WAITING, then waits for DEVICE_TO_PERSISTENT_TASK; a barrier lets
 * everyone start together. */
__device__ __forceinline__ bool wgm_standalone_handshake(const wgm_launch &L,
                                                         wgm_cta *c) {
  if (c->id == 0 && threadIdx.x == 0) {
    wgm_st_release_sys(&L.hf->persistent_flag, c->ngroups);
    wgm_st_release_sys(&L.hf->scheduler_flag, WGM_DEVICE_WAITING);
    wgm_spin s = wgm_spin_start(L);
    while (wgm_ld_acquire_sys(&L.hf->scheduler_flag) != WGM_DEVICE_TO_PERSISTENT_TASK) {
      if (wgm_spin_giveup(L, s, WGM_SITE_HANDSHAKE)) {
        c->ok = 0;
        break;
      }
    }
  }
  return wgm_barrier(L, c);
}

/* End of a standalone persistent kernel (standalone.cl:316-319). */
__device__ __forceinline__ void wgm_standalone_exit(const wgm_launch &L) {
  __syncthreads();
  if (threadIdx.x == 0) wgm_atom_add_acqrel_sys(&L.hf->persistent_flag, -1);
}

/* ------------------------------------------------------------------------ */
/* Warp utilities                                                            */
/* ------------------------------------------------------------------------ */

#define WGM_FULL 0xffffffffu

__device__ __forceinline__ int wgm_lane() { return (int)(threadIdx.x & 31); }
__device__ __forceinline__ unsigned wgm_lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
__device__ __forceinline__ int wgm_warp_incl_scan(int x) {
  int lane = wgm_lane();
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(WGM_FULL, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

/* Warp-aggregated push of one item per flagged lane onto a worklist segment
 * (one atomic per warp: __ballot_sync/__popc/__shfl_sync).  `back` lists grow
 * downwards from base[cap-1].  Returns false on overflow (item dropped). */
__device__ __forceinline__ bool wgm_warp_push(bool flag, int item, int *counter,
                                              int *base, int cap, bool back) {
  unsigned m = __ballot_sync(WGM_FULL, flag);
  if (m == 0) return true;
  int leader = __ffs(m) - 1;
  int start = 0;
  if (wgm_lane() == leader) start = atomicAdd(counter, __popc(m));
  start = __shfl_sync(WGM_FULL, start, leader);
  if (flag) {
    int pos = start + __popc(m & wgm_lanemask_lt());
    if (pos >= cap) return false;
    if (back)
      base[cap - 1 - pos] = item;
    else
      base[pos] = item;
  }
  return true;
}

#endif
