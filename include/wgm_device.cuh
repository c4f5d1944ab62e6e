/*
 * wgm_device.cuh - the device side of the GB300 cooperative-kernel runtime,
 * the header persistent apps are compiled against (with wgm.h,
 * wgm_common.h and wgm_protocol.h beside it; nvcc, sm_103a).  libwgm.so's
 * own kernels use it, and so can an app built outside the library and
 * registered with wgm_app_register (include/wgm.h).
 *
 * GB300 counterpart of the reference's scheduler_rt/rt_device and of the
 * kernel API its persistent kernels are written against:
 *   ticket_lock.cl:5-26      -> wgm_tl_lock / wgm_tl_unlock
 *   discovery.cl:10-72       -> wgm_discover (ticket or reference mode)
 *   iw_barrier.cl:63-109     -> wgm_barrier_xf (master/slave flags)
 *   iw_barrier.cl:315-351    -> wgm_barrier_sense (counter + generation)
 *                               and wgm_barrier_tree (two-level counters)
 *   iw_barrier.cl:165-305, scheduler_1.cl, cl_scheduler.cl,
 *   main_device_body.cl      -> the megakernel runtime (wgm_mega_body)
 *   kernel_merge/stubs/stubs.h:4-7 -> global_barrier, resizing_global_barrier,
 *                               offer_kill, offer_fork, wgm_group_id, ...
 *                               and the kernel templates wgm_app_kernel /
 *                               wgm_app_mega_kernel (end of this file)
 * Memory-order choices: every cross-CTA hand-off is an explicit .gpu-scope
 * release (writer) / acquire (reader) pair; host-visible words use .sys scope.
 * Every wait is bounded by a %globaltimer deadline and by the device error
 * word, so a lost CTA turns into a recorded WGM_DEV_TIMEOUT, never a hang.
 */
#ifndef WGM_DEVICE_CUH
#define WGM_DEVICE_CUH

#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

#include "wgm.h"
#include "wgm_common.h"
#include "wgm_protocol.h"

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

/* Thread-block clusters (launches with a cluster dimension). */
__device__ __forceinline__ unsigned wgm_cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned wgm_cluster_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
/* Every thread of every CTA of the cluster: the hardware cluster barrier
 * (release on arrival, acquire on the wait, cluster scope). */
__device__ __forceinline__ void wgm_cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
/* Store v into the same shared-memory word of the cluster's CTA `rank`. */
__device__ __forceinline__ void wgm_st_cluster_peer(int *smem_word, unsigned rank, int v) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(smem_word);
  unsigned ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(ra), "r"(v) : "memory");
}

/* Cluster barrier (WGM_BARRIER_CLUSTER; the launch has a cluster dimension
 * and every discovered CTA's cluster is whole).  The CTAs of a cluster meet
 * at the hardware cluster barrier; the cluster's rank-0 CTA alone takes part
 * in a counting barrier over the clusters (one red.release per cluster,
 * ld.acquire polls), then copies its outcome into the other CTAs' shared
 * memory and releases them with a second cluster barrier.  With 8 CTAs per
 * cluster the L2 line sees one arrival and one poller per 8 CTAs, which is
 * what makes a barrier over every co-resident 256-thread CTA cheaper than
 * the single-counter barriers.  Cumulativity carries every CTA's writes
 * before the barrier through its cluster's release/acquire and the leaders'
 * gpu-scope release/acquire to every CTA after it. */
__device__ __forceinline__ bool wgm_barrier_cluster(const wgm_launch &L, wgm_cta *c, int ngroups) {
  const unsigned csize = wgm_cluster_size(), rank = wgm_cluster_rank();
  wgm_cluster_sync();
  if (rank == 0 && threadIdx.x < 32) {
    int ok = c->ok;
    if (threadIdx.x == 0) {
      int *ctr = &L.st->bar_arrivals[(L.gen & 1) * WGM_LINE];
      const unsigned target = (unsigned)c->tmp[2] + (unsigned)(ngroups / (int)csize);
      c->tmp[2] = (int)target;
      wgm_red_add_release_gpu(ctr, 1);
      wgm_spin s = wgm_spin_start(L);
      while ((int)((unsigned)wgm_ld_acquire_gpu(ctr) - target) < 0) {
        if (wgm_spin_giveup(L, s, WGM_SITE_BARRIER)) {
          ok = 0;
          break;
        }
      }
      c->ok = ok;
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    for (unsigned r = 1 + threadIdx.x; r < csize; r += 32) wgm_st_cluster_peer(&c->ok, r, ok);
  }
  wgm_cluster_sync();
  return c->ok;
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
  /* one group: a CTA barrier is the whole barrier (its threads see each
   * other's global writes after it); no L2 round trip.  Its own failures
   * and the host abort above clear c->ok. */
  if (c->ngroups == 1) {
    __syncthreads();
    return c->ok;
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
    case WGM_BARRIER_CLUSTER:
      return wgm_barrier_cluster(L, c, c->ngroups);
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

/* ------------------------------------------------------------------------ */
/* Resumable phases                                                          */
/* ------------------------------------------------------------------------ */

/* Every app runs as a sequence of phases separated by inter-CTA barriers.
 * A phase is named by (target, round); target 0 is the device-side init.
 * A phase function does its work, names the next phase and returns
 * WGM_PHASE_NEXT (a barrier follows) or WGM_PHASE_DONE.  Everything a phase
 * needs is in global memory or derivable from (target, round), so a group
 * forked in at a resizing barrier starts at the next phase with nothing but
 * that pair: the role of the reference's generated Restoration_ctx and its
 * `switch (target)` resume points (lonestar/graph_apps/bfs/device/
 * merged.cl:310-397, kernel_merge/src/ProcessPersistentKernelVisitor.cpp:
 * 110-137,401-431). */
struct wgm_step {
  int target;
  int round;
};
#define WGM_PHASE_DONE 0
#define WGM_PHASE_NEXT 1

/* Work split of the current phase: group id and group count can change at
 * every resizing barrier, so each phase reads them afresh. */
struct wgm_split {
  int lane, warp, gw, NW, tid, nth;
  __device__ __forceinline__ explicit wgm_split(const wgm_cta *c) {
    lane = wgm_lane();
    warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    gw = c->id * nw + warp;
    NW = c->ngroups * nw;
    tid = c->id * blockDim.x + threadIdx.x;
    nth = c->ngroups * blockDim.x;
  }
};

/* Run phases from `cur` until done, with `sync` between phases. */
template <class Sync, class Phase>
__device__ __forceinline__ void wgm_drive(const wgm_launch &L, wgm_cta *c, wgm_step cur,
                                          Sync &&sync, Phase &&phase) {
  for (;;) {
    wgm_step nxt = cur;
    if (phase(cur, &nxt) != WGM_PHASE_NEXT) return;
    if (!sync(L, c, nxt)) return;
    cur = nxt;
  }
}

/* Plain barrier between phases (standalone persistent kernels). */
struct wgm_plain_sync {
  __device__ __forceinline__ bool operator()(const wgm_launch &L, wgm_cta *c, wgm_step) const {
    return wgm_barrier(L, c);
  }
};

/* ======================================================================== */
/* Megakernel runtime: non-persistent tasks, offer_kill / offer_fork, the    */
/* resizing barrier and the device-side scheduler                            */
/*                                                                           */
/* Reference counterparts (paths relative to the reference):                 */
/*   src/scheduler_rt/rt_device/main_device_body.cl:1-93  -> wgm_mega_body   */
/*   src/scheduler_rt/rt_device/cl_scheduler.cl:168-308  -> wgm_scheduler    */
/*   src/scheduler_rt/rt_device/scheduler_1.cl:10-135    -> wgm_offer_fork,  */
/*                                   wgm_offer_kill, the assignment loops    */
/*   src/scheduler_rt/rt_device/iw_barrier.cl:165-305    -> wgm_resize_barrier*/
/*   src/non_persistent_kernels/{matmult,reduce}/device  -> wgm_np_*         */
/* ======================================================================== */

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

/* Control block of every megakernel launch: the non-persistent task, the
 * budget of host-paced waits and the resizing barrier's flavour. */
struct wgm_mega_ctl {
  wgm_np_args np;
  unsigned long long idle_ns; /* budget of host-driven waits */
  int use_query_barrier;      /* skel.cpp:34: the query variant */
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
 * resize = false: a plain barrier over the persistent groups (no kill, no
 * fork), for app code that synchronises where it cannot be resumed.
 * Query variant (iw_barrier.cl:229-305): the master reads groups_to_kill and
 * the chosen highest ids leave after the release instead of on arrival. */
static __device__ int wgm_resize_barrier(const wgm_launch &L, wgm_cta *c, wgm_step nxt, bool query,
                                         bool resize = true) {
  wgm_dev_state *st = L.st;
  int *kng = &st->k_num_groups[1][0];
  __syncthreads();
  if (threadIdx.x == 0) {
    const int g = c->gen;
    int res = 1;
    if (c->id != 0) {
      if (resize && !query && wgm_offer_kill(L, c->id)) {
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
        const int tk = (resize && query) ? wgm_ld_acquire_gpu(&st->groups_to_kill) : 0;
        if (tk > 0) {
          /* query barrier: shrink by min(to_kill, n-1) from the top; no fork
           * while the scheduler wants groups */
          const int k = wgm_proto_take_kills<wgm_gpu_ops>(&st->groups_to_kill, n - 1);
          wgm_atom_add_acqrel_gpu(kng, -k);
          n -= k;
        } else if (resize) {
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
static __device__ void wgm_scheduler(const wgm_launch &L, unsigned long long idle, int lpg) {
  wgm_dev_state *st = L.st;
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


/* main_device_body.cl:1-93: discovered group 0 runs the scheduler; every
 * other group loops "TASK_WAIT, available++ -> get_task -> run".  A
 * persistent task runs `run(pc, start, sync)`: pc is the group's view of
 * the persistent task (k-ids, resized at every barrier), start the phase its
 * restoration record names, sync the resizing barrier to put between
 * phases (true: continue, false: this group leaves the task). */
template <class RunApp>
__device__ __forceinline__ void wgm_mega_body(const wgm_launch &L, const wgm_mega_ctl &M,
                                              RunApp &&run) {
  __shared__ wgm_cta c;  /* discovered view */
  __shared__ wgm_cta pc; /* persistent-task view: k-ids, resizing */
  __shared__ int s_task;
  __shared__ wgm_rctx s_rc;
  if (!wgm_discover(L, &c)) return;
  wgm_dev_state *st = L.st;
  if (c.id == 0) {
    if (threadIdx.x == 0) wgm_scheduler(L, M.idle_ns, c.ngroups - 1);
    __syncthreads();
    return;
  }
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      wgm_st_relaxed_gpu(&st->task_array[c.id], WGM_TASK_WAIT);
      wgm_atom_add_acqrel_gpu(&st->available_workgroups, 1);
      /* get_task (cl_scheduler.cl:168-187) */
      wgm_spin s = wgm_idle_start(L, M.idle_ns);
      int t;
      for (;;) {
        t = wgm_ld_acquire_gpu(&st->task_array[c.id]);
        if (t != WGM_TASK_WAIT) break;
        if (wgm_spin_giveup(L, s, WGM_SITE_GET_TASK)) {
          t = WGM_TASK_QUIT;
          break;
        }
      }
      s_task = t;
      if (t == WGM_TASK_PERSIST) {
        s_rc = st->r_ctx_arr[c.id];
        pc.id = __ldcg(&st->k_group_ids[1][c.id]);
        pc.ngroups = s_rc.w[WGM_RC_NGROUPS];
        pc.gen = s_rc.w[WGM_RC_GEN];
        pc.ok = 1;
        pc.tmp[0] = 0;
      }
    }
    __syncthreads();
    const int t = s_task;
    if (t == WGM_TASK_QUIT) break;
    if (t == WGM_TASK_MULT) {
      int kid = __ldcg(&st->k_group_ids[0][c.id]);
      int kn = __ldcg(&st->k_num_groups[0][0]);
      if (M.np.kind == WGM_NP_MATMULT_I32 || M.np.kind == WGM_NP_MATMULT_F32)
        wgm_np_matmult(L, M.np, kid, kn);
      else
        wgm_np_reduce(M.np, kid, kn);
      __syncthreads();
      if (threadIdx.x == 0) wgm_atom_add_acqrel_gpu(&st->k_executing[0][0], -1);
    } else if (t == WGM_TASK_PERSIST) {
      const wgm_step start = {s_rc.w[WGM_RC_TARGET], s_rc.w[WGM_RC_ROUND]};
      const bool query = M.use_query_barrier != 0;
      auto sync = [&](const wgm_launch &Lx, wgm_cta *cx, wgm_step nx) {
        return wgm_resize_barrier(Lx, cx, nx, query) == 1;
      };
      run(&pc, start, sync);
      __syncthreads();
      if (threadIdx.x == 0) {
        wgm_atom_add_acqrel_gpu(&st->k_executing[1][0], -1);
        wgm_atom_add_acqrel_sys(&L.hf->persistent_flag, -1);
      }
    }
  }
}

/* ======================================================================== */
/* The kernel API persistent apps are written against                        */
/*                                                                           */
/* The reference's persistent kernels call four stubs (kernel_merge/stubs/   */
/* stubs.h:4-7: resizing_global_barrier, global_barrier, offer_kill,         */
/* offer_fork) and the work-group queries, which kernel_merge rewrites to    */
/* the discovered (p_), barrier (b_) and kernel-context (k_) forms           */
/* (kernel_merge/src/ProcessPersistentKernelVisitor.cpp:87-103).  Here they  */
/* are device functions over a context that knows whether the app runs as a */
/* standalone persistent kernel or inside the megakernel; each returns       */
/* WGM_OK, WGM_KILLED (this group left the task: return at once, as the      */
/* reference's offer_kill_barrier macro returns -1, scheduler_1.cl:137-138)  */
/* or WGM_ERR_TIMEOUT (a bounded wait gave up: return as well).              */
/*                                                                           */
/* An app is a struct with a POD `Args` and a phase function                 */
/*   static __device__ int phase(wgm_ctx &x, const Args &a, wgm_step cur,    */
/*                               wgm_step *nxt);                             */
/* that runs phase `cur` (target 0 = the device-side init), names the next   */
/* phase in *nxt and returns WGM_PHASE_NEXT (a resizing barrier follows) or  */
/* WGM_PHASE_DONE.  The rules that make it resumable (the contract           */
/* kernel_merge generated, ProcessPersistentKernelVisitor.cpp:253-436):      */
/*  1. nothing lives in registers or shared memory across a phase boundary:  */
/*     what the next phase needs is in global memory or follows from         */
/*     (target, round), the whole restoration record of a forked group;      */
/*  2. every phase splits its work by wgm_group_id / wgm_num_groups read in  */
/*     that phase (they change at resizing barriers);                        */
/*  3. a counter a phase fills and the next reads is triple-buffered by      */
/*     round, the phase clearing the one two rounds ahead, so one barrier    */
/*     per phase suffices.                                                   */
/* wgm_app_kernel<App> and wgm_app_mega_kernel<App> turn the phase function  */
/* into the standalone kernel and the megakernel; wgm_app_kernels<App> has   */
/* the host launchers an app's wgm_app_vtable points at.                     */
/* ======================================================================== */

#ifndef WGM_KILLED
#define WGM_KILLED 1 /* not an error: this group left the persistent task */
#endif

struct wgm_ctx {
  const wgm_launch *L;
  wgm_cta *c;  /* this group's view: id, group count, barrier generation */
  int mega;    /* 1 inside the megakernel: barriers resize */
  int query;   /* the query variant of the resizing barrier */
};

/* p_get_group_id / k_get_group_id (discovery.cl:59-72, kernel_ctx.cl:6-28) */
__device__ __forceinline__ int wgm_group_id(const wgm_ctx &x) { return x.c->id; }
/* p_get_num_groups / k_get_num_groups */
__device__ __forceinline__ int wgm_num_groups(const wgm_ctx &x) { return x.c->ngroups; }
/* p_get_global_id / k_get_global_id */
__device__ __forceinline__ int wgm_global_id(const wgm_ctx &x) {
  return x.c->id * (int)blockDim.x + (int)threadIdx.x;
}
/* p_get_global_size / k_get_global_size */
__device__ __forceinline__ int wgm_global_size(const wgm_ctx &x) {
  return x.c->ngroups * (int)blockDim.x;
}

/* global_barrier (iw_barrier.cl:63-109): every thread of every group of
 * the task; inside the megakernel a barrier over the persistent groups that
 * neither kills nor forks (a point the app cannot be resumed from). */
static __device__ int global_barrier(wgm_ctx &x) {
  if (!x.mega) return wgm_barrier(*x.L, x.c) ? WGM_OK : WGM_ERR_TIMEOUT;
  return wgm_resize_barrier(*x.L, x.c, wgm_step{0, 0}, false, false) == 1 ? WGM_OK
                                                                          : WGM_ERR_TIMEOUT;
}

/* resizing_global_barrier (iw_barrier.cl:165-305): inside the megakernel the
 * highest groups may leave (WGM_KILLED) and free groups join, starting at
 * phase `next`; a standalone kernel gets a plain barrier. */
static __device__ int resizing_global_barrier(wgm_ctx &x, wgm_step next) {
  if (!x.mega) return wgm_barrier(*x.L, x.c) ? WGM_OK : WGM_ERR_TIMEOUT;
  const int r = wgm_resize_barrier(*x.L, x.c, next, x.query != 0);
  return r == 1 ? WGM_OK : r == 0 ? WGM_KILLED : WGM_ERR_TIMEOUT;
}

/* offer_kill (scheduler_1.cl:59-81) for a task loop without barriers, called
 * by the whole group: the highest persistent group leaves when the scheduler
 * wants groups.  `lock` is a zeroed device word of the app that offer_kill
 * and offer_fork hold, so a kill never lands between a fork's read of the
 * group count and its growth (a busy lock defers the offer).  A standalone
 * kernel never leaves. */
static __device__ int offer_kill(wgm_ctx &x, int *lock) {
  if (!x.mega) return WGM_OK;
  __shared__ int s_killed;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_killed = 0;
    if (x.c->id != 0 && wgm_try_lock(lock)) {
      s_killed = wgm_offer_kill(*x.L, x.c->id) ? 1 : 0;
      wgm_unlock(lock);
    }
  }
  __syncthreads();
  return s_killed ? WGM_KILLED : WGM_OK;
}

/* offer_fork (scheduler_1.cl:10-57) for a task loop without barriers,
 * called by the whole group: persistent group 0 takes every free group into
 * the task, each starting at phase `next`, under the app's `lock` (see
 * offer_kill). */
static __device__ int offer_fork(wgm_ctx &x, int *lock, wgm_step next) {
  if (!x.mega) return WGM_OK;
  __syncthreads();
  if (threadIdx.x == 0 && x.c->id == 0 && wgm_try_lock(lock)) {
    wgm_rctx rc;
    for (int k = 0; k < WGM_RCTX_WORDS; k++) rc.w[k] = 0;
    rc.w[WGM_RC_TARGET] = next.target;
    rc.w[WGM_RC_ROUND] = next.round;
    rc.w[WGM_RC_GEN] = x.c->gen;
    wgm_offer_fork(*x.L, -1, rc);
    wgm_unlock(lock);
  }
  __syncthreads();
  return WGM_OK;
}

/* The standalone persistent kernel of an app (standalone.cl:247-320):
 * discovery, the optional host handshake, the phases with plain barriers
 * between them, the persistent_flag decrement. */
template <class App, int MaxThreads = 1024>
__global__ void __launch_bounds__(MaxThreads) wgm_app_kernel(wgm_launch L, typename App::Args a) {
  __shared__ wgm_cta c;
  if (!wgm_discover(L, &c)) return;
  if (L.handshake && !wgm_standalone_handshake(L, &c)) {
    wgm_standalone_exit(L);
    return;
  }
  wgm_ctx x{&L, &c, 0, 0};
  wgm_drive(L, &c, wgm_step{0, 0}, wgm_plain_sync(),
            [&](wgm_step cur, wgm_step *nxt) { return App::phase(x, a, cur, nxt); });
  if (L.handshake) wgm_standalone_exit(L);
}

/* The megakernel hosting an app (the kernel_merge output,
 * KernelMerge.cpp:52-112, with main_device_body.cl): the scheduler, the
 * non-persistent task, and the app's phases with resizing barriers. */
template <class App, int MaxThreads = 1024>
__global__ void __launch_bounds__(MaxThreads)
    wgm_app_mega_kernel(wgm_launch L, wgm_mega_ctl M, typename App::Args a) {
  wgm_mega_body(L, M, [&](wgm_cta *pc, wgm_step start, auto &sync) {
    wgm_ctx x{&L, pc, 1, M.use_query_barrier};
    wgm_drive(L, pc, start, sync,
              [&](wgm_step cur, wgm_step *nxt) { return App::phase(x, a, cur, nxt); });
  });
}

/* Host launchers of an app's two kernels, for its wgm_app_vtable (launch,
 * launch_mega, occupancy).  `launch` points at the runtime's launch record
 * (wgm_launch) and `mega` at its megakernel control block (wgm_mega_ctl);
 * both are filled by libwgm for every launch. */
template <class App, int MaxThreads = 1024>
struct wgm_app_kernels {
  static int launch(const typename App::Args &a, const void *launch, int grid, int block,
                    void *stream) {
    if (!launch || grid < 1 || block < 32 || block > MaxThreads) return WGM_ERR_INVALID;
    wgm_app_kernel<App, MaxThreads>
        <<<grid, block, 0, (cudaStream_t)stream>>>(*(const wgm_launch *)launch, a);
    return cudaGetLastError() == cudaSuccess ? WGM_OK : WGM_ERR_CUDA;
  }
  static int launch_mega(const typename App::Args &a, const void *launch, const void *mega,
                         int grid, int block, void *stream) {
    if (!launch || !mega || grid < 2 || block < 32 || block > MaxThreads) return WGM_ERR_INVALID;
    wgm_app_mega_kernel<App, MaxThreads><<<grid, block, 0, (cudaStream_t)stream>>>(
        *(const wgm_launch *)launch, *(const wgm_mega_ctl *)mega, a);
    return cudaGetLastError() == cudaSuccess ? WGM_OK : WGM_ERR_CUDA;
  }
  /* CTAs per SM of the standalone kernel (mega = 0) or the megakernel. */
  static int occupancy(int mega, int block, int *ctas_per_sm) {
    if (!ctas_per_sm || block < 32 || block > MaxThreads) return WGM_ERR_INVALID;
    const void *fn = mega ? (const void *)wgm_app_mega_kernel<App, MaxThreads>
                          : (const void *)wgm_app_kernel<App, MaxThreads>;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, fn, block, 0) ==
                   cudaSuccess
               ? WGM_OK
               : WGM_ERR_CUDA;
  }
};

#endif
