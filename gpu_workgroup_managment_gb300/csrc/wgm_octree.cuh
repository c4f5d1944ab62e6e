/*
 * Work-stealing octree build: a persistent task without a global barrier in
 * its loop, the reference's stress test of offer_kill / offer_fork
 * (src/test_suite/final_octree/device/octree.cl:130-320, host plugin
 * src/test_suite/final_octree/octree.h).
 *
 * A task is a box (centre, half-width) and a range [beg, end) of particles
 * in one of two buffers.  A CTA pops a task from a pool (its own first, then
 * the others, octree.cl:196-203), counts its particles per octant, scatters
 * them by octant into the other buffer, and for each octant either pushes a
 * child task (more than maxchilds particles: a new block of 8 tree entries,
 * the child's position recorded in the parent's entry) or closes a leaf
 * (entry = 0x80000000 | count, the particles moved to the first buffer,
 * particlesDone += count).  The build ends when particlesDone reaches N.
 *
 * GB300 choices: per-warp ballots count and place the particles (one shared
 * atomic per warp, octant and pass instead of one per particle); every pool
 * lock, idle wait and pool or tree overflow is bounded and reported; pools
 * are fewer than groups (group g uses pool g % num_pools) so their memory
 * stays modest at 1000+ CTAs.  Particles are read with ld.global.cg: another
 * SM may have rewritten a range this SM cached before.
 */
#ifndef WGM_OCTREE_CUH
#define WGM_OCTREE_CUH

#include "wgm_device.cuh"

struct __align__(16) wgm_octree_task {
  float4 middle; /* centre xyz, half-width w */
  int flip;      /* particles of the range are in the second buffer */
  unsigned end, beg, treepos;
};

struct wgm_octree_args {
  const float4 *input;   /* [n] the particles every run starts from */
  float4 *particles;     /* [n] output, leaf by leaf */
  float4 *newparticles;  /* [n] the second buffer */
  unsigned *tree;        /* [tree_cap] */
  long long tree_cap;
  unsigned *tree_size;   /* next free tree entry (starts at 100, octree.cl:127) */
  unsigned *done;        /* particles in closed leaves */
  int n, maxchilds;
  wgm_octree_task *pools; /* [num_pools][pool_size] stacks */
  int *locks, *heads;     /* [num_pools] */
  int num_pools, pool_size;
  int *tasks_out;         /* tasks processed by the last run */
  int *rlock;             /* megakernel: makes offer_kill and offer_fork exclusive */
};

#define WGM_OCTREE_ROOT_FREE 100u /* first tree entry handed to a child block */

__device__ __forceinline__ int wgm_oct_box(const float4 p, const float4 m) {
  return (p.x < m.x ? 0 : 1) + (p.y < m.y ? 0 : 2) + (p.z < m.z ? 0 : 4); /* octree.cl:96-101 */
}

/* Bounded pool lock (pool_try_lock spun, octree.cl:31-42). */
__device__ __forceinline__ bool wgm_oct_lock(const wgm_launch &L, int *m) {
  wgm_spin s = wgm_spin_start(L);
  while (wgm_atom_exch_acquire_gpu(m, 1) != 0) {
    if (wgm_spin_giveup(L, s, WGM_SITE_QUEUE)) return false;
  }
  return true;
}

/* wgm_task_pop (octree.cl:48-63), thread 0: 1 got a task, 0 pool empty,
 * -1 the lock wait gave up. */
__device__ __forceinline__ int wgm_oct_pop(const wgm_launch &L, const wgm_octree_args &a,
                                           wgm_octree_task *t, int pool) {
  if (!wgm_oct_lock(L, &a.locks[pool])) return -1;
  int got = 0;
  const int h = __ldcg(&a.heads[pool]);
  if (h > 0) {
    const float4 *src = reinterpret_cast<const float4 *>(&a.pools[(size_t)pool * a.pool_size + h - 1]);
    const float4 w0 = __ldcg(src), w1 = __ldcg(src + 1);
    t->middle = w0;
    t->flip = __float_as_int(w1.x);
    t->end = __float_as_uint(w1.y);
    t->beg = __float_as_uint(w1.z);
    t->treepos = __float_as_uint(w1.w);
    a.heads[pool] = h - 1;
    got = 1;
  }
  wgm_st_release_gpu(&a.locks[pool], 0);
  return got;
}

/* wgm_task_push (octree.cl:68-82), thread 0: 1 pushed, 0 pool full, -1 the
 * lock wait gave up. */
__device__ __forceinline__ int wgm_oct_push(const wgm_launch &L, const wgm_octree_args &a,
                                            const wgm_octree_task &t, int pool) {
  if (!wgm_oct_lock(L, &a.locks[pool])) return -1;
  int pushed = 0;
  const int h = __ldcg(&a.heads[pool]);
  if (h < a.pool_size) {
    float4 *dst = reinterpret_cast<float4 *>(&a.pools[(size_t)pool * a.pool_size + h]);
    dst[0] = t.middle;
    dst[1] = make_float4(__int_as_float(t.flip), __uint_as_float(t.end), __uint_as_float(t.beg),
                         __uint_as_float(t.treepos));
    a.heads[pool] = h + 1;
    pushed = 1;
  }
  wgm_st_release_gpu(&a.locks[pool], 0);
  return pushed;
}

/* A pool or the tree ran out of room (octree.cl:283-286 gives up the build
 * by declaring every particle done): record the overflow, then end it. */
__device__ __forceinline__ void wgm_oct_overflow(const wgm_launch &L, const wgm_octree_args &a,
                                                 int detail) {
  wgm_fail(L, WGM_DEV_OVERFLOW, WGM_SITE_QUEUE, detail);
  atomicMax(a.done, (unsigned)a.n);
}

/* Start of a run (octree_init, octree.cl:106-147, and the host reset of
 * octree.h:80-96): every group copies its share of the input particles;
 * group 0 clears the pools, the counters and the root block of the tree and
 * pushes the root task.  A barrier must follow. */
__device__ __forceinline__ void wgm_octree_init(const wgm_launch &L, const wgm_cta *c,
                                                const wgm_octree_args &a) {
  const int tid = c->id * blockDim.x + threadIdx.x, nth = c->ngroups * blockDim.x;
  for (int i = tid; i < a.n; i += nth) a.particles[i] = __ldg(&a.input[i]);
  if (c->id != 0) return;
  for (int p = threadIdx.x; p < a.num_pools; p += blockDim.x) {
    a.heads[p] = 0;
    a.locks[p] = 0;
  }
  for (int i = threadIdx.x; i < (int)WGM_OCTREE_ROOT_FREE; i += blockDim.x) a.tree[i] = 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    if (a.rlock) *a.rlock = 0;
    *a.tree_size = WGM_OCTREE_ROOT_FREE;
    *a.done = 0;
    if (a.tasks_out) *a.tasks_out = 0;
    wgm_octree_task t;
    t.middle = make_float4(0.f, 0.f, 0.f, 256.f);
    t.flip = 0;
    t.beg = 0;
    t.end = (unsigned)a.n;
    t.treepos = 0;
    if (wgm_oct_push(L, a, t, 0) != 1) wgm_oct_overflow(L, a, 0);
    __threadfence();
  }
}

/* Process one task with the whole CTA (octree.cl:215-316). */
__device__ __forceinline__ void wgm_octree_task_run(const wgm_launch &L,
                                                    const wgm_octree_args &a,
                                                    const wgm_octree_task &t, int pool,
                                                    unsigned *cnt, unsigned *cur) {
  const float4 *from = t.flip ? a.newparticles : a.particles;
  float4 *to = t.flip ? a.particles : a.newparticles;
  const int lane = wgm_lane(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned beg = t.beg, end = t.end;
  if (threadIdx.x < 8) cnt[threadIdx.x] = 0;
  __syncthreads();
  /* count per octant: one ballot per octant and warp step */
  for (unsigned b = beg + warp * 32; b < end; b += nw * 32) {
    const unsigned i = b + lane;
    const int box = i < end ? wgm_oct_box(__ldcg(&from[i]), t.middle) : -1;
#pragma unroll
    for (int o = 0; o < 8; o++) {
      const unsigned m = __ballot_sync(WGM_FULL, box == o);
      if (lane == 0 && m) atomicAdd(&cnt[o], __popc(m));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned s = 0;
    for (int o = 0; o < 8; o++) {
      cur[o] = s; /* start of octant o within the range */
      s += cnt[o];
    }
  }
  __syncthreads();
  /* scatter by octant: one shared reservation per octant and warp step */
  for (unsigned b = beg + warp * 32; b < end; b += nw * 32) {
    const unsigned i = b + lane;
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    int box = -1;
    if (i < end) {
      p = __ldcg(&from[i]);
      box = wgm_oct_box(p, t.middle);
    }
#pragma unroll
    for (int o = 0; o < 8; o++) {
      const unsigned m = __ballot_sync(WGM_FULL, box == o);
      if (!m) continue;
      const int lead = __ffs(m) - 1;
      unsigned base = 0;
      if (lane == lead) base = atomicAdd(&cur[o], __popc(m));
      base = __shfl_sync(WGM_FULL, base, lead);
      if (box == o) to[beg + base + __popc(m & wgm_lanemask_lt())] = p;
    }
  }
  __syncthreads();
  /* cur[o] is now the end of octant o; its start is cur[o] - cnt[o] */
  /* leaves of a range that ended up in the second buffer move to the first */
  if (!t.flip) {
    for (int o = 0; o < 8; o++) {
      if (cnt[o] > (unsigned)a.maxchilds) continue;
      const unsigned s0 = beg + cur[o] - cnt[o], s1 = beg + cur[o];
      for (unsigned j = s0 + threadIdx.x; j < s1; j += blockDim.x) a.particles[j] = __ldcg(&to[j]);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence(); /* the scattered range before any child task is visible */
    for (int o = 0; o < 8; o++) {
      const unsigned c = cnt[o];
      const unsigned s0 = cur[o] - c;
      if (c > (unsigned)a.maxchilds) {
        wgm_octree_task nt;
        nt.middle.x = t.middle.x + t.middle.w * (float)((o & 1) ? 1 : -1);
        nt.middle.y = t.middle.y + t.middle.w * (float)((o & 2) ? 1 : -1);
        nt.middle.z = t.middle.z + t.middle.w * (float)((o & 4) ? 1 : -1);
        nt.middle.w = t.middle.w / 2.0f;
        nt.flip = !t.flip;
        nt.beg = beg + s0;
        nt.end = nt.beg + c;
        const unsigned pos = atomicAdd(a.tree_size, 8u);
        if ((long long)pos + 8 > a.tree_cap) {
          wgm_oct_overflow(L, a, 1);
          break;
        }
        a.tree[t.treepos + o] = pos;
        nt.treepos = pos;
        int r = 0;
        for (int k = 0; k < a.num_pools && r == 0; k++) r = wgm_oct_push(L, a, nt, (pool + k) % a.num_pools);
        if (r != 1) {
          if (r == 0) wgm_oct_overflow(L, a, 2);
          break;
        }
      } else {
        a.tree[t.treepos + o] = 0x80000000u | c;
        atomicAdd(a.done, c);
      }
    }
    if (a.tasks_out) atomicAdd(a.tasks_out, 1);
  }
  __syncthreads();
}

/* The task loop (octree.cl:170-317).  `offer(c)` runs on thread 0 at the
 * top of every iteration and returns true when this group must leave (the
 * megakernel's offer_fork by group 0 and offer_kill by the others; the
 * standalone kernel offers nothing).  Returns when the build is done, the
 * group left, or a wait gave up. */
template <class Offer>
__device__ void wgm_octree_loop(const wgm_launch &L, wgm_cta *c, const wgm_octree_args &a,
                                Offer &&offer) {
  __shared__ wgm_octree_task t;
  __shared__ unsigned cnt[8], cur[8];
  __shared__ int s_state;
  const int pool = c->id % a.num_pools;
  wgm_spin idle = wgm_spin_start(L);
  for (;;) {
    if (threadIdx.x == 0) {
      int state = 0; /* 0 no task yet, 1 task, 2 done, 3 leave */
      if (offer(c)) {
        state = 3;
      } else {
        for (int k = 0; k < a.num_pools; k++) {
          const int r = wgm_oct_pop(L, a, &t, (pool + k) % a.num_pools);
          if (r != 0) {
            state = r > 0 ? 1 : 3;
            break;
          }
        }
        if (state == 0) {
          if (wgm_ld_acquire_gpu(reinterpret_cast<const int *>(a.done)) >= a.n ||
              wgm_ld_relaxed_gpu(&L.st->dev_error) != 0)
            state = 2;
          else if (wgm_spin_giveup(L, idle, WGM_SITE_GET_TASK))
            state = 3;
          else
            __nanosleep(256);
        } else if (state == 1) {
          idle = wgm_spin_start(L);
        }
      }
      s_state = state;
    }
    __syncthreads();
    const int state = s_state;
    if (state >= 2) break;
    if (state == 1) wgm_octree_task_run(L, a, t, pool, cnt, cur);
    __syncthreads();
  }
}

#endif
