/*
 * Steps of the resizing protocol written once for two executors: the GPU
 * (instantiated with the scoped PTX operations of wgm_device.cuh) and a
 * CPU-thread model (host std::atomic operations, with a hook between the
 * steps so a test can force an interleaving).  The model runs the same code
 * the kernels run, so a race in these steps shows up on the CPU, without a
 * GPU.
 *
 * Ops supplies static functions over int words:
 *   ld_acquire(p), cas(p, expected, desired) -> old (acq_rel),
 *   add(p, v) -> old (acq_rel), and between() (a no-op on the GPU).
 *
 * Reference: the kill side of __offer_kill (src/scheduler_rt/rt_device/
 * scheduler_1.cl:59-81) reads groups_to_kill and stores the value minus one.
 * Here the scheduler may store the word at any moment (a request that no
 * longer needs groups clears it), so the decrement is one compare-and-swap:
 * a clear that lands between the read and the write makes the swap fail
 * instead of being overwritten by the stale value minus one.
 */
#ifndef WGM_PROTOCOL_H
#define WGM_PROTOCOL_H

#if defined(__CUDACC__)
#define WGM_PROTO __host__ __device__ __forceinline__
#define WGM_PROTO_NOCHECK _Pragma("nv_exec_check_disable")
#else
#define WGM_PROTO inline
#define WGM_PROTO_NOCHECK
#endif

/* Attempts of a contended compare-and-swap before the caller defers: each
 * failure means the word changed, and the next offer tries again. */
#define WGM_PROTO_CAS_TRIES 64

/* Take up to `want` kills from *to_kill atomically; returns how many were
 * taken (0 when the word is zero or keeps changing). */
WGM_PROTO_NOCHECK
template <class Ops>
WGM_PROTO int wgm_proto_take_kills(int *to_kill, int want) {
  int tk = Ops::ld_acquire(to_kill);
  for (int tries = 0; tk > 0 && want > 0 && tries < WGM_PROTO_CAS_TRIES; tries++) {
    const int k = tk < want ? tk : want;
    Ops::between();
    const int old = Ops::cas(to_kill, tk, tk - k);
    if (old == tk) return k;
    tk = old;
  }
  return 0;
}

/* __offer_kill: the group with the highest persistent id `kid` leaves when
 * the scheduler asked for groups.  Being the highest id is the lock - only
 * one group can be it - and the decrement of the group count releases it to
 * the next highest.  Returns true when this group must leave. */
WGM_PROTO_NOCHECK
template <class Ops>
WGM_PROTO bool wgm_proto_offer_kill(int *num_groups, int *to_kill, int kid) {
  if (kid != Ops::ld_acquire(num_groups) - 1) return false;
  if (wgm_proto_take_kills<Ops>(to_kill, 1) == 0) return false;
  Ops::add(num_groups, -1);
  return true;
}

#endif
