/*
 * OpenCL C 2.0 -> C++20 shim used to compile the reference's own kernel
 * sources on the CPU, so that the oracle restatement can be checked against
 * the reference's actual arithmetic (the reference ships no golden vectors and
 * no OpenCL 2.0 CPU runtime with SVM atomics exists here).
 *
 * TEST INFRASTRUCTURE ONLY.  Model: ONE work-group of `local_size` work-items,
 * each a std::thread.  With one group the discovery protocol finds count == 1,
 * the inter-workgroup barriers have no peers and reduce to their local
 * barrier() calls, and `__local` declarations inside the kernel body (turned
 * into `static` by build_ref.py before compilation) are shared by all
 * work-items exactly as work-group local memory is.
 *
 * Atomics map to std::atomic with the same memory orders; scopes are ignored
 * (a CPU has one coherent memory).  OpenCL 1.x atomic_add/atomic_min on plain
 * pointers map to GCC __atomic builtins.
 */
#pragma once

#include <atomic>
#include <barrier>
#include <climits>
#include <cstddef>
#include <cstdint>

#define __OPENCL_C_VERSION__ 200
#define __kernel
#define kernel
#define __global
#define __constant const
/* In parameter lists `__local` is just a pointer qualifier.  Declarations of
 * work-group arrays inside kernel bodies are rewritten to `static` by the
 * build script, so the empty expansion here only ever meets parameters. */
#define __local
/* cl_execution.h:96-101 builds the reference with -DAMD_MEM_ORDERS. */
#ifndef AMD_MEM_ORDERS
#define AMD_MEM_ORDERS 1
#endif

typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef std::atomic<int> atomic_int;

constexpr std::memory_order memory_order_relaxed = std::memory_order_relaxed;
constexpr std::memory_order memory_order_acquire = std::memory_order_acquire;
constexpr std::memory_order memory_order_release = std::memory_order_release;
constexpr std::memory_order memory_order_acq_rel = std::memory_order_acq_rel;
constexpr std::memory_order memory_order_seq_cst = std::memory_order_seq_cst;

enum cl_shim_scope {
  memory_scope_work_item = 0,
  memory_scope_work_group,
  memory_scope_device,
  memory_scope_all_svm_devices
};

#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2

namespace clshim {
extern thread_local int lid;
extern int local_size;
extern std::barrier<> *wg_barrier;
}  // namespace clshim

inline size_t get_local_id(int) { return (size_t)clshim::lid; }
inline size_t get_local_size(int) { return (size_t)clshim::local_size; }
inline size_t get_group_id(int) { return 0; }
inline size_t get_num_groups(int) { return 1; }
inline size_t get_global_id(int) { return (size_t)clshim::lid; }
inline size_t get_global_size(int) { return (size_t)clshim::local_size; }
inline void barrier(int) { clshim::wg_barrier->arrive_and_wait(); }

/* OpenCL 2.0 explicit atomics on atomic_int (scopes ignored). */
inline int atomic_load_explicit(atomic_int *p, std::memory_order o, int) { return p->load(o); }
inline int atomic_load_explicit(atomic_int *p, std::memory_order o) { return p->load(o); }
inline void atomic_store_explicit(atomic_int *p, int v, std::memory_order o, int) { p->store(v, o); }
inline void atomic_store_explicit(atomic_int *p, int v, std::memory_order o) { p->store(v, o); }
inline int atomic_fetch_add_explicit(atomic_int *p, int v, std::memory_order o, int) { return p->fetch_add(v, o); }
inline int atomic_fetch_add_explicit(atomic_int *p, int v, std::memory_order o) { return p->fetch_add(v, o); }
inline int atomic_fetch_sub_explicit(atomic_int *p, int v, std::memory_order o, int) { return p->fetch_sub(v, o); }
inline int atomic_fetch_sub_explicit(atomic_int *p, int v, std::memory_order o) { return p->fetch_sub(v, o); }
inline int atomic_exchange_explicit(atomic_int *p, int v, std::memory_order o, int) { return p->exchange(v, o); }
inline int atomic_exchange_explicit(atomic_int *p, int v, std::memory_order o) { return p->exchange(v, o); }
inline int atomic_load(atomic_int *p) { return p->load(); }
inline void atomic_store(atomic_int *p, int v) { p->store(v); }
inline int atomic_fetch_add(atomic_int *p, int v) { return p->fetch_add(v); }
inline int atomic_fetch_sub(atomic_int *p, int v) { return p->fetch_sub(v); }
inline int atomic_fetch_min(atomic_int *p, int v) {
  int cur = p->load();
  while (v < cur && !p->compare_exchange_weak(cur, v)) {
  }
  return cur;
}
inline void atomic_work_item_fence(int, std::memory_order o, int) { std::atomic_thread_fence(o); }

/* OpenCL 1.x atomics on plain global pointers. */
inline int atomic_add(int *p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
inline unsigned atomic_add(unsigned *p, unsigned v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
inline unsigned atomic_min(unsigned *p, unsigned v) {
  unsigned cur = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (v < cur && !__atomic_compare_exchange_n(p, &cur, v, true, __ATOMIC_SEQ_CST,
                                                 __ATOMIC_SEQ_CST)) {
  }
  return cur;
}
inline int atomic_min(int *p, int v) {
  int cur = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (v < cur && !__atomic_compare_exchange_n(p, &cur, v, true, __ATOMIC_SEQ_CST,
                                                 __ATOMIC_SEQ_CST)) {
  }
  return cur;
}
