/*
 * Shared host/device layout of the cooperative-kernel runtime state.
 *
 * GB300 counterpart of the reference's scheduler_rt/rt_common headers
 * (constants.h:3-8, ticket_lock.h:14-19, discovery.h:23-33, kernel_ctx.h:6-11,
 * iw_barrier.h:4-19, cl_scheduler.h:15-56).  The state-machine constants keep
 * the reference's names and values so host code written against
 * cl_scheduler.h reads the same; the layouts differ:
 *
 *  - capacities are sized for a GB300 (WGM_MAX_GROUPS co-resident CTAs,
 *    152 SMs x up to 16 CTAs of >= 128 threads) instead of MAX_P_GROUPS=512;
 *  - every word that CTAs contend on sits on its own 128-byte line;
 *  - the words the host polls (scheduler_flag, persistent_flag, ...) live in
 *    mapped pinned host memory (wgm_host_flags), everything else in HBM
 *    (wgm_dev_state); the device reaches the former with .sys-scope
 *    atomics and the latter with .gpu-scope atomics;
 *  - every spin has a time budget; expiry records a status instead of hanging.
 */
#ifndef WGM_COMMON_H
#define WGM_COMMON_H

#include <stdint.h>

#define WGM_MAX_GROUPS 4096
#define WGM_LINE 32 /* ints per 128-byte line */
#define WGM_RCTX_WORDS 16

/* Task values of task_array (constants.h:4-8). */
#define WGM_TASK_UNINIT (-2)
#define WGM_TASK_WAIT (-1)
#define WGM_TASK_QUIT 0
#define WGM_TASK_MULT 1
#define WGM_TASK_PERSIST 2

/* Scheduler states (cl_scheduler.h:15-21). */
#define WGM_DEVICE_SCHEDULER_INIT 0
#define WGM_DEVICE_WAITING 1
#define WGM_DEVICE_TO_QUIT 2
#define WGM_DEVICE_TO_TASK 3
#define WGM_DEVICE_GOT_GROUPS 4
#define WGM_DEVICE_TO_EXECUTE 5
#define WGM_DEVICE_TO_PERSISTENT_TASK 6

/* Device status codes written into wgm_host_flags.status. */
#define WGM_DEV_OK 0
#define WGM_DEV_TIMEOUT 1
#define WGM_DEV_ABORTED 2
#define WGM_DEV_OVERFLOW 3
#define WGM_DEV_BAD_INPUT 4

/* Spin sites (recorded with a timeout so the host can say which wait gave up). */
#define WGM_SITE_DISCOVERY 1
#define WGM_SITE_BARRIER 2
#define WGM_SITE_HANDSHAKE 3
#define WGM_SITE_SCHEDULER 4
#define WGM_SITE_GET_TASK 5
#define WGM_SITE_FORK 6
#define WGM_SITE_XF_BARRIER 7
#define WGM_SITE_TICKET_LOCK 8
#define WGM_SITE_RESIZE_BARRIER 9
#define WGM_SITE_QUEUE 10

/* Discovery modes. */
#define WGM_DISCOVERY_TICKET 0    /* one fetch-add ticket per CTA; ticket 0 closes */
#define WGM_DISCOVERY_REFERENCE 1 /* ticket lock + extra lock rounds (discovery.cl:26-57) */

/* Barrier kinds. */
#define WGM_BARRIER_SENSE 0 /* counter + generation word (sense reversal) */
#define WGM_BARRIER_XF 1    /* master/slave flags (iw_barrier.cl:63-109) */
#define WGM_BARRIER_TREE 2  /* two-level counter tree, then generation word */
#define WGM_BARRIER_COUNT 3 /* monotonic arrival counter, waiters poll it */
#define WGM_BARRIER_SPREAD 4 /* counter + generation copied on 16 lines */
/* COUNT when the launch has at most WGM_BARRIER_AUTO_COUNT_MAX groups, else
 * SENSE: one line that every CTA both updates and polls is the fastest
 * barrier for a few hundred CTAs and the slowest for a thousand. */
#define WGM_BARRIER_AUTO 5
#define WGM_BARRIER_AUTO_COUNT_MAX 384
/* cluster barrier: launches with a cluster dimension only */
#define WGM_BARRIER_CLUSTER 6

#define WGM_POLL_CLOSED 0x40000000

/* Restoration record handed to forked groups (the reference's per-app
 * Restoration_ctx, e.g. lonestar/graph_apps/bfs/restoration_ctx.h:1-10):
 * word 0 is `target`, the rest is app-defined loop-carried state. */
typedef struct wgm_rctx {
  int32_t w[WGM_RCTX_WORDS];
} wgm_rctx;

/* Host-visible words (mapped pinned host memory). */
typedef struct wgm_host_flags {
  int32_t scheduler_flag;       /* cl_scheduler.h:38 */
  int32_t pad0[WGM_LINE - 1];
  int32_t persistent_flag;      /* cl_scheduler.h:50 */
  int32_t pad1[WGM_LINE - 1];
  int32_t task_size;            /* cl_scheduler.h:41 */
  int32_t participating_groups; /* cl_scheduler.h:32 */
  int32_t check_value;          /* cl_scheduler.h:54 */
  int32_t abort_flag;           /* host -> device: give up every wait */
  int32_t pad2[WGM_LINE - 4];
  int32_t status;               /* first device error (WGM_DEV_*) */
  int32_t status_site;          /* WGM_SITE_* of the failing wait */
  int32_t status_detail;
  int32_t discovered;           /* groups found by the last discovery */
  int32_t pad3[WGM_LINE - 4];
} wgm_host_flags;

/* Device-resident runtime state (HBM). */
typedef struct wgm_dev_state {
  /* First device-side error of the current launch (fast path of the
   * mapped wgm_host_flags.status word). */
  int32_t dev_error;
  int32_t pad_e0[WGM_LINE - 1];

  /* Discovery (discovery.h:23-33).  Launch generation g uses slot g&1, so a
   * launch never needs the host to re-initialise discovery: the closer of
   * launch g clears slot (g+1)&1 for the next launch. */
  int32_t poll_word[2]; /* ticket mode: WGM_POLL_CLOSED | tickets taken */
  int32_t pad_d0[WGM_LINE - 2];
  int32_t count[2];     /* discovered groups of the launch */
  int32_t published;    /* generation whose count is valid */
  int32_t closed_gen;   /* reference mode: poll closed for this generation */
  int32_t pad_d1[WGM_LINE - 4];
  int32_t tl_counter; /* ticket lock (ticket_lock.h:14-19) */
  int32_t pad_d2[WGM_LINE - 1];
  int32_t tl_now_serving;
  int32_t pad_d3[WGM_LINE - 1];

  /* Barrier (iw_barrier.h:4-19 plus a two-level tree). */
  int32_t bar_count;
  int32_t pad_b0[WGM_LINE - 1];
  int32_t bar_gen;
  int32_t pad_b1[WGM_LINE - 1];
  int32_t bar_num_groups; /* resizing barrier: groups after the last resize */
  int32_t bar_to_kill;
  int32_t pad_b2[WGM_LINE - 2];
  int32_t tree_count[128 * WGM_LINE]; /* leaf counters, one line each */
  /* Counting barrier: arrivals of launch generation g on line g&1; the
   * discovery closer of launch g zeroes line (g+1)&1 for the next launch. */
  int32_t bar_arrivals[2 * WGM_LINE];
  /* Spread barrier: the generation word copied on 16 lines, CTA i polls
   * line i % 16. */
  int32_t bar_gen_spread[16 * WGM_LINE];

  /* Kernel contexts (kernel_ctx.h:6-11): [0] non-persistent, [1] persistent. */
  int32_t k_num_groups[2][WGM_LINE];
  int32_t k_executing[2][WGM_LINE];

  /* Scheduler (cl_scheduler.h:29-56), device side. */
  int32_t available_workgroups;
  int32_t pad_s0[WGM_LINE - 1];
  int32_t pool_lock;
  int32_t pad_s1[WGM_LINE - 1];
  int32_t groups_to_kill;
  int32_t pad_s2[WGM_LINE - 1];
  int32_t np_counter; /* last-group detection of the non-persistent task */
  int32_t pad_s3[WGM_LINE - 1];

  int32_t p_group_ids[WGM_MAX_GROUPS]; /* blockIdx -> discovered id */
  int32_t group_smid[WGM_MAX_GROUPS];  /* discovered id -> SM */
  int32_t xf_flags[WGM_MAX_GROUPS];    /* XF barrier arrival flags */
  int32_t task_array[WGM_MAX_GROUPS];  /* discovered id -> WGM_TASK_* */
  int32_t k_group_ids[2][WGM_MAX_GROUPS];
  wgm_rctx r_ctx_arr[WGM_MAX_GROUPS];
} wgm_dev_state;

#endif
