/*
 * Connect-four look-ahead: the reference's second work-stealing persistent
 * task (src/test_suite/connect_four/device/connect_four.cl:350-487, host
 * plugin connect_four.h).
 *
 * Nodes are move sequences from a base board; the 7 first moves are the
 * roots.  A CTA pops a node id, replays the moves on the base board, scores
 * the board (25 line scans, connect_four.cl:94-176), stores the score as the
 * node's value and either closes the node (level maxlevel, or a four-in-a-row
 * score +-666) and propagates it up - min into a parent of even level, max
 * into odd, the seventh answer moving on to the grandparent, a root writing
 * next_move_value - or creates the 7 children and pushes them
 * (connect_four.cl:440-485).  The search ends when the 7 roots are done.
 * min and max do not depend on the order of the answers, so the result is
 * deterministic whatever the schedule.
 *
 * GB300 choices: one thread per line scan (threads 0..24) and a thread-0
 * reduction in thread order (the reference's rule: the first +-666 wins,
 * otherwise the sum); bounded pool locks and idle waits; node and pool
 * overflows reported (the reference writes one node past its array at the
 * capacity limit and spins forever on full pools).
 */
#ifndef WGM_C4_CUH
#define WGM_C4_CUH

#include "wgm_octree.cuh" /* bounded pool lock, overflow reporting */

#define WGM_C4_ROWS 6
#define WGM_C4_COLS 7
#define WGM_C4_CELLS 42
#define WGM_C4_PLUS_INF 666
#define WGM_C4_MINUS_INF (-666)
#define WGM_C4_MAX_LOOKAHEAD 7
#define WGM_C4_EMPTY 0
#define WGM_C4_HUMAN 1
#define WGM_C4_COMPUTER 2

struct wgm_c4_node {
  int parent;
  int level;
  int value;   /* own score, then min/max of the children's answers */
  int answers; /* children that answered */
  unsigned char moves[8];
};

struct wgm_c4_args {
  const unsigned char *base_board; /* [42], row-major, row 0 at the top */
  int maxlevel;
  wgm_c4_node *nodes;
  int num_nodes;
  int *node_head;
  int *pool, *locks, *heads; /* [num_pools][pool_size] node ids */
  int num_pools, pool_size;
  int *next_move_value; /* [7] output */
  int *root_done;
  int *tasks_out;
  int *rlock; /* megakernel: makes offer_kill and offer_fork exclusive */
};

__device__ __forceinline__ int wgm_c4_push(const wgm_launch &L, const wgm_c4_args &a, int node,
                                           int p) {
  if (!wgm_oct_lock(L, &a.locks[p])) return -1;
  int pushed = 0;
  const int h = __ldcg(&a.heads[p]);
  if (h < a.pool_size) {
    a.pool[(size_t)p * a.pool_size + h] = node;
    a.heads[p] = h + 1;
    pushed = 1;
  }
  wgm_st_release_gpu(&a.locks[p], 0);
  return pushed;
}

/* 1: *node set, 0: pool empty, -1: the lock wait gave up. */
__device__ __forceinline__ int wgm_c4_pop(const wgm_launch &L, const wgm_c4_args &a, int *node,
                                          int p) {
  if (!wgm_oct_lock(L, &a.locks[p])) return -1;
  int got = 0;
  const int h = __ldcg(&a.heads[p]);
  if (h > 0) {
    *node = __ldcg(&a.pool[(size_t)p * a.pool_size + h - 1]);
    a.heads[p] = h - 1;
    got = 1;
  }
  wgm_st_release_gpu(&a.locks[p], 0);
  return got;
}

__device__ __forceinline__ void wgm_c4_fail(const wgm_launch &L, const wgm_c4_args &a, int d) {
  wgm_fail(L, WGM_DEV_OVERFLOW, WGM_SITE_QUEUE, d);
  atomicMax(a.root_done, WGM_C4_COLS);
}

/* chain_value (connect_four.cl:70-80). */
__device__ __forceinline__ void wgm_c4_chain(int *v, int player, int chain) {
  if (player != WGM_C4_EMPTY) {
    if (chain >= 4)
      *v = player == WGM_C4_COMPUTER ? WGM_C4_PLUS_INF : WGM_C4_MINUS_INF;
    else if (chain >= 2)
      *v += player == WGM_C4_COMPUTER ? 1 : -1;
  }
}

/* scan_board (connect_four.cl:84-130): chains along one line. */
__device__ __forceinline__ int wgm_c4_scan(const unsigned char *board, int row, int col, int dr,
                                           int dc) {
  int res = 0, player = WGM_C4_EMPTY, chain = 0;
  do {
    const int cell = board[row * WGM_C4_COLS + col];
    if (cell == player) {
      chain++;
    } else {
      wgm_c4_chain(&res, player, chain);
      if (res == WGM_C4_PLUS_INF || res == WGM_C4_MINUS_INF) return res;
      player = cell;
      chain = 1;
    }
    row += dr;
    col += dc;
  } while (0 <= row && row < WGM_C4_ROWS && 0 <= col && col < WGM_C4_COLS);
  wgm_c4_chain(&res, player, chain);
  return res;
}

/* Line scan number i of board_value (connect_four.cl:135-170): 0-5 rows,
 * 6-12 columns, 13-18 down-right diagonals, 19-24 down-left diagonals. */
__device__ __forceinline__ int wgm_c4_line(const unsigned char *board, int i) {
  if (i < 6) return wgm_c4_scan(board, i, 0, 0, 1);
  if (i < 13) return wgm_c4_scan(board, 0, i - 6, 1, 0);
  if (i < 19) {
    const int j = i - 13;
    return j < 3 ? wgm_c4_scan(board, j, 0, 1, 1) : wgm_c4_scan(board, 0, j - 2, 1, 1);
  }
  const int j = i - 19;
  return j < 3 ? wgm_c4_scan(board, j, WGM_C4_COLS - 1, 1, -1) : wgm_c4_scan(board, 0, j, 1, -1);
}

/* Start of a run (connect_four.cl:356-397 and the host reset of
 * connect_four.h:148-191): group 0 clears pools and counters, creates the 7
 * roots and queues them.  A barrier must follow. */
__device__ __forceinline__ void wgm_c4_init(const wgm_launch &L, const wgm_cta *c,
                                            const wgm_c4_args &a) {
  if (c->id != 0) return;
  for (int p = threadIdx.x; p < a.num_pools; p += blockDim.x) {
    a.heads[p] = 0;
    a.locks[p] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (a.rlock) *a.rlock = 0;
    *a.root_done = 0;
    if (a.tasks_out) *a.tasks_out = 0;
    for (int i = 0; i < WGM_C4_COLS; i++) {
      a.next_move_value[i] = WGM_C4_MINUS_INF;
      wgm_c4_node &n = a.nodes[i];
      n.parent = -1;
      n.level = 1;
      for (int k = 0; k < 8; k++) n.moves[k] = 0;
      n.moves[0] = (unsigned char)i;
      n.value = 0;
      n.answers = 0;
      if (wgm_c4_push(L, a, i, i % a.num_pools) != 1) wgm_c4_fail(L, a, 0);
    }
    *a.node_head = WGM_C4_COLS;
    __threadfence();
  }
}

/* wgm_update_parent (connect_four.cl:305-340), thread 0. */
__device__ __forceinline__ void wgm_c4_answer(const wgm_c4_args &a, int id) {
  for (;;) {
    wgm_c4_node *n = &a.nodes[id];
    const int level = __ldcg(&n->level);
    const int value = wgm_ld_acquire_gpu(&n->value);
    if (level == 1) {
      a.next_move_value[id] = value;
      wgm_atom_add_acqrel_gpu(a.root_done, 1);
      return;
    }
    const int parent = __ldcg(&n->parent);
    wgm_c4_node *p = &a.nodes[parent];
    if (((level - 1) % 2) == 0)
      atomicMin(&p->value, value); /* even level: the human takes the lowest */
    else
      atomicMax(&p->value, value); /* odd level: the computer takes the highest */
    if (wgm_atom_add_acqrel_gpu(&p->answers, 1) != 6) return;
    id = parent; /* the seventh answer moves up */
  }
}

/* One node with the whole CTA (connect_four.cl:428-485). */
__device__ __forceinline__ void wgm_c4_task(const wgm_launch &L, const wgm_c4_args &a, int id,
                                            int pool, unsigned char *board, int *val) {
  const wgm_c4_node *n = &a.nodes[id];
  for (int i = threadIdx.x; i < WGM_C4_CELLS; i += blockDim.x) board[i] = __ldg(&a.base_board[i]);
  __syncthreads();
  if (threadIdx.x == 0) {
    /* update_board (connect_four.cl:180-220): the computer moves first; a
     * move into a full column is skipped without changing the player */
    int player = WGM_C4_COMPUTER;
    const int level = __ldcg(&n->level);
    for (int i = 0; i < level; i++) {
      const int col = (int)__ldcg(reinterpret_cast<const int *>(n->moves) + (i >> 2)) >>
                          ((i & 3) * 8) & 0xff;
      if (board[col] != WGM_C4_EMPTY) continue;
      int row = 0;
      while (row < WGM_C4_ROWS && board[row * WGM_C4_COLS + col] == WGM_C4_EMPTY) row++;
      board[(row - 1) * WGM_C4_COLS + col] = (unsigned char)player;
      player = player == WGM_C4_COMPUTER ? WGM_C4_HUMAN : WGM_C4_COMPUTER;
    }
  }
  __syncthreads();
  val[threadIdx.x] = threadIdx.x < 25 ? wgm_c4_line(board, threadIdx.x) : 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    int value = 0;
    for (int i = 0; i < (int)blockDim.x; i++) {
      if (val[i] == WGM_C4_PLUS_INF || val[i] == WGM_C4_MINUS_INF) {
        value = val[i];
        break;
      }
      value += val[i];
    }
    wgm_c4_node *w = &a.nodes[id];
    const int level = __ldcg(&n->level);
    wgm_st_release_gpu(&w->value, value);
    if (level >= a.maxlevel || value == WGM_C4_PLUS_INF || value == WGM_C4_MINUS_INF) {
      wgm_st_release_gpu(&w->answers, 7);
      wgm_c4_answer(a, id);
    } else {
      unsigned char mv[8];
      for (int k = 0; k < 8; k++) mv[k] = (unsigned char)(
          (int)__ldcg(reinterpret_cast<const int *>(n->moves) + (k >> 2)) >> ((k & 3) * 8) & 0xff);
      for (int i = 0; i < WGM_C4_COLS; i++) {
        const int cid = atomicAdd(a.node_head, 1);
        if (cid >= a.num_nodes) {
          wgm_c4_fail(L, a, 1);
          break;
        }
        wgm_c4_node &ch = a.nodes[cid];
        ch.parent = id;
        ch.level = level + 1;
        for (int k = 0; k < 8; k++) ch.moves[k] = k < level ? mv[k] : 0;
        ch.moves[level] = (unsigned char)i;
        ch.value = 0;
        ch.answers = 0;
        __threadfence();
        int r = 0;
        for (int k = 0; k < a.num_pools && r == 0; k++) r = wgm_c4_push(L, a, cid, (pool + k) % a.num_pools);
        if (r != 1) {
          if (r == 0) wgm_c4_fail(L, a, 2);
          break;
        }
      }
    }
    if (a.tasks_out) atomicAdd(a.tasks_out, 1);
  }
  __syncthreads();
}

/* The task loop (connect_four.cl:399-486); `offer` as in wgm_octree_loop. */
template <class Offer>
__device__ void wgm_c4_loop(const wgm_launch &L, wgm_cta *c, const wgm_c4_args &a,
                            Offer &&offer) {
  __shared__ unsigned char board[WGM_C4_CELLS];
  __shared__ int val[1024];
  __shared__ int s_state, s_node;
  const int pool = c->id % a.num_pools;
  wgm_spin idle = wgm_spin_start(L);
  for (;;) {
    if (threadIdx.x == 0) {
      int state = 0; /* 0 no task yet, 1 task, 2 done, 3 leave */
      if (offer(c)) {
        state = 3;
      } else {
        for (int k = 0; k < a.num_pools; k++) {
          const int r = wgm_c4_pop(L, a, &s_node, (pool + k) % a.num_pools);
          if (r != 0) {
            state = r > 0 ? 1 : 3;
            break;
          }
        }
        if (state == 0) {
          if (wgm_ld_acquire_gpu(a.root_done) >= WGM_C4_COLS ||
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
    if (state == 1) wgm_c4_task(L, a, s_node, pool, board, val);
    __syncthreads();
  }
}

#endif
