/*
 * Served form (include/wgm.h "served form"): the serving megakernel
 * wgm_k_serve and its host side - resident datasets, the request-state arena
 * with admission by free device memory, a Poisson request generator, the
 * host request and completion rings, and latency statistics.
 *
 * Host side follows the reference's communicator (src/scheduler_rt/rt_host/
 * cl_communicator.h:19-465: launch, persistent task, timed non-persistent
 * tasks, redlines and summary) generalised from one synchronous task at a
 * time to a stream of concurrent requests.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "../../include/wgm.h"
#include "wgm_internal.h"
#include "wgm_kernels.cuh"
#include "wgm_serve.cuh"

/* ------------------------------------------------------------------------ */
/* Kernel                                                                    */
/* ------------------------------------------------------------------------ */

__global__ void __launch_bounds__(1024) wgm_k_serve(wgm_launch L, wgm_serve_args A) {
  __shared__ wgm_cta c;  /* discovered view */
  __shared__ wgm_cta pc; /* persistent-job view */
  __shared__ wgm_warp_smem sm;
  __shared__ int s_task, s_req, s_rank;
  __shared__ wgm_rctx s_rc;
  __shared__ int s_claim[WGM_SERVE_FORK_MAX];
  if (!wgm_discover(L, &c)) return;
  wgm_dev_state *st = L.st;
  const int nslots = c.ngroups;
  if (c.id == 0) {
    if (threadIdx.x < 32) wgm_serve_scheduler(L, A, c.ngroups - 1, s_claim);
    __syncthreads();
    return;
  }
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      wgm_pool_enter(L, A.sd, c.id);
      wgm_spin s = wgm_idle_start(L, A.idle_ns);
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
        pc.tmp[3] = s_rc.w[WGM_RC_SERVE_SLOW];
      } else if (t == WGM_TASK_REQ) {
        s_req = __ldcg(&A.sd->slot_req[c.id]);
        s_rank = __ldcg(&A.sd->slot_rank[c.id]);
      }
    }
    __syncthreads();
    const int t = s_task;
    if (t == WGM_TASK_QUIT) break;
    if (t == WGM_TASK_PERSIST) {
      wgm_step cur = {s_rc.w[WGM_RC_TARGET], s_rc.w[WGM_RC_ROUND]};
      for (;;) {
        wgm_step nxt = cur;
        if (wgm_phase_combo(L, &pc, A, &sm, cur, &nxt) != WGM_PHASE_NEXT) break;
        if (wgm_serve_barrier(L, &pc, nxt, A, nslots, s_claim) != 1) break;
        cur = nxt;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        wgm_atom_add_acqrel_gpu(&st->k_executing[1][0], -1);
        wgm_atom_add_acqrel_sys(&L.hf->persistent_flag, -1);
      }
    } else if (t == WGM_TASK_REQ) {
      const wgm_req r = wgm_load_req(&A.dreq[s_req]);
      const int rank = s_rank;
      if (r.kind == WGM_REQ_BFS)
        wgm_req_bfs(A, r, rank, &sm);
      else if (r.kind == WGM_REQ_REDUCE)
        wgm_req_reduce(A, r, rank);
      else if (r.kind == WGM_REQ_MATMUL)
        wgm_req_matmul(A, r, rank);
      else if (r.kind == WGM_REQ_REDUCE_I32)
        wgm_req_reduce_i32(A, r, rank);
      else if (r.kind == WGM_REQ_MATMUL_I32)
        wgm_req_matmul_i32(A, r, rank);
      __syncthreads();
      if (threadIdx.x == 0) {
        int *ctl = wgm_req_ctl(A, r);
        /* the last group of the team posts the completion */
        if (wgm_atom_add_acqrel_gpu(ctl, 1) == r.groups - 1) {
          if (A.rtimes && r.id < A.max_requests)
            A.rtimes[2 * (size_t)r.id + 1] = wgm_globaltimer();
          wgm_st_release_sys(&A.completions[r.id % A.ring_size], r.id + 1);
          wgm_atom_add_acqrel_gpu(&A.sd->completed, 1);
        }
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Host side                                                                 */
/* ------------------------------------------------------------------------ */

using wgm_clk = std::chrono::steady_clock;
static uint64_t wgm_serve_now() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             wgm_clk::now().time_since_epoch())
      .count();
}

/* First-fit allocator over the request-state arena (host bookkeeping only;
 * the memory is device memory).  Admission = a successful allocation. */
struct wgm_arena_alloc {
  size_t size = 0;
  std::map<size_t, size_t> free_; /* offset -> length */
  void init(size_t n) {
    size = n;
    free_.clear();
    free_[0] = n;
  }
  bool alloc(size_t n, size_t *off) {
    n = (n + 255) & ~(size_t)255;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        *off = it->first;
        size_t rest = it->second - n, at = it->first + n;
        free_.erase(it);
        if (rest) free_[at] = rest;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t n) {
    n = (n + 255) & ~(size_t)255;
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

struct wgm_serve_req_log {
  int kind, arg0, arg1, groups;
  uint64_t arrive_ns, submit_ns, done_ns;
  size_t state_off, state_bytes;
  int64_t result_at; /* offset into results, -1 if not kept */
};

struct wgm_serve {
  wgm_runtime *rt = nullptr;
  /* the persistent job's group count sampled every millisecond of the last
   * run (CL_Communicator's groups-over-time series) */
  std::vector<std::pair<int64_t, int32_t>> gtrace;
  wgm_app *color = nullptr, *bfs = nullptr;
  /* resident datasets */
  std::vector<wgm_serve_graph> graphs;
  std::vector<long long> gE;
  int *d_rows = nullptr, *d_cols = nullptr;
  wgm_serve_graph *d_graphs = nullptr;
  float *d_vecs = nullptr, *d_mats = nullptr;
  int nvecs = 0, vec_len = 0, nmats = 0, mat_n = 0;
  int *d_ivecs = nullptr, *d_imats = nullptr; /* int32 reference variants */
  int nivecs = 0, ivec_len = 0, nimats = 0, imat_n = 0;
  /* request state */
  char *d_arena = nullptr;
  size_t arena_bytes = 0;
  wgm_arena_alloc arena;
  /* rings and words */
  int ring = 4096;
  wgm_req *ring_h = nullptr, *ring_d = nullptr;       /* mapped */
  int *comp_h = nullptr, *comp_d = nullptr;            /* mapped */
  wgm_serve_host *hs_h = nullptr, *hs_d = nullptr;     /* mapped */
  wgm_serve_dev *d_sd = nullptr;
  wgm_req *d_dreq = nullptr;
  int *d_err = nullptr;
  cudaStream_t side = nullptr;
  /* last run */
  std::vector<wgm_serve_req_log> log;
  std::vector<char> results;
  std::string diag; /* where the last failed run stood */
  unsigned long long *d_rtimes = nullptr; /* per request: device start, end */
  int rtimes_cap = 0;
  std::vector<unsigned long long> rtimes;  /* copy of the last run's */
};

static size_t wgm_req_bytes(const wgm_serve *s, int kind, int arg0) {
  size_t b = WGM_REQ_CTL_BYTES;
  if (kind == WGM_REQ_BFS) {
    const wgm_serve_graph &g = s->graphs[arg0];
    b += (size_t)((g.V + 63) & ~63) * 4 + 4 * (size_t)g.cap * 4;
  } else if (kind == WGM_REQ_MATMUL) {
    b += (size_t)s->mat_n * s->mat_n * 4;
  } else if (kind == WGM_REQ_MATMUL_I32) {
    b += (size_t)s->imat_n * s->imat_n * 4;
  }
  return b;
}

static size_t wgm_req_result_bytes(const wgm_serve *s, int kind, int arg0) {
  if (kind == WGM_REQ_BFS) return (size_t)s->graphs[arg0].V * 4;
  if (kind == WGM_REQ_MATMUL) return (size_t)s->mat_n * s->mat_n * 4;
  if (kind == WGM_REQ_MATMUL_I32) return 4 + (size_t)s->imat_n * s->imat_n * 4;
  return 4;
}

static size_t wgm_req_result_off(int kind) {
  /* reduce results and the int32 product's hash sit on line 5; the int32
   * product's C follows the control lines like the other payloads, and its
   * result is read as hash + C (line 5 is copied with the lines after it) */
  if (kind == WGM_REQ_REDUCE || kind == WGM_REQ_REDUCE_I32) return 5 * WGM_LINE * 4;
  return WGM_REQ_CTL_BYTES;
}

extern "C" int wgm_serve_destroy(wgm_serve *s) {
  if (!s) return WGM_ERR_INVALID;
  cudaSetDevice(s->rt->device);
  cudaStreamSynchronize(s->rt->stream);
  if (s->side) cudaStreamSynchronize(s->side);
  void *dev[] = {s->d_rows, s->d_cols,   s->d_graphs, s->d_vecs,  s->d_mats,   s->d_arena,
                 s->d_sd,   s->d_dreq,   s->d_err,    s->d_ivecs, s->d_imats, s->d_rtimes};
  for (void *p : dev)
    if (p) cudaFree(p);
  void *host[] = {s->ring_h, s->comp_h, s->hs_h};
  for (void *p : host)
    if (p) cudaFreeHost(p);
  if (s->side) cudaStreamDestroy(s->side);
  delete s;
  return WGM_OK;
}

extern "C" int wgm_serve_create(wgm_runtime *rt, wgm_app *color, wgm_app *bfs, int num_graphs,
                                const wgm_graph_desc *graphs, int num_vecs, int vec_len,
                                const float *vecs, int num_mats, int mat_n, const float *mats,
                                int64_t arena_bytes, wgm_serve **out) {
  if (!rt || !out || num_graphs < 0 || num_vecs < 0 || num_mats < 0 || arena_bytes < 4096 ||
      (num_graphs && !graphs) || (num_vecs && (!vecs || vec_len < 1)) ||
      (num_mats && (!mats || mat_n < 32 || mat_n % 32)) ||
      (color && color->kind != WGM_APP_PANNOTIA_COLOR) ||
      (bfs && bfs->kind != WGM_APP_LONESTAR_BFS) || (!color) != (!bfs) ||
      (color && color->rt != rt) || (bfs && bfs->rt != rt))
    return WGM_ERR_INVALID;
  *out = nullptr;
  wgm_serve *s = new (std::nothrow) wgm_serve();
  if (!s) return WGM_ERR_OOM;
  s->rt = rt;
  s->color = color;
  s->bfs = bfs;
  s->nvecs = num_vecs;
  s->vec_len = vec_len;
  s->nmats = num_mats;
  s->mat_n = mat_n;
  /* resident BFS graphs: one arena, piece layout as the Lonestar app */
  long long rows = 0, cols = 0;
  for (int g = 0; g < num_graphs; g++) {
    const wgm_graph_desc &d = graphs[g];
    if (d.num_nodes < 1 || !d.row_ptr || d.num_edges < 0 || (d.num_edges && !d.col) ||
        d.row_ptr[0] != 0 || d.row_ptr[d.num_nodes] > d.num_edges) {
      delete s;
      return WGM_ERR_INVALID;
    }
    for (int64_t e = 0; e < d.num_edges; e++)
      if (d.col[e] < 0 || d.col[e] >= d.num_nodes) {
        delete s;
        return WGM_ERR_INVALID;
      }
    wgm_serve_graph sg;
    sg.V = d.num_nodes;
    long long p = std::max<long long>(32LL, (d.num_edges + d.num_nodes - 1) / d.num_nodes);
    sg.piece = (int)p;
    sg.cap = (int)(d.num_nodes + (d.num_edges + p - 1) / p + 64);
    sg.pad = 0;
    sg.row_off = rows;
    sg.col_off = cols;
    rows += d.num_nodes + 1;
    cols += d.num_edges;
    s->graphs.push_back(sg);
    s->gE.push_back(d.num_edges);
  }
  cudaSetDevice(rt->device);
  cudaError_t e = cudaSuccess;
  auto dalloc = [&](void **p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(bytes, 256));
  };
  auto halloc = [&](void **p, size_t bytes) {
    if (e == cudaSuccess) e = cudaHostAlloc(p, bytes, cudaHostAllocMapped);
    if (e == cudaSuccess) std::memset(*p, 0, bytes);
  };
  dalloc((void **)&s->d_rows, rows * 4);
  dalloc((void **)&s->d_cols, cols * 4);
  dalloc((void **)&s->d_graphs, sizeof(wgm_serve_graph) * std::max(num_graphs, 1));
  dalloc((void **)&s->d_vecs, (size_t)num_vecs * vec_len * 4);
  dalloc((void **)&s->d_mats, (size_t)num_mats * 2 * mat_n * mat_n * 4);
  dalloc((void **)&s->d_arena, (size_t)arena_bytes);
  dalloc((void **)&s->d_sd, sizeof(wgm_serve_dev));
  dalloc((void **)&s->d_dreq, sizeof(wgm_req) * s->ring);
  dalloc((void **)&s->d_err, 2 * 4);
  halloc((void **)&s->ring_h, sizeof(wgm_req) * s->ring);
  halloc((void **)&s->comp_h, 4 * (size_t)s->ring);
  halloc((void **)&s->hs_h, sizeof(wgm_serve_host));
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->ring_d, s->ring_h, 0);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->comp_d, s->comp_h, 0);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->hs_d, s->hs_h, 0);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
  for (int g = 0; g < num_graphs && e == cudaSuccess; g++) {
    const wgm_graph_desc &d = graphs[g];
    e = cudaMemcpy(s->d_rows + s->graphs[g].row_off, d.row_ptr, (size_t)(d.num_nodes + 1) * 4,
                   cudaMemcpyHostToDevice);
    if (e == cudaSuccess && d.num_edges)
      e = cudaMemcpy(s->d_cols + s->graphs[g].col_off, d.col, (size_t)d.num_edges * 4,
                     cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess && num_graphs)
    e = cudaMemcpy(s->d_graphs, s->graphs.data(), sizeof(wgm_serve_graph) * num_graphs,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess && num_vecs)
    e = cudaMemcpy(s->d_vecs, vecs, (size_t)num_vecs * vec_len * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && num_mats)
    e = cudaMemcpy(s->d_mats, mats, (size_t)num_mats * 2 * mat_n * mat_n * 4,
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    int st = wgm_cuda_fail(rt, e);
    wgm_serve_destroy(s);
    return st;
  }
  /* pageable-source copies may still be in flight when cudaMemcpy returns;
   * the serving kernel runs on the runtime's non-blocking stream */
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) {
    int st = wgm_cuda_fail(rt, e);
    wgm_serve_destroy(s);
    return st;
  }
  s->arena_bytes = (size_t)arena_bytes;
  *out = s;
  return WGM_OK;
}

/* Where a failed run stood: host counters, then the serving and pool words
 * after the kernel ended. */
static void wgm_serve_diag_fill(wgm_serve *s, const char *why, int64_t head, size_t inflight,
                                size_t waiting, size_t next, size_t narr) {
  wgm_runtime *rt = s->rt;
  wgm_serve_dev sd;
  std::memset(&sd, 0, sizeof(sd));
  int avail = -1, lock = -1, tk = -1, exe = -1, err[2] = {0, 0};
  cudaMemcpy(&sd, s->d_sd, sizeof(sd), cudaMemcpyDeviceToHost);
  cudaMemcpy(&avail, &rt->st->available_workgroups, 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(&lock, &rt->st->pool_lock, 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(&tk, &rt->st->groups_to_kill, 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(&exe, &rt->st->k_executing[1][0], 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(err, s->d_err, 8, cudaMemcpyDeviceToHost);
  char buf[640];
  std::snprintf(buf, sizeof(buf),
                "%s: host head=%lld inflight=%zu waiting=%zu arrivals=%zu/%zu; device "
                "seen=%d started=%d completed=%d pending=%d persist_reps=%d kills=%d forks=%d "
                "available=%d pool_lock=%d to_kill=%d executing=%d discovered=%d; team err=%d "
                "site=%d; device status=%d site=%d detail=%d",
                why, (long long)head, inflight, waiting, next, narr, s->hs_h->seen,
                s->hs_h->started, sd.completed, sd.pending, sd.persist_done, sd.kills, sd.forks,
                avail, lock, tk, exe, rt->hf->discovered, err[0], err[1], rt->hf->status,
                rt->hf->status_site, rt->hf->status_detail);
  s->diag = buf;
}

extern "C" int wgm_serve_set_int_data(wgm_serve *s, int num_ivecs, int ivec_len,
                                      const int32_t *ivecs, int num_imats, int imat_n,
                                      const int32_t *imats) {
  if (!s || num_ivecs < 0 || num_imats < 0 || (num_ivecs && (!ivecs || ivec_len < 1)) ||
      (num_imats && (!imats || imat_n < 32 || imat_n % 32)))
    return WGM_ERR_INVALID;
  cudaSetDevice(s->rt->device);
  cudaStreamSynchronize(s->rt->stream);
  if (s->d_ivecs) cudaFree(s->d_ivecs);
  if (s->d_imats) cudaFree(s->d_imats);
  s->d_ivecs = s->d_imats = nullptr;
  cudaError_t e = cudaMalloc((void **)&s->d_ivecs, std::max<size_t>(4, (size_t)num_ivecs * ivec_len * 4));
  if (e == cudaSuccess)
    e = cudaMalloc((void **)&s->d_imats,
                   std::max<size_t>(4, (size_t)num_imats * 2 * imat_n * imat_n * 4));
  if (e == cudaSuccess && num_ivecs)
    e = cudaMemcpy(s->d_ivecs, ivecs, (size_t)num_ivecs * ivec_len * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && num_imats)
    e = cudaMemcpy(s->d_imats, imats, (size_t)num_imats * 2 * imat_n * imat_n * 4,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaDeviceSynchronize(); /* pageable sources */
  if (e != cudaSuccess) return wgm_cuda_fail(s->rt, e);
  s->nivecs = num_ivecs;
  s->ivec_len = ivec_len;
  s->nimats = num_imats;
  s->imat_n = imat_n;
  return WGM_OK;
}

static int wgm_serve_fail_run(wgm_serve *s, int status, const char *why, int64_t head,
                              size_t inflight, size_t waiting, size_t next, size_t narr) {
  wgm_set_abort(s->rt, 1);
  __atomic_store_n(&s->hs_h->quit, 1, __ATOMIC_RELEASE);
  cudaStreamSynchronize(s->rt->stream);
  wgm_serve_diag_fill(s, why, head, inflight, waiting, next, narr);
  wgm_set_abort(s->rt, 0);
  int ds = 0, site = 0;
  wgm_finish_launch(s->rt, &ds, &site);
  return status;
}

extern "C" int wgm_serve_run(wgm_serve *s, const wgm_serve_config *cfg, wgm_serve_stats *st) {
  if (!s || !cfg || cfg->rate_per_s < 0 || cfg->duration_s < 0 || cfg->reps < 0 ||
      cfg->frac_bfs < 0 || cfg->frac_reduce < 0 || cfg->frac_bfs + cfg->frac_reduce > 1.0 + 1e-9 ||
      (cfg->reps > 0 && !s->color))
    return WGM_ERR_INVALID;
  const double fb = cfg->frac_bfs, fr = cfg->frac_reduce;
  if (cfg->rate_per_s > 0 && ((fb > 0 && s->graphs.empty()) || (fr > 0 && s->nvecs == 0) ||
                              (fb + fr < 1.0 - 1e-9 && s->nmats == 0)))
    return WGM_ERR_INVALID;
  if (cfg->frac_int < 0 || cfg->frac_int > 1 ||
      (cfg->rate_per_s > 0 && cfg->frac_int > 0 &&
       ((fr > 0 && s->nivecs == 0) || (fb + fr < 1.0 - 1e-9 && s->nimats == 0))))
    return WGM_ERR_INVALID;
  wgm_runtime *rt = s->rt;
  cudaSetDevice(rt->device);
  int block = cfg->threads_per_wg > 0 ? cfg->threads_per_wg : rt->cfg.threads_per_wg;
  if (block < 32 || block > 1024 || block % 32) return WGM_ERR_INVALID;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wgm_k_serve, block, 0);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  const int grid = std::min(per_sm * rt->prop.multiProcessorCount, WGM_MAX_GROUPS);
  if (grid < 2) return WGM_ERR_INVALID;
  const int lpg_max = grid - 1;
  auto team = [&](int g) { return std::max(1, std::min(g, std::min(lpg_max, WGM_SERVE_FORK_MAX))); };
  const int tb = team(cfg->bfs_groups > 0 ? cfg->bfs_groups : 4);
  const int tr = team(cfg->reduce_groups > 0 ? cfg->reduce_groups : 4);
  const int tm = team(cfg->matmul_groups > 0 ? cfg->matmul_groups : 4);
  const int max_inflight = std::max(1, std::min(cfg->max_in_flight > 0 ? cfg->max_in_flight : 256,
                                                s->ring - 96));

  /* the request stream, drawn up front: Poisson arrivals, seeded mix */
  struct arrival {
    uint64_t t;
    int kind, arg0, arg1;
  };
  std::vector<arrival> arr;
  if (cfg->rate_per_s > 0 && cfg->duration_s > 0) {
    std::mt19937_64 rng(cfg->seed);
    std::exponential_distribution<double> gap(cfg->rate_per_s);
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    double t = 0;
    for (;;) {
      t += gap(rng);
      if (t > cfg->duration_s) break;
      arrival a;
      a.t = (uint64_t)(t * 1e9);
      double x = u01(rng);
      a.kind = x < fb ? WGM_REQ_BFS : (x < fb + fr ? WGM_REQ_REDUCE : WGM_REQ_MATMUL);
      if (a.kind != WGM_REQ_BFS && u01(rng) < cfg->frac_int)
        a.kind = a.kind == WGM_REQ_REDUCE ? WGM_REQ_REDUCE_I32 : WGM_REQ_MATMUL_I32;
      a.arg1 = 0;
      if (a.kind == WGM_REQ_BFS) {
        a.arg0 = (int)(rng() % s->graphs.size());
        a.arg1 = (int)(rng() % (uint64_t)s->graphs[a.arg0].V);
      } else if (a.kind == WGM_REQ_REDUCE) {
        a.arg0 = (int)(rng() % (uint64_t)s->nvecs);
      } else if (a.kind == WGM_REQ_MATMUL) {
        a.arg0 = (int)(rng() % (uint64_t)s->nmats);
      } else if (a.kind == WGM_REQ_REDUCE_I32) {
        a.arg0 = (int)(rng() % (uint64_t)s->nivecs);
      } else {
        a.arg0 = (int)(rng() % (uint64_t)s->nimats);
      }
      arr.push_back(a);
    }
  }
  for (const arrival &a : arr)
    if (wgm_req_bytes(s, a.kind, a.arg0) > s->arena_bytes) return WGM_ERR_OOM;
  if ((int)arr.size() > s->rtimes_cap) {
    if (s->d_rtimes) cudaFree(s->d_rtimes);
    s->d_rtimes = nullptr;
    s->rtimes_cap = 0;
    cudaError_t ea = cudaMalloc((void **)&s->d_rtimes, 16 * arr.size());
    if (ea != cudaSuccess) return wgm_cuda_fail(rt, ea);
    s->rtimes_cap = (int)arr.size();
  }

  /* reset the serving words */
  std::memset(s->ring_h, 0, sizeof(wgm_req) * s->ring);
  std::memset(s->comp_h, 0, 4 * (size_t)s->ring);
  std::memset((void *)s->hs_h, 0, sizeof(wgm_serve_host));
  /* stream-ordered before the launch (the runtime's stream does not wait
   * for the legacy stream): the serving words, the error word, and the pool
   * words of the runtime state, which a previous megakernel may have left
   * elsewhere */
  cudaStream_t rs = rt->stream;
  e = cudaMemsetAsync(s->d_sd, 0, sizeof(wgm_serve_dev), rs);
  if (e == cudaSuccess) e = cudaMemsetAsync(&rt->st->available_workgroups, 0, 4, rs);
  if (e == cudaSuccess) e = cudaMemsetAsync(&rt->st->pool_lock, 0, 4, rs);
  if (e == cudaSuccess) e = cudaMemsetAsync(&rt->st->bar_count, 0, 4, rs);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->d_err, 0, 8, rs);
  if (e != cudaSuccess) return wgm_cuda_fail(rt, e);
  s->arena.init(s->arena_bytes);
  s->diag.clear();
  s->log.clear();
  s->results.clear();
  s->gtrace.clear();

  wgm_serve_args A;
  std::memset(&A, 0, sizeof(A));
  if (s->color) {
    wgm_mega_args M;
    std::memset(&M, 0, sizeof(M));
    int r1 = wgm_app_fill_mega(s->color, &M);
    int r2 = wgm_app_fill_mega(s->bfs, &M);
    if (r1 || r2) return WGM_ERR_INVALID;
    A.color = M.color;
    A.ls = M.ls;
  }
  A.reps = s->color ? cfg->reps : 0;
  /* by default the resident job starts on every group but the reserve, so
   * the first requests need not wait for a kill */
  A.persist_groups =
      A.reps > 0 ? (cfg->persist_groups > 0 ? cfg->persist_groups
                                            : std::max(1, lpg_max - std::max(0, cfg->reserve)))
                 : 0;
  A.ring = s->ring_d;
  A.ring_size = s->ring;
  A.completions = s->comp_d;
  A.hs = s->hs_d;
  A.sd = s->d_sd;
  A.dreq = s->d_dreq;
  A.arena = s->d_arena;
  A.g_rows = s->d_rows;
  A.g_cols = s->d_cols;
  A.graphs = s->d_graphs;
  A.vecs = s->d_vecs;
  A.vec_len = s->vec_len;
  A.mats = s->d_mats;
  A.mat_n = s->mat_n;
  A.ivecs = s->d_ivecs;
  A.ivec_len = s->ivec_len;
  A.imats = s->d_imats;
  A.imat_n = s->imat_n;
  A.err = s->d_err;
  A.reserve = std::max(0, cfg->reserve);
  A.persist_max = cfg->persist_max_groups > 0 ? cfg->persist_max_groups : lpg_max;
  A.persist_groups = std::min(A.persist_groups, A.persist_max);
  A.rtimes = s->d_rtimes;
  A.max_requests = s->rtimes_cap;
  const uint64_t run_budget = rt->cfg.run_timeout_ns ? rt->cfg.run_timeout_ns : 120000000000ull;
  A.idle_ns = run_budget;
  __atomic_store_n(&rt->hf->persistent_flag, 0, __ATOMIC_RELEASE);

  wgm_launch L = wgm_make_launch(rt, grid, 0, 0);
  const uint64_t t0 = wgm_serve_now();
  wgm_k_serve<<<grid, block, 0, rt->stream>>>(L, A);
  if ((e = cudaGetLastError()) != cudaSuccess) return wgm_cuda_fail(rt, e);

  /* host loop: arrivals, admission, doorbell, completions */
  std::vector<int> waiting;     /* arrived, not admitted (arrival indices, FIFO) */
  size_t wait_head = 0;
  std::vector<int64_t> inflight; /* log indices */
  int64_t head = 0, waited_mem = 0;
  size_t next = 0;
  bool stream_open = true;
  uint64_t persist_done_at = 0, next_sample = 0;
  const int reps = A.reps;
  for (;;) {
    const uint64_t now = wgm_serve_now() - t0;
    /* cl_communicator.h:186-200: the persistent group count every 1 ms */
    if (reps > 0 && !persist_done_at && now >= next_sample) {
      s->gtrace.emplace_back((int64_t)now,
                             (int32_t)__atomic_load_n(&s->hs_h->persist_groups, __ATOMIC_ACQUIRE));
      next_sample = now + 1000000ull;
    }
    if (now > run_budget)
      return wgm_serve_fail_run(s, WGM_ERR_TIMEOUT, "run budget", head, inflight.size(),
                                waiting.size() - wait_head, next, arr.size());
    if (__atomic_load_n(&rt->hf->status, __ATOMIC_ACQUIRE) != 0)
      return wgm_serve_fail_run(s, WGM_ERR_TIMEOUT, "device failure", head, inflight.size(),
                                waiting.size() - wait_head, next, arr.size());
    if (reps > 0 && !persist_done_at &&
        __atomic_load_n(&s->hs_h->persist_reps, __ATOMIC_ACQUIRE) >= reps) {
      persist_done_at = now;
      stream_open = false;
    }
    if (stream_open && next == arr.size()) stream_open = false;
    while (stream_open && next < arr.size() && arr[next].t <= now) waiting.push_back((int)next++);
    /* admission in arrival order: ring space, then arena memory */
    int64_t oldest = head;
    for (int64_t li : inflight) oldest = std::min(oldest, li);
    /* ring slots are reused: never run more than ring-1 ids ahead of the
     * oldest unfinished request */
    while (wait_head < waiting.size() && (int64_t)inflight.size() < max_inflight &&
           head - oldest < s->ring - 1) {
      const arrival &a = arr[waiting[wait_head]];
      const size_t bytes = wgm_req_bytes(s, a.kind, a.arg0);
      size_t off = 0;
      if (!s->arena.alloc(bytes, &off)) {
        waited_mem++;
        break;
      }
      wgm_serve_req_log lg;
      lg.kind = a.kind;
      lg.arg0 = a.arg0;
      lg.arg1 = a.arg1;
      lg.groups = a.kind == WGM_REQ_BFS ? tb
                  : (a.kind == WGM_REQ_REDUCE || a.kind == WGM_REQ_REDUCE_I32) ? tr
                                                                               : tm;
      if (a.kind == WGM_REQ_BFS && cfg->bfs_edges_per_group > 0)
        lg.groups = team((int)std::min<long long>(
            tb, (s->gE[a.arg0] + cfg->bfs_edges_per_group - 1) / cfg->bfs_edges_per_group));
      lg.arrive_ns = a.t;
      lg.submit_ns = now;
      lg.done_ns = 0;
      lg.state_off = off;
      lg.state_bytes = bytes;
      lg.result_at = -1;
      wgm_req &r = s->ring_h[head % s->ring];
      std::memset(&r, 0, sizeof(r));
      r.kind = a.kind;
      r.groups = lg.groups;
      r.arg0 = a.arg0;
      r.arg1 = a.arg1;
      r.state_off = (long long)off;
      r.id = (int)head;
      s->log.push_back(lg);
      inflight.push_back((int64_t)s->log.size() - 1);
      head++;
      __atomic_store_n(&s->hs_h->head, (int)head, __ATOMIC_RELEASE);
      wait_head++;
    }
    /* completions */
    for (size_t k = 0; k < inflight.size();) {
      const int64_t li = inflight[k];
      const int id = (int)li; /* ids are log indices */
      if (__atomic_load_n(&s->comp_h[id % s->ring], __ATOMIC_ACQUIRE) == id + 1) {
        wgm_serve_req_log &lg = s->log[li];
        lg.done_ns = wgm_serve_now() - t0;
        if (cfg->keep_results) {
          const size_t rb = wgm_req_result_bytes(s, lg.kind, lg.arg0);
          lg.result_at = (int64_t)s->results.size();
          s->results.resize(s->results.size() + rb);
          if (lg.kind == WGM_REQ_MATMUL_I32) { /* hash (line 5), then C */
            e = cudaMemcpyAsync(s->results.data() + lg.result_at,
                                s->d_arena + lg.state_off + 5 * WGM_LINE * 4, 4,
                                cudaMemcpyDeviceToHost, s->side);
            if (e == cudaSuccess)
              e = cudaMemcpyAsync(s->results.data() + lg.result_at + 4,
                                  s->d_arena + lg.state_off + WGM_REQ_CTL_BYTES, rb - 4,
                                  cudaMemcpyDeviceToHost, s->side);
          } else {
            e = cudaMemcpyAsync(s->results.data() + lg.result_at,
                                s->d_arena + lg.state_off + wgm_req_result_off(lg.kind), rb,
                                cudaMemcpyDeviceToHost, s->side);
          }
          if (e == cudaSuccess) e = cudaStreamSynchronize(s->side);
          if (e != cudaSuccess)
            return wgm_serve_fail_run(s, wgm_cuda_fail(rt, e), "result copy", head,
                                      inflight.size(), 0, next, arr.size());
        }
        s->arena.release(lg.state_off, lg.state_bytes);
        inflight[k] = inflight.back();
        inflight.pop_back();
      } else {
        k++;
      }
    }
    if (!stream_open && wait_head == waiting.size() && inflight.empty() &&
        (reps == 0 || persist_done_at))
      break;
  }
  __atomic_store_n(&s->hs_h->quit, 1, __ATOMIC_RELEASE);
  int status = wgm_synchronize(rt);
  if (status) wgm_serve_diag_fill(s, "after quit", head, inflight.size(), 0, next, arr.size());
  const uint64_t t_end = wgm_serve_now() - t0;
  int herr[2] = {0, 0};
  if (cudaMemcpy(herr, s->d_err, 8, cudaMemcpyDeviceToHost) == cudaSuccess && herr[0] && !status)
    status = wgm_status_from_device(herr[0]);
  wgm_serve_dev sd;
  if (cudaMemcpy(&sd, s->d_sd, sizeof(sd), cudaMemcpyDeviceToHost) != cudaSuccess)
    std::memset(&sd, 0, sizeof(sd));
  s->rtimes.assign(2 * s->log.size(), 0ull);
  if (!s->log.empty() && s->d_rtimes)
    cudaMemcpy(s->rtimes.data(), s->d_rtimes, 16 * s->log.size(), cudaMemcpyDeviceToHost);
  if (st) {
    std::memset(st, 0, sizeof(*st));
    std::vector<double> lat, exe, wait;
    for (size_t i = 0; i < s->log.size(); i++) {
      const auto &lg = s->log[i];
      const unsigned long long t0 = s->rtimes[2 * i], t1 = s->rtimes[2 * i + 1];
      if (!lg.done_ns || !t0 || t1 < t0) continue;
      const double ex = (double)(t1 - t0) / 1000.0;
      exe.push_back(ex);
      wait.push_back(std::max(0.0, (double)(lg.done_ns - lg.arrive_ns) / 1000.0 - ex));
    }
    auto pct = [](std::vector<double> &v, double p) {
      if (v.empty()) return 0.0;
      std::sort(v.begin(), v.end());
      size_t i = (size_t)std::ceil(p * (double)v.size()) - 1;
      return v[std::min(i, v.size() - 1)];
    };
    st->exec_p50_us = pct(exe, 0.5);
    st->exec_p99_us = pct(exe, 0.99);
    st->wait_p50_us = pct(wait, 0.5);
    st->wait_p99_us = pct(wait, 0.99);
    uint64_t first = ~0ull, last = 0;
    for (const auto &lg : s->log) {
      if (!lg.done_ns) continue;
      lat.push_back((double)(lg.done_ns - lg.arrive_ns) / 1000.0);
      first = std::min(first, lg.arrive_ns);
      last = std::max(last, lg.done_ns);
    }
    st->arrived = (int64_t)next;
    st->completed = (int64_t)lat.size();
    st->waited_for_memory = waited_mem;
    if (!lat.empty()) {
      std::sort(lat.begin(), lat.end());
      auto q = [&](double p) {
        size_t i = (size_t)std::ceil(p * (double)lat.size()) - 1;
        return lat[std::min(i, lat.size() - 1)];
      };
      st->lat_p50_us = q(0.50);
      st->lat_p99_us = q(0.99);
      double sum = 0;
      for (double x : lat) sum += x;
      st->lat_mean_us = sum / (double)lat.size();
      st->lat_max_us = lat.back();
      st->stream_s = (double)(last - first) / 1e9;
      st->achieved_rate = st->stream_s > 0 ? (double)lat.size() / st->stream_s : 0;
    }
    st->persist_ms = persist_done_at ? (double)persist_done_at / 1e6 : 0;
    st->persist_reps = sd.persist_done;
    st->kills = sd.kills;
    st->forks = sd.forks;
    if (!s->gtrace.empty()) {
      double sum = 0;
      int mn = INT_MAX;
      for (const auto &p : s->gtrace) {
        sum += p.second;
        mn = std::min(mn, (int)p.second);
      }
      st->persist_groups_mean = sum / (double)s->gtrace.size();
      st->persist_groups_min = mn;
    }
    st->groups = __atomic_load_n(&rt->hf->discovered, __ATOMIC_ACQUIRE);
    st->run_ms = (double)t_end / 1e6;
  }
  return status;
}

extern "C" int wgm_serve_requests(wgm_serve *s, int64_t *count, int32_t *kind, int32_t *arg0,
                                  int32_t *arg1, int64_t *latency_ns, int32_t *groups) {
  if (!s || !count) return WGM_ERR_INVALID;
  const int64_t n = (int64_t)s->log.size();
  if (kind || arg0 || arg1 || latency_ns || groups) {
    if (*count < n) return WGM_ERR_INVALID;
    for (int64_t i = 0; i < n; i++) {
      const auto &lg = s->log[i];
      if (kind) kind[i] = lg.kind;
      if (arg0) arg0[i] = lg.arg0;
      if (arg1) arg1[i] = lg.arg1;
      if (latency_ns) latency_ns[i] = lg.done_ns ? (int64_t)(lg.done_ns - lg.arrive_ns) : -1;
      if (groups) groups[i] = lg.groups;
    }
  }
  *count = n;
  return WGM_OK;
}

extern "C" int wgm_serve_result(wgm_serve *s, int64_t i, void *out, int64_t bytes) {
  if (!s || !out || i < 0 || i >= (int64_t)s->log.size()) return WGM_ERR_INVALID;
  const auto &lg = s->log[i];
  if (lg.result_at < 0) return WGM_ERR_STATE;
  const size_t rb = wgm_req_result_bytes(s, lg.kind, lg.arg0);
  if (bytes < (int64_t)rb) return WGM_ERR_INVALID;
  std::memcpy(out, s->results.data() + lg.result_at, rb);
  return WGM_OK;
}

extern "C" int wgm_serve_diag(wgm_serve *s, char *buf, size_t len) {
  if (!s || !buf || len == 0) return WGM_ERR_INVALID;
  std::snprintf(buf, len, "%s", s->diag.c_str());
  return WGM_OK;
}

/* Device execution time of each request of the last run (from the moment the
 * scheduler gave it its team to the moment its last group finished), ns; -1
 * where not recorded. */
extern "C" int wgm_serve_exec_times(wgm_serve *s, int64_t n, int64_t *exec_ns) {
  if (!s || !exec_ns || n < (int64_t)s->log.size()) return WGM_ERR_INVALID;
  for (size_t i = 0; i < s->log.size(); i++) {
    const unsigned long long t0 = i * 2 < s->rtimes.size() ? s->rtimes[2 * i] : 0;
    const unsigned long long t1 = i * 2 + 1 < s->rtimes.size() ? s->rtimes[2 * i + 1] : 0;
    exec_ns[i] = (t0 && t1 >= t0 && s->log[i].done_ns) ? (int64_t)(t1 - t0) : -1;
  }
  return WGM_OK;
}

/* The groups-over-time series of the last run (print_groups_time_data,
 * cl_communicator.h:241): sample k at t_ns[k] (from the launch) saw the
 * persistent job on groups[k] groups.  NULL arrays: *count only. */
extern "C" int wgm_serve_groups_trace(wgm_serve *s, int64_t *t_ns, int32_t *groups,
                                      int64_t capacity, int64_t *count) {
  if (!s || !count) return WGM_ERR_INVALID;
  *count = (int64_t)s->gtrace.size();
  if (!t_ns && !groups) return WGM_OK;
  const int64_t n = std::min<int64_t>(capacity, (int64_t)s->gtrace.size());
  for (int64_t k = 0; k < n; k++) {
    if (t_ns) t_ns[k] = s->gtrace[k].first;
    if (groups) groups[k] = s->gtrace[k].second;
  }
  return WGM_OK;
}
