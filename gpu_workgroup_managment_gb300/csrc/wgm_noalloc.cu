/*
 * wgm_bfs_noalloc: the persistent Lonestar BFS for callers that cannot
 * allocate GPU memory.
 *
 * Who needs it: a host application that hands every byte of device memory to
 * its own pool allocator and forbids third-party cudaMalloc (a serving
 * framework that budgets the whole GPU, a plugin host that accounts for all
 * allocations), or a latency-critical loop that cannot afford the device-wide
 * synchronisation cudaFree (and sometimes cudaMalloc) implies.  The regular
 * entry points allocate through wgm_runtime_create / wgm_app_create; this one
 * allocates nothing, neither device nor pinned host memory.
 *
 * Its scratch (worklists, level counters, the discovery/barrier state and the
 * status words) lives in one file-scope static __device__ array sized for
 * WGM_NOALLOC_MAX_NODES vertices (about 8.5 MB).  Every GPU that loads
 * libwgm.so holds that array until the process exits.
 *
 * The first call on a device (with that device current) looks the array's
 * device address up with cudaGetSymbolAddress; in host code the array's name
 * is only a host-side stand-in, never a device address.  Make that first call
 * before any stream capture.  Every call waits for its BFS to finish (it
 * reads the status word back and synchronises `stream`), which a stream
 * under capture cannot do: on a capturing stream the call returns
 * WGM_ERR_STATE at once and leaves the capture as it was.  All calls share
 * the one array and it keeps the last call's contents: each call clears the
 * words that must start at zero, and two calls whose kernels overlap on the
 * GPU race on the array, so the caller must keep calls on one device ordered
 * (one stream, or synchronised).  Calls from several host threads are
 * serialised per device.
 */
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/wgm.h"
#include "wgm_kernels.cuh"

namespace {

/* Worklist capacity per level: V + E/piece pieces with piece >= E/V, so at
 * most 2V (plus slack) for any graph of WGM_NOALLOC_MAX_NODES vertices. */
constexpr int kCap = 2 * WGM_NOALLOC_MAX_NODES + 64;

struct wgm_noalloc_scratch {
  wgm_dev_state st;      /* discovery + barrier state */
  wgm_host_flags flags;  /* status words (device-resident here) */
  int cnt[3 * WGM_LINE]; /* piece counters by level mod 3 */
  int levels;
  int pad[WGM_LINE - 1];
  int wl_start[2 * kCap]; /* two worklists of pieces (first edge, count) */
  int wl_cnt[2 * kCap];
};

constexpr int kMaxDevices = 64;

struct wgm_noalloc_device {
  std::mutex mu;                      /* orders the calls on this device */
  bool ready = false;
  wgm_noalloc_scratch *ptr = nullptr; /* device address of the array */
  int gen = 0;                        /* launch generation of this device */
  int grid = 0;
};

wgm_noalloc_device g_dev[kMaxDevices];

}  // namespace

static __device__ __align__(256) unsigned char
    wgm_noalloc_scratch_mem[sizeof(wgm_noalloc_scratch)];

/* Per-device set-up, with `dev` current: look up the array's device address
 * and the launch size.  Called by the first wgm_bfs_noalloc on each device. */
static int wgm_noalloc_setup(int dev, wgm_noalloc_device *d) {
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, wgm_noalloc_scratch_mem) != cudaSuccess || !p)
    return WGM_ERR_CUDA;
  int sms = 0, per_sm = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return WGM_ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wgm_kernel_fn(WGM_K_BFS), 256, 0) !=
      cudaSuccess)
    return WGM_ERR_CUDA;
  long grid = (long)sms * per_sm;
  if (grid > WGM_MAX_GROUPS) grid = WGM_MAX_GROUPS;
  if (grid < 1) return WGM_ERR_CUDA;
  d->ptr = static_cast<wgm_noalloc_scratch *>(p);
  d->grid = (int)grid;
  d->gen = 0;
  d->ready = true;
  return WGM_OK;
}

extern "C" int wgm_bfs_noalloc(const int32_t *d_row_ptr, const int32_t *d_col,
                               int32_t num_nodes, int64_t num_edges, int32_t source,
                               uint32_t *d_dist, void *stream) {
  if (num_nodes < 1 || num_nodes > WGM_NOALLOC_MAX_NODES) return WGM_ERR_INVALID;
  if (!d_row_ptr || !d_dist || num_edges < 0 || (num_edges > 0 && !d_col))
    return WGM_ERR_INVALID;
  if (source < 0 || source >= num_nodes) return WGM_ERR_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return WGM_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return WGM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  /* The status read-back and the stream synchronisation below would fail on
   * a capturing stream and invalidate the caller's capture. */
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return WGM_ERR_STATE;

  wgm_noalloc_device *d = &g_dev[dev];
  std::lock_guard<std::mutex> lock(d->mu);
  if (!d->ready) {
    int st = wgm_noalloc_setup(dev, d);
    if (st) return st;
  }
  wgm_noalloc_scratch *sc = d->ptr;

  /* Words that must read zero at launch: the error word and the status. */
  if (cudaMemsetAsync(&sc->st.dev_error, 0, sizeof(int), s) != cudaSuccess ||
      cudaMemsetAsync(&sc->flags, 0, sizeof(wgm_host_flags), s) != cudaSuccess)
    return WGM_ERR_CUDA;

  wgm_launch L;
  std::memset(&L, 0, sizeof(L));
  L.st = &sc->st;
  L.hf = &sc->flags;
  L.spin_ns = 2000000000ull;
  L.window_ns = 200000ull;
  L.gen = ++d->gen;
  /* Wrap by an even amount, as the runtime's launches do: the discovery
   * slot parity keeps alternating and no stale `published` value matches a
   * new generation. */
  if (d->gen >= (1 << 29)) d->gen -= (1 << 28);
  L.expected = d->grid;
  L.disc_mode = WGM_DISCOVERY_TICKET;
  L.barrier_kind = WGM_BARRIER_SENSE;
  L.tree_fanin = 8;

  wgm_lonestar_args a;
  std::memset(&a, 0, sizeof(a));
  a.V = num_nodes;
  a.row = d_row_ptr;
  a.col = d_col;
  a.wt = nullptr;
  a.dist = d_dist;
  int64_t avg = (num_edges + num_nodes - 1) / num_nodes;
  a.piece = (int)(avg > 32 ? avg : 32);
  a.cap = kCap;
  a.wl_start = sc->wl_start;
  a.wl_cnt = sc->wl_cnt;
  a.wl_u = nullptr;
  a.cnt = sc->cnt;
  a.stamp = nullptr;
  a.source = source;
  a.levels_out = &sc->levels;
  if (wgm_launch_lonestar(false, L, a, d->grid, 256, s) != cudaSuccess) return WGM_ERR_CUDA;

  int status = 0;
  if (cudaMemcpyAsync(&status, &sc->flags.status, sizeof(int), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return WGM_ERR_CUDA;
  if (status != WGM_DEV_OK) {
    /* A failed launch can leave barrier counters mid-flight: clear the whole
     * runtime state and restart the generations. */
    if (cudaMemsetAsync(&sc->st, 0, sizeof(wgm_dev_state), s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return WGM_ERR_CUDA;
    d->gen = 0;
    return status == WGM_DEV_TIMEOUT ? WGM_ERR_TIMEOUT
           : status == WGM_DEV_OVERFLOW ? WGM_ERR_OVERFLOW
                                        : WGM_ERR_INVALID;
  }
  return WGM_OK;
}
