/*
 * wgm.h - C-ABI of the GB300 cooperative-kernel runtime (libwgm.so).
 *
 * Drop-in boundary for the reference's persistent path (reference paths are
 * relative to the reference project):
 *   - host runtime:  src/scheduler_rt/rt_host/cl_scheduler.h:7-88,
 *                    src/scheduler_rt/rt_host/discovery.h:6-29,
 *                    src/scheduler_rt/rt_host/cl_communicator.h:19-465,
 *                    src/host_skeleton/skel.cpp:127-240 (reset/occupancy helpers);
 *   - app plugins:   src/lonestar/graph_apps/{bfs,sssp}/*.h,
 *                    src/pannotia/graph_apps/{color,mis,sssp}/*.h,
 *                    src/non_persistent_kernels/{matmult,reduce}/*.h;
 *   - microbenchmark: src/test_suite/os_freq/host/os_freq.cpp:274-330.
 * Each declaration names the reference interface it replaces.
 *
 * Conventions: every call returns an int status (WGM_OK or a negative
 * WGM_ERR_*); nothing calls exit().  Pointers are host pointers unless the
 * name says _device.  A runtime object may be used from one thread at a time,
 * except wgm_comm_* calls which are internally locked.
 */
#ifndef WGM_H
#define WGM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference calls exit(1) instead: rt_host/ggc_ocl.h:11-18) */
#define WGM_OK 0
#define WGM_ERR_INVALID (-1)
#define WGM_ERR_TOO_MANY_GROUPS (-2) /* cl_communicator.h:125-130,209-214 */
#define WGM_ERR_TIMEOUT (-3)
#define WGM_ERR_OOM (-4)
#define WGM_ERR_CUDA (-5)
#define WGM_ERR_OVERFLOW (-6)
#define WGM_ERR_NO_DEVICE (-7)
#define WGM_ERR_ABORTED (-8)
#define WGM_ERR_STATE (-9)
/* Device-side result of the kernel API (wgm_device.cuh), not an error: this
 * group left the persistent task at a resizing barrier or offer_kill. */
#define WGM_KILLED 1

/* ---- discovery / barrier flavours */
#define WGM_DISCOVERY_TICKET 0
#define WGM_DISCOVERY_REFERENCE 1
#define WGM_BARRIER_SENSE 0
#define WGM_BARRIER_XF 1
#define WGM_BARRIER_TREE 2
#define WGM_BARRIER_COUNT 3 /* monotonic arrival counter, waiters poll it */
#define WGM_BARRIER_SPREAD 4 /* counter, generation released on 16 lines */
#define WGM_BARRIER_AUTO 5   /* COUNT up to 384 groups, SENSE above (the default) */
#define WGM_BARRIER_CLUSTER 6 /* CTAs of a thread-block cluster meet at the hardware
                                 cluster barrier, one leader per cluster at a counting
                                 barrier (wgm_barrier_bench_cluster) */

/* ---- persistent apps (the reference selects them by macro, skel.cpp:50-77) */
#define WGM_APP_LONESTAR_BFS 1
#define WGM_APP_LONESTAR_SSSP 2
#define WGM_APP_PANNOTIA_COLOR 3
#define WGM_APP_PANNOTIA_MIS 4
#define WGM_APP_PANNOTIA_SSSP 5
#define WGM_APP_PAGERANK 6
#define WGM_APP_OCTREE 7 /* work-stealing octree build (test_suite/final_octree) */
#define WGM_APP_CONNECT_FOUR 8 /* work-stealing look-ahead (test_suite/connect_four) */
#define WGM_APP_PANNOTIA_BC 9  /* betweenness centrality (pannotia/graph_apps/bc) */

typedef struct wgm_runtime wgm_runtime;
typedef struct wgm_app wgm_app;
typedef struct wgm_host_graph wgm_host_graph;

/* Runtime configuration: the reference's gflags of skel.cpp:21-44 that apply
 * to the persistent path, plus the GB300 knobs. */
typedef struct wgm_config {
  int device;
  int threads_per_wg;          /* skel.cpp:39 */
  int num_wgs;                 /* skel.cpp:40; <=0: every co-resident CTA */
  int use_query_barrier;       /* skel.cpp:34 */
  int non_persistent_wgs;      /* skel.cpp:30 */
  int non_persistent_frequency_ms; /* skel.cpp:32 */
  int skip_tasks;              /* skel.cpp:31 */
  int host_handshake;          /* standalone.cl:277-289 handshake on/off */
  int discovery_mode;          /* WGM_DISCOVERY_* */
  int discovery_extra_rounds;  /* discovery.cl:43 (reference mode) */
  int barrier_kind;            /* WGM_BARRIER_* */
  int tree_fanin;              /* groups per leaf of WGM_BARRIER_TREE */
  int hub_threshold;           /* degree above which edges spread grid-wide */
  uint64_t spin_timeout_ns;    /* budget of every device wait */
  uint64_t run_timeout_ns;     /* host budget of one blocking run; then abort */
  uint64_t discovery_window_ns;/* ticket discovery closing window */
} wgm_config;

/* Statistics of one persistent run (skel.cpp:346-354 records time, error and
 * occupancy per iteration). */
typedef struct wgm_run_stats {
  int groups;          /* discovered groups that ran the task */
  int rounds;          /* levels / rounds / iterations executed */
  int device_status;   /* 0, or the first device-side failure */
  int device_site;     /* which wait failed */
  double kernel_ms;    /* CUDA-event time of the launch */
  double host_ms;      /* host handshake time (skel.cpp:337-340), 0 without it */
} wgm_run_stats;

/* Host CSR (0-based): row_ptr[num_nodes+1], col[row_ptr[num_nodes]]. */
typedef struct wgm_graph_desc {
  int32_t num_nodes;
  int64_t num_edges;        /* entries in col/weights */
  const int32_t *row_ptr;
  const int32_t *col;
  const uint32_t *weights;  /* may be NULL */
} wgm_graph_desc;

/* ---- runtime ----------------------------------------------------------- */
void wgm_config_default(wgm_config *cfg);
const char *wgm_status_string(int status);
/* Replaces mk_init_scheduler_ctx + mk_init_discovery_ctx + the IW_barrier
 * buffer setup (rt_host/cl_scheduler.h:7-33, rt_host/discovery.h:6-16,
 * skel.cpp:278-295). */
int wgm_runtime_create(const wgm_config *cfg, wgm_runtime **out);
/* Replaces free_scheduler_ctx (rt_host/cl_scheduler.h:52-63). */
int wgm_runtime_destroy(wgm_runtime *rt);
/* Replaces restart_scheduler + reset_barrier + reset_discovery
 * (rt_host/cl_scheduler.h:35-50, skel.cpp:127-155). */
int wgm_reset(wgm_runtime *rt);
int wgm_last_cuda_error(const wgm_runtime *rt);
/* The device-side failure of the current launch, else the last one recorded
 * (status WGM_DEV_*, the WGM_SITE_* of the wait that gave up, a detail word);
 * no reference counterpart: the reference spins forever. */
int wgm_device_status(const wgm_runtime *rt, int *status, int *site, int *detail);
/* Raise/clear the host abort word every device wait polls. */
int wgm_set_abort(wgm_runtime *rt, int value);
int wgm_sm_count(const wgm_runtime *rt, int *sms);

/* ---- discovery --------------------------------------------------------- */
/* Replaces get_occupancy_d_ctx (skel.cpp:223-240) and
 * CL_Communicator::get_occupancy_bound (cl_communicator.h:350-374): launches
 * the discovery protocol in occupancy-only mode (mk_init_discovery_ctx_occupancy,
 * rt_host/discovery.h:18-29) and returns the number of co-resident groups. */
int wgm_get_occupancy_bound(wgm_runtime *rt, int threads_per_wg, int *groups);
/* Hardware bound: cudaOccupancyMaxActiveBlocksPerMultiprocessor x SMs for the
 * given app's kernel (no reference counterpart). */
int wgm_hw_occupancy_bound(wgm_runtime *rt, int app_kind, int threads_per_wg, int *groups);

/* ---- barrier microbenchmark (os_freq.cpp:280-330 / os_freq.cl:8-46) ---- */
int wgm_barrier_bench(wgm_runtime *rt, int threads_per_wg, int num_wgs, int iterations,
                      int barrier_kind, double *ns_per_barrier, double *kernel_ms,
                      int *groups);
/* The same over every co-resident cluster of cluster_size CTAs (1-8),
 * launched as a cluster grid, with WGM_BARRIER_CLUSTER (no reference
 * counterpart: OpenCL has no clusters).  num_clusters <= 0: as many as fit. */
int wgm_barrier_bench_cluster(wgm_runtime *rt, int threads_per_wg, int cluster_size,
                              int num_clusters, int iterations, double *ns_per_barrier,
                              double *kernel_ms, int *groups);

/* ---- persistent app plugins -------------------------------------------- */
/* persistent_app_name / persistent_kernel_name (e.g. bfs.h:192-198). */
const char *wgm_persistent_app_name(int app_kind);
const char *wgm_persistent_kernel_name(int app_kind);
/* init_persistent_app_for_occupancy (e.g. bfs.h:209-282, color.h:41-81):
 * allocates device buffers and uploads the graph. */
int wgm_app_create(wgm_runtime *rt, int app_kind, const wgm_graph_desc *g, wgm_app **out);
/* Re-upload a graph with the same node and edge counts (reset_persistent_task
 * re-writes the graph buffers, bfs.h:284-313). */
int wgm_app_upload(wgm_app *app, const wgm_graph_desc *g);
/* Source vertex (the reference hard-wires 0: bfs.cl:236-240, pannotia sssp.h:21). */
int wgm_app_set_source(wgm_app *app, int32_t source);
/* Colour/MIS priorities node_value[V] (color.h:49-55, mis.h:52-56). */
int wgm_app_set_node_values(wgm_app *app, const float *node_value);
int wgm_app_set_pagerank(wgm_app *app, float damping, int iterations);
/* How a standalone Pannotia colour run proceeds (no reference counterpart):
 * 0 (the default) a grid barrier per round (color.cl's structure; the
 * megakernel and the served form always run rounds, where they resize);
 * 1 without rounds - a vertex is coloured as soon as its last larger
 * out-neighbour is, the warp that colours it releasing its smaller
 * neighbours next (slower on RMAT graphs: 16 ms against 8.3 ms at scale
 * 20).  Same colours, same round count (the largest colour). */
int wgm_app_set_color_mode(wgm_app *app, int32_t mode);
/* How a standalone Lonestar BFS run proceeds (no reference counterpart):
 * 0 the reference's shape - discovered groups, a grid barrier per level;
 * 1 one CTA, the visited set and the frontier in shared memory and
 * __syncthreads as the level barrier (graphs of at most 2^20 vertices);
 * -1 (the default) 1 for graphs of at most 65,536 vertices and average
 * degree at most 8 when num_wgs <= 1 and without the host handshake, else
 * 0.  An explicit num_wgs > 1 always runs the grid form.  Same levels, same
 * level count.  The megakernel always runs the grid form. */
int wgm_app_set_bfs_mode(wgm_app *app, int32_t mode);
/* Betweenness centrality from sources 0 .. num_sources-1 (bc.cl:160-235
 * loops over every vertex; a smaller count bounds the run on big graphs). */
int wgm_app_set_bc_sources(wgm_app *app, int32_t num_sources);
/* How a standalone run spreads the work (no reference counterpart): 0 one
 * source at a time over every group, a barrier per level (bc.cl's shape;
 * the megakernel always runs this); 1 the sources over the CTAs, each
 * source's state in shared memory, no grid barrier (graphs of at most
 * 10240 vertices; the default there).  Same arithmetic, same tolerance. */
int wgm_app_set_bc_mode(wgm_app *app, int32_t mode);
/* One iteration of run_persistent (skel.cpp:316-355): launch the persistent
 * kernel on up to num_wgs groups and wait.  num_wgs <= 0: all co-resident,
 * except where fewer groups run the many short rounds faster - Pannotia
 * colour takes 512 threads per SM (two 256-thread CTAs, at least one CTA),
 * Lonestar BFS/SSSP one group per 8192 edges rounded up to a multiple of
 * the SM count, Pannotia SSSP 1024 threads per SM or one thread per 128
 * edges, whichever is more; never more than all.  An explicit num_wgs is
 * always honoured. */
int wgm_run_persistent(wgm_runtime *rt, wgm_app *app, int num_wgs, wgm_run_stats *stats);
/* Asynchronous launch on a caller stream (cudaStream_t; NULL = the runtime's
 * stream).  With cfg.host_handshake set the kernel waits for
 * DEVICE_TO_PERSISTENT_TASK like the reference's standalone kernel, and
 * nothing here sends it: the wait runs out after spin_timeout_ns and the
 * launch ends with WGM_ERR_TIMEOUT (used to test the timeout path). */
int wgm_launch_persistent(wgm_runtime *rt, wgm_app *app, int num_wgs, void *stream);
/* Wait (bounded by run_timeout_ns, then abort) for everything queued on the
 * runtime's stream and report the first device-side failure. */
int wgm_synchronize(wgm_runtime *rt);
/* check_persistent_task's read-back (bfs.h:367-370): dist (uint32) for the
 * Lonestar apps, colours / s_array / cost (int32) for Pannotia, pr (float). */
int wgm_app_read_result(wgm_app *app, void *host_out, size_t bytes);
int wgm_app_result_device_ptr(wgm_app *app, void **device_ptr, size_t *bytes);
int wgm_app_rounds(wgm_app *app, int *rounds);
/* clean_persistent_task (bfs.h:330-334). */
int wgm_app_destroy(wgm_app *app);

/* An app built outside the library (no reference counterpart for the
 * mechanism; the reference selects its app at compile time, skel.cpp:50-77,
 * and binds it through the plugin functions of e.g. bfs.h:192-370):
 * the app compiles its phase function against include/wgm_device.cuh into
 * its own standalone kernel and megakernel (wgm_app_kernel /
 * wgm_app_mega_kernel) and hands the runtime this table.  Each entry gets
 * `user` first; entries marked optional may be NULL.  The runtime then
 * runs it like a built-in app: wgm_run_persistent / wgm_launch_persistent
 * (standalone, on discovered groups), the communicator (wgm_comm_*,
 * resizable inside the megakernel next to non-persistent tasks),
 * wgm_app_read_result, wgm_app_rounds, wgm_app_check, wgm_app_destroy. */
#define WGM_APP_PLUGIN 100
#define WGM_APP_VTABLE_VERSION 1
typedef struct wgm_app_vtable {
  int version;             /* WGM_APP_VTABLE_VERSION */
  void *user;              /* the app's own state */
  const char *app_name;    /* persistent_app_name (bfs.h:192-194) */
  const char *kernel_name; /* persistent_kernel_name (bfs.h:196-198) */
  /* init_persistent_app_for_occupancy / _for_real (bfs.h:209-282): device
   * buffers and inputs, on `device`; called once by wgm_app_register.
   * Optional. */
  int (*init)(void *user, int device);
  /* reset_persistent_task (bfs.h:284-313): inputs back to their initial
   * state, queued on `stream` (cudaStream_t) before every standalone run.
   * Optional. */
  int (*reset)(void *user, void *stream);
  /* check_persistent_task (bfs.h:336-370): *ok = 1 if the last run's output
   * is right.  Optional. */
  int (*check)(void *user, int *ok);
  /* output_persistent_solution (color.h:180-195): the output, copied to
   * host memory.  Optional. */
  int (*read_result)(void *user, void *host_out, size_t bytes);
  /* Rounds (levels, iterations) of the last run.  Optional. */
  int (*rounds)(void *user, int *rounds);
  /* clean_persistent_task (bfs.h:330-334).  Optional. */
  void (*clean)(void *user);
  /* CTAs per SM of the standalone kernel (mega = 0) or of the megakernel
   * (mega = 1) at threads_per_wg threads: wgm_app_kernels<App>::occupancy. */
  int (*occupancy)(void *user, int mega, int threads_per_wg, int *ctas_per_sm);
  /* Queue the standalone kernel on `stream` with the runtime's launch record
   * `launch` (a wgm_launch of wgm_device.cuh): wgm_app_kernels<App>::launch. */
  int (*launch)(void *user, const void *launch, int grid, int threads_per_wg, void *stream);
  /* Queue the megakernel with `launch` and the control block `mega` (a
   * wgm_mega_ctl): wgm_app_kernels<App>::launch_mega.  Optional: without it
   * the app cannot be the communicator's persistent app. */
  int (*launch_mega)(void *user, const void *launch, const void *mega, int grid,
                     int threads_per_wg, void *stream);
} wgm_app_vtable;
/* Register an app table (copied) and call its init; the app runs on this
 * runtime's device.  If init fails, the table's clean is called and its
 * status returned; once registered, wgm_app_destroy calls clean. */
int wgm_app_register(wgm_runtime *rt, const wgm_app_vtable *vt, wgm_app **out);
/* check_persistent_task of a registered app (the table's check), or of the
 * octree (wgm_octree_check); WGM_ERR_INVALID for other built-in apps, whose
 * outputs the caller compares itself. */
int wgm_app_check(wgm_app *app, int *ok);

/* Octree app (test_suite/final_octree/octree.h:98-132 init_persistent_app_for_real,
 * octree.cl:150-320): num_particles float4 positions (xyzw, host), boxes of
 * more than maxchilds particles split (FLAGS_maxChildren), task pools of
 * pool_size tasks (FLAGS_pool_size), tree_cap tree entries (MAXTREESIZE).
 * Runs with wgm_run_persistent or as the megakernel's persistent app; every
 * run starts from the same particles.  wgm_app_read_result returns the
 * particles in leaf order (16 bytes each). */
int wgm_octree_create(wgm_runtime *rt, int32_t num_particles, const float *xyzw,
                      int32_t maxchilds, int32_t pool_size, int64_t tree_cap, wgm_app **out);
/* The tree of the last run: entries [0, *tree_size) into tree_out (an entry
 * is a child block's first index, or 0x80000000 | leaf particle count),
 * particlesDone and the number of tasks run. */
int wgm_octree_read(wgm_app *app, uint32_t *tree_out, int64_t tree_len, uint32_t *tree_size,
                    uint32_t *done, int32_t *tasks);
/* check_persistent_task (octree.h:190-236): leaf counts and particlesDone
 * both equal the particle count. */
int wgm_octree_check(wgm_app *app, int32_t *ok);

/* Connect-four app (test_suite/connect_four/connect_four.h:148-230): the 42
 * cells of the base board row by row from the top (0 empty, 1 human "o", 2
 * computer "x"), maxlevel moves of look-ahead (1..7, FLAGS_maxlevel), task
 * pools of pool_size node ids (FLAGS_pool_size).  wgm_app_read_result returns
 * next_move_value[7] (int32), the value of each first move. */
int wgm_c4_create(wgm_runtime *rt, const uint8_t *board, int32_t maxlevel, int32_t pool_size,
                  wgm_app **out);

/* ---- megakernel and communicator --------------------------------------- */
/* One persistent launch in which discovered group 0 runs the device-side
 * scheduler (cl_scheduler.cl:54-308) and the other groups take either slices
 * of the resident persistent app (grown and shrunk at every barrier by
 * offer_fork/offer_kill, iw_barrier.cl:165-305, scheduler_1.cl:10-81) or the
 * non-persistent task.  The host drives it with the reference's
 * CL_Communicator protocol (cl_communicator.h:19-465). */
#define WGM_NP_NONE 0
#define WGM_NP_MATMULT_I32 1 /* matmult.cl: int32, djb2 hash of the diagonal */
#define WGM_NP_REDUCE_I32 2  /* reduce.cl: int32 min */
#define WGM_NP_MATMULT_F32 3 /* FP32 n x n product (no reference counterpart) */
#define WGM_NP_REDUCE_F32 4  /* FP32 min (no reference counterpart) */
typedef struct wgm_comm wgm_comm;
/* Communicator for a persistent app (may be NULL) plus one non-persistent
 * task kind of size np_size (matmult: n, reduce: elements):
 * CL_Communicator's constructor + init_non_persistent_app (matmult.h:163-231,
 * reduce.h:330-348). */
int wgm_comm_create(wgm_runtime *rt, wgm_app *persistent, int np_kind, int np_size,
                    wgm_comm **out);
int wgm_comm_destroy(wgm_comm *comm);
/* launch_mega_kernel (cl_communicator.h:71-95); num_wgs <= 0: all co-resident. */
int wgm_comm_launch_mega_kernel(wgm_comm *comm, int num_wgs);
/* number_of_discovered_groups (cl_communicator.h:97-99): groups available to
 * tasks (the scheduler's group excluded). */
int wgm_comm_number_of_discovered_groups(wgm_comm *comm, int *groups);
/* send_persistent_task (cl_communicator.h:207-224): starts the monitor thread. */
int wgm_comm_send_persistent_task(wgm_comm *comm, int groups);
/* send_task_synchronous (cl_communicator.h:123-166). */
int wgm_comm_send_task_synchronous(wgm_comm *comm, int groups, uint64_t *exec_ns,
                                   uint64_t *resp_ns);
int wgm_comm_is_executing_persistent(wgm_comm *comm, int *executing);
int wgm_comm_get_persistent_time(wgm_comm *comm, uint64_t *ns);
int wgm_comm_send_quit(wgm_comm *comm);
/* Wait for the megakernel to exit (the reference's exec_queue.finish()). */
int wgm_comm_finish(wgm_comm *comm);
int wgm_comm_reset(wgm_comm *comm);              /* cl_communicator.h:376-393 */
int wgm_comm_add_redline(wgm_comm *comm);        /* cl_communicator.h:67-69 */
int wgm_comm_summary(wgm_comm *comm, char *buf, size_t len); /* :296-336 */
int wgm_comm_task_times(wgm_comm *comm, uint64_t *resp_ns, uint64_t *exec_ns, int capacity,
                        int *count);
int wgm_comm_average_persistent_groups(wgm_comm *comm, double *avg);
int wgm_comm_reset_non_persistent(wgm_comm *comm);              /* reset_non_persistent */
int wgm_comm_check_non_persistent(wgm_comm *comm, int *ok);     /* check_non_persistent_task */
int wgm_comm_get_occupancy_bound(wgm_comm *comm, int *groups);  /* :350-374 */
/* execute_merged_iteration (skel.cpp:405-463). */
int wgm_run_merged_iteration(wgm_comm *comm, int num_wgs, int np_groups, int frequency_ms,
                             int skip_tasks, int *np_errors, int *np_tasks);

/* ---- batched form ------------------------------------------------------- */
/* Many graphs and many (graph, algorithm, source) jobs in one persistent
 * launch: CTAs pull team slots largest job first from a device queue; a job
 * runs its Lonestar BFS (algo 0) or SSSP (algo 1) on a team of CTAs sized by
 * its edges (one CTA and a CTA barrier per level for most jobs, a team
 * counting barrier for the large ones).  No counterpart in the reference,
 * which runs one graph per launch. */
typedef struct wgm_batch wgm_batch;
int wgm_batch_create(wgm_runtime *rt, int num_graphs, const wgm_graph_desc *graphs,
                     int num_jobs, const int32_t *job_graph, const int32_t *job_algo,
                     const int32_t *job_source, wgm_batch **out);
/* Re-upload graphs of the same shapes. */
int wgm_batch_upload(wgm_batch *b, const wgm_graph_desc *graphs);
/* Re-upload every graph from host arrays packed like the device arena (graph
 * g's rows at row_off[g], its cols and weights at col_off[g], as returned by
 * wgm_batch_graph_offsets): three copies in all. */
int wgm_batch_upload_packed(wgm_batch *b, const int32_t *rows, const int32_t *cols,
                            const uint32_t *weights);
int wgm_batch_graph_offsets(wgm_batch *b, int64_t *row_off, int64_t *col_off);
/* threads per CTA, CTAs per SM (0: occupancy maximum), piece (0: per graph). */
int wgm_batch_configure(wgm_batch *b, int threads_per_cta, int ctas_per_sm, int piece);
/* Team sizing: a job of E edges runs on ceil(E / team_edges) CTAs, at most
 * max_team.  0 selects the defaults: total edges / grid, a quarter of the grid. */
int wgm_batch_configure_teams(wgm_batch *b, int64_t team_edges, int max_team);
int wgm_batch_team_info(wgm_batch *b, int64_t *team_edges, int *max_team);
/* Warp-local continuation: after its share of a level a warp relaxes the
 * vertices it just improved for up to `rounds` more rounds (0..12; 0 = plain
 * levels).  Both give the same distances; the autotuner picks. */
int wgm_batch_configure_local(wgm_batch *b, int rounds);
/* SSSP schedule (no reference counterpart; the reference's sssp.cl runs the
 * Bellman-Ford worklist): near-far buckets of delta_mult x the graph's mean
 * edge weight (default 20; 0 = the worklist), far lists of far_cap entries
 * (0 = 2V + 64; a full list relaxes the vertex at once).  Distances are the
 * same for every setting; only the work and the level count change. */
int wgm_batch_configure_sssp(wgm_batch *b, double delta_mult, int far_cap);
int wgm_batch_sssp_info(wgm_batch *b, double *delta_mult, int *far_cap);
/* SSSP jobs on dense graphs (average degree at least 6) can instead use
 * buckets of light_mult x the mean weight and relax heavy edges - weight at
 * least the bucket width - once per bucket (delta-stepping's light/heavy
 * split).  0 (the default) gives them the schedule of
 * wgm_batch_configure_sssp; the autotuner tries 0.1-0.4.  Distances do not
 * change. */
int wgm_batch_configure_sssp_dense(wgm_batch *b, double light_mult);
int wgm_batch_sssp_dense_info(wgm_batch *b, double *light_mult);
/* BFS jobs on graphs of average degree at most max_avg_degree (default 5:
 * grids, meshes, road-like graphs; 0: none) run on one CTA whatever their
 * edge count: their levels are chains of dependent round trips over small
 * frontiers, which a team speeds up little at several times the CTA time.
 * Distances do not change. */
int wgm_batch_configure_bfs_one_cta(wgm_batch *b, double max_avg_degree);
/* Register budget of the batched kernel (no reference counterpart): 64, 80
 * or 96 registers per thread (blocks of at most 1024, 768, 640 threads);
 * fewer registers fit more warps on an SM, more avoid spilling. */
int wgm_batch_configure_kernel(wgm_batch *b, int max_regs);
int wgm_batch_kernel_info(wgm_batch *b, int *max_regs);
/* Queue one batched launch on the runtime's stream (use_cuda_graph: replay a
 * captured CUDA graph of the queue reset and the launch). */
int wgm_batch_launch(wgm_batch *b, int use_cuda_graph);
int wgm_batch_run(wgm_batch *b, int use_cuda_graph, double *device_ms);
/* The plain form for comparison: one standalone persistent launch per job,
 * each on every co-resident CTA (the reference's standalone run,
 * src/host_skeleton/skel.cpp:316-355, uses the discovered group count). */
int wgm_batch_launch_per_graph(wgm_batch *b);
int wgm_batch_run_per_graph(wgm_batch *b, double *device_ms);
/* The same with a group-count policy: WGM_PER_GRAPH_ALL (every co-resident
 * CTA, as above) or WGM_PER_GRAPH_DEFAULT (the count wgm_run_persistent
 * picks with num_wgs <= 0 for a Lonestar app: one group per 8192 edges,
 * rounded up to a multiple of the SM count). */
#define WGM_PER_GRAPH_ALL 0
#define WGM_PER_GRAPH_DEFAULT 1
int wgm_batch_launch_per_graph_sized(wgm_batch *b, int policy);
int wgm_batch_run_per_graph_sized(wgm_batch *b, int policy, double *device_ms);
/* Pipelined batches (no reference counterpart): upload_packed + launch +
 * read_all of one step, queued without waiting.  Steps alternate between two
 * device copies of the graphs and distances, so the upload of step k+1 and
 * the read-back of step k-1 overlap the kernel of step k; every step copies
 * all of its graphs in and all of its distances into `out` (dist_total
 * values in the caller's job order).  Host buffers should be pinned, and
 * stay untouched until wgm_batch_wait returns.  The second device copy is
 * allocated by the first submit. */
int wgm_batch_submit_packed(wgm_batch *b, const int32_t *rows, const int32_t *cols,
                            const uint32_t *weights, uint32_t *out);
int wgm_batch_wait(wgm_batch *b);
int wgm_batch_read(wgm_batch *b, int job, uint32_t *out, int64_t n);
int wgm_batch_read_all(wgm_batch *b, uint32_t *out, int64_t n);
/* Per job (caller's order) of the last batched launch: device start and end
 * (ns from the earliest start), team size, levels run. */
int wgm_batch_job_stats(wgm_batch *b, int64_t *start_ns, int64_t *end_ns, int32_t *team,
                        int32_t *levels);
/* Per job (caller's order) of the last batched launch: edges walked, every
 * visit of a vertex counting its edges (the component's edge count for a job
 * that relaxes each vertex once; more where distances are lowered again). */
int wgm_batch_job_work(wgm_batch *b, int64_t *edges_walked);
int wgm_batch_info(wgm_batch *b, int64_t *total_nodes, int64_t *total_edges, int *threads,
                   int *ctas_per_sm, int *piece);
/* Queue the jobs longest first by their device time in the last batched
 * launch (profile-guided order; results and offsets are unchanged). */
int wgm_batch_reorder_by_last_run(wgm_batch *b);
/* Sweep block size {128,256,512} x CTAs per SM x piece {16,32,64}, then the
 * team size at the winner. */
int wgm_batch_autotune(wgm_batch *b, int reps, int *best_threads, int *best_ctas_per_sm,
                       int *best_piece, double *best_ms);
int wgm_batch_destroy(wgm_batch *b);

/* ---- served form -------------------------------------------------------- */
/* One serving megakernel launch hosts a resident persistent job (Pannotia
 * colour then Lonestar BFS on one graph, `reps` times, resizable at every
 * barrier) while a Poisson stream of requests arrives: BFS queries on
 * resident graphs, FP32 min reductions over resident vectors, FP32 n x n
 * products of resident operand pairs.  A request is admitted when its state
 * fits in the device arena (first fit), runs on a team of groups beside
 * other requests, and the persistent job cedes groups to waiting requests at
 * its resizing barriers (offer_kill) and takes free ones back (offer_fork).
 * Generalises the reference's one-task-at-a-time CL_Communicator loop
 * (cl_communicator.h:19-465, skel.cpp:387-463). */
#define WGM_REQ_BFS 1
#define WGM_REQ_REDUCE 2
#define WGM_REQ_MATMUL 3
#define WGM_REQ_REDUCE_I32 4 /* reduce.cl int32 min */
#define WGM_REQ_MATMUL_I32 5 /* matmult.cl int32 product and its diagonal djb2 hash */
typedef struct wgm_serve wgm_serve;
typedef struct wgm_serve_config {
  double rate_per_s;   /* Poisson arrival rate (0: no requests) */
  double duration_s;   /* stream length; with reps > 0 the stream also stops when
                          the persistent job ends */
  uint64_t seed;
  double frac_bfs;     /* request mix; the rest after frac_reduce are matmuls */
  double frac_reduce;
  int reps;            /* persistent job repetitions (0: no persistent job) */
  int persist_groups;  /* groups the persistent job starts with (0: all but the
                          reserve) */
  int reserve;         /* free groups the persistent job leaves to requests */
  int bfs_groups, reduce_groups, matmul_groups; /* team sizes */
  int max_in_flight;   /* admitted and unfinished requests (<= 4000) */
  int keep_results;    /* copy every request's output to the host (tests) */
  int threads_per_wg;  /* 0: the runtime's */
  int64_t bfs_edges_per_group; /* > 0: a BFS query gets ceil(E / this) groups, at
                                  most bfs_groups */
  double frac_int;     /* share of reduce/matmul requests run as the int32
                          reference variants (needs wgm_serve_set_int_data) */
  int persist_max_groups; /* most groups the persistent job forks up to (0: no
                             limit); the rest stay free for requests */
} wgm_serve_config;
typedef struct wgm_serve_stats {
  int64_t arrived, completed, waited_for_memory;
  double stream_s;       /* from the first arrival to the last completion */
  double achieved_rate;  /* completed / stream_s */
  double lat_p50_us, lat_p99_us, lat_mean_us, lat_max_us;
  double persist_ms;     /* launch to the persistent job's last repetition */
  int persist_reps;
  int kills, forks;      /* groups ceded and taken back by the persistent job */
  int groups;            /* discovered groups (scheduler included) */
  double run_ms;         /* whole launch, host clock */
  /* the reference communicator's split (cl_communicator.h:296-336): execution
   * = device time from team assignment to the last group's end; wait = the
   * rest of the latency (admission, ring, waiting for groups, completion seen) */
  double exec_p50_us, exec_p99_us, wait_p50_us, wait_p99_us;
  /* the persistent job's group count over the run, sampled every 1 ms
   * (cl_communicator.h:186-200): mean and least */
  double persist_groups_mean;
  int persist_groups_min;
} wgm_serve_stats;
/* color/bfs: the persistent job's apps (both NULL: requests only), created
 * with wgm_app_create on the same graph.  graphs: BFS query graphs; vecs:
 * num_vecs x vec_len floats (>= 0); mats: num_mats pairs (A, B) of mat_n x
 * mat_n floats, mat_n a multiple of 32; arena_bytes: request-state memory. */
int wgm_serve_create(wgm_runtime *rt, wgm_app *color, wgm_app *bfs, int num_graphs,
                     const wgm_graph_desc *graphs, int num_vecs, int vec_len, const float *vecs,
                     int num_mats, int mat_n, const float *mats, int64_t arena_bytes,
                     wgm_serve **out);
/* Resident data of the int32 reference variants: num_ivecs x ivec_len int32
 * reduce inputs, num_imats pairs (A, B) of imat_n x imat_n int32. */
int wgm_serve_set_int_data(wgm_serve *s, int num_ivecs, int ivec_len, const int32_t *ivecs,
                           int num_imats, int imat_n, const int32_t *imats);
int wgm_serve_run(wgm_serve *s, const wgm_serve_config *cfg, wgm_serve_stats *stats);
/* Requests of the last run, in arrival order: kind, arg0 (graph / vector /
 * pair), arg1 (BFS source), latency (ns, arrival to completion seen by the
 * host; -1 if not completed), team size. */
int wgm_serve_requests(wgm_serve *s, int64_t *count, int32_t *kind, int32_t *arg0,
                       int32_t *arg1, int64_t *latency_ns, int32_t *groups);
/* Output of request i of the last run (keep_results): BFS dist (uint32 x V),
 * reduce min (one float / int32), matmul C (mat_n^2 floats), int32 matmul
 * hash followed by C (1 + imat_n^2 int32). */
int wgm_serve_result(wgm_serve *s, int64_t i, void *out, int64_t bytes);
/* Device execution time (ns) of each request of the last run, -1 if none. */
int wgm_serve_exec_times(wgm_serve *s, int64_t n, int64_t *exec_ns);
/* The persistent job's group count sampled every millisecond of the last
 * run (CL_Communicator::print_groups_time_data, cl_communicator.h:186-241):
 * t_ns from the launch, groups at that time; NULL arrays give *count only. */
int wgm_serve_groups_trace(wgm_serve *s, int64_t *t_ns, int32_t *groups, int64_t capacity,
                           int64_t *count);
/* Where the last failed run stood (host and device counters), "" if none. */
int wgm_serve_diag(wgm_serve *s, char *buf, size_t len);
int wgm_serve_destroy(wgm_serve *s);

/* ---- device timing on the runtime's stream (CUDA events) --------------- */
/* os_freq.cpp:311-328 reads CL profiling events; here a pair of CUDA events
 * brackets everything queued on the runtime's stream in between. */
int wgm_timer_start(wgm_runtime *rt);
int wgm_timer_stop(wgm_runtime *rt, double *elapsed_ms);

/* ---- allocation-free BFS ------------------------------------------------ */
/* No counterpart in the reference.  For callers that cannot allocate GPU
 * memory (their own pool allocator owns the device, or cudaMalloc/cudaFree's
 * implicit synchronisation is not acceptable where they call from): runs the
 * persistent Lonestar BFS from `source` over a device CSR the caller owns and
 * writes the levels to the caller's d_dist[num_nodes], allocating nothing.
 * Its scratch is one static device array sized for WGM_NOALLOC_MAX_NODES
 * vertices (about 8.5 MB, held by every GPU that loads the library until the
 * process exits); larger graphs return WGM_ERR_INVALID.  The first call on a
 * device does a one-time set-up (the array's device address), so make it
 * before any stream capture.  Calls share the array: calls whose kernels
 * overlap on the GPU race, so keep them ordered on one device.  `stream` is a
 * cudaStream_t (NULL: the default stream); the call returns when the BFS has
 * finished, so it cannot run on a stream under capture: there it returns
 * WGM_ERR_STATE without touching the capture.  d_row_ptr must be a valid CSR
 * (row_ptr[V] may be one short of num_edges, as the Lonestar loader
 * produces). */
#define WGM_NOALLOC_MAX_NODES (1 << 18)
int wgm_bfs_noalloc(const int32_t *d_row_ptr, const int32_t *d_col, int32_t num_nodes,
                    int64_t num_edges, int32_t source, uint32_t *d_dist, void *stream);

/* ---- profiler range (no reference counterpart) -------------------------- */
/* cudaProfilerStart / cudaProfilerStop on the runtime's device: a profiler
 * started with its capture off (ncu --profile-from-start off) sees only the
 * launches in between. */
int wgm_profiler_start(wgm_runtime *rt);
int wgm_profiler_stop(wgm_runtime *rt);

/* ---- host memory helpers (pinned, for H2D/D2H at full bandwidth) ------- */
void *wgm_host_alloc(size_t bytes);
void wgm_host_free(void *p);

/* ---- synthetic inputs (the reference reads them from files) ------------ */
/* 4-connected rows x cols grid, node id r*cols+c, neighbours in
 * (up, left, right, down) order.  row_ptr[rows*cols+1], col[...]. */
int wgm_gen_grid(int32_t rows, int32_t cols, int32_t *row_ptr, int32_t *col, int64_t *num_edges);
/* RMAT (scale, edge factor, a, b, c), symmetrised, self loops and
 * duplicates removed, rows sorted; optional seeded relabelling; uint32
 * weights uniform in [wmin, wmax] per undirected edge when wmax > 0. */
int wgm_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed,
                 int permute, uint32_t wmin, uint32_t wmax, wgm_host_graph **out);
int wgm_host_graph_info(const wgm_host_graph *g, int32_t *num_nodes, int64_t *num_edges);
int wgm_host_graph_arrays(const wgm_host_graph *g, const int32_t **row_ptr,
                          const int32_t **col, const uint32_t **weights);
void wgm_host_graph_free(wgm_host_graph *g);

#ifdef __cplusplus
}
#endif
#endif
