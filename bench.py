"""Benchmark of the cooperative-kernel runtime on one GB300 (or N replicas).

Headline (default): the batched form.  512 seeded graphs, node counts
lognormal between 2^8 and 2^18 (half RMAT (0.57,0.19,0.19) with average degree
8-32, half near-square 2D grids), one BFS and one SSSP job per graph from
seeded sources (uint32 weights U[1,1000]) - 1024 jobs in one persistent launch
with a device work queue, replayed from a CUDA graph, shape and team size
chosen by the autotuner.  A step = one batched launch over all 1024 jobs with
the graphs resident in HBM (1.4 GB of CSR, larger than L2).

JSON line keys (one line, rank 0):
  value        batched GTEPS = sum over jobs of traversed edges (out-degree
               summed over reached vertices) / device time per step (CUDA
               events on the launching stream)
  e2e          the same metric through the public API with host buffers:
               per step pinned H2D of every graph, the launch, D2H of every
               job's distances, queued with wgm_batch_submit_packed (step
               k+1's upload and step k-1's read-back under step k's kernel;
               serial_value: the same steps one after another)
  roofline     algorithmic GB/s of the batched kernel vs the HBM peak
  cpu_baseline the oracle (the reference's algorithm restated in C) over
               the same 1024 jobs, jobs spread over the host cores
  extra        plain per-graph launches of the same jobs and the speed-up,
               ns per global barrier (10^6 barriers over every co-resident
               CTA), persistent SSSP on RMAT-20, served-form latency
`--impl reference` times the reference's algorithm on the host cores (the
oracle port: the reference's OpenCL 2.0 program needs fine-grained SVM atomics,
which no runtime on the box provides) on the same jobs.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

INF = 1000000000
HBM_FALLBACK_GBS = 6800.0
METRIC = "batched GTEPS vs per-graph launches, bit-exact; barrier ns; p99 task latency"
WORKLOAD = ("batched Lonestar BFS+SSSP: 512 graphs (log2 V ~ N(13, 2.5) in [8, 18], "
            "half RMAT (0.57,0.19,0.19) avg degree 8-32, half 2D grids), 1024 jobs, "
            "seed 2024, weights U[1,1000]")


def _peak_hbm() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        for k in ("hbm_gbs", "hbm_GBs", "hbm"):
            if k in d:
                v = d[k]
                if isinstance(v, dict):
                    v = v.get("value", v.get("gbs"))
                return float(v), "measured"
    except Exception:
        pass
    return HBM_FALLBACK_GBS, "fallback"


def _traffic(kernel: str, workload: str):
    """Per-launch DRAM bytes from a committed ncu summary, when one exists."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.json")
    try:
        with open(p) as f:
            return float(json.load(f)["dram_bytes_per_launch"])
    except Exception:
        return None


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.out = ""

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            # the sampler is live (its first line printed, and dropped: it
            # precedes the timed region) before the timed region starts
            self.proc.stdout.readline()
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                self.out = ""

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _max_over_ranks(dist, x: float) -> float:
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _job_edges(gs, jobs, res, offsets):
    """Per job: traversed edges E_t and reached vertices V_r."""
    et, vr = [], []
    for k, (gi, _algo, _src) in enumerate(jobs):
        d = res[offsets[k]:offsets[k + 1]]
        reached = d != INF
        et.append(int(gs[gi].degrees()[reached].sum()))
        vr.append(int(reached.sum()))
    return np.array(et, np.int64), np.array(vr, np.int64)


def _alg_bytes(gs, jobs, et, vr) -> int:
    """Algorithmic bytes of one batched launch, per job: per traversed edge
    col (4) and dist[dst] (4), plus the weight (4) for SSSP; per reached
    vertex its row pair (8), its worklist piece written and read once (start
    and count, plus the vertex for SSSP: 16 or 24) and its distance (4); per
    vertex the initialisation of dist (4), and of the SSSP stamp (4)."""
    total = 0
    for k, (gi, algo, _src) in enumerate(jobs):
        V = gs[gi].num_nodes
        if algo == "sssp":
            total += 12 * int(et[k]) + 36 * int(vr[k]) + 8 * V
        else:
            total += 8 * int(et[k]) + 28 * int(vr[k]) + 4 * V
    return total


def _batch_inputs():
    from gpu_workgroup_managment_gb300.batch import batch_workload
    return batch_workload()


def _cpu_best(fn, budget_s: float = 10.0, max_runs: int = 3) -> float:
    """Best wall time (s) of up to max_runs calls of fn, stopping once the
    calls have taken budget_s."""
    best, total, runs = float("inf"), 0.0, 0
    while runs < max_runs and (runs == 0 or total < budget_s):
        t0 = time.perf_counter()
        fn()
        dt = time.perf_counter() - t0
        best, total, runs = min(best, dt), total + dt, runs + 1
    return best


def _reference_arm(args, ws, rank) -> int:
    """The reference's algorithm on the host cores: the oracle's job-parallel
    batched restatement of lonestar bfs.cl / sssp.cl over the same 1024 jobs,
    every host thread busy.  One step = the whole batch.  The graphs come from
    oracle/workload.py (the same arrays as the GPU arm's), so this arm loads
    no product library."""
    if rank != 0:
        return 0
    from oracle import oracle
    from oracle.workload import batch_workload
    gs, jobs, meta = batch_workload()
    arena = oracle.BatchArena(gs, jobs)
    d = arena.run()
    offsets = np.concatenate([[0], np.cumsum(arena.V.astype(np.int64))])
    et, _ = _job_edges(gs, jobs, d, offsets)
    E = int(et.sum())
    warm = max(args.warmup, 3)
    for _ in range(warm - 1):
        arena.run()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        arena.run()
        times.append(time.perf_counter() - t0)
    mean = sum(times) / len(times)
    v = E / mean / 1e9
    sample = (f"{args.steps} runs of all {len(jobs)} jobs ({E} traversed edges each), jobs "
              f"spread over {oracle.threads()} threads, each job the serial restatement "
              "of the reference's bfs.cl/sssp.cl; the reference's OpenCL 2.0 SVM program "
              "cannot run here")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "GTEPS",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": warm, "ms_per_step": mean * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic", "config": {"workload": WORKLOAD, "jobs": len(jobs),
                                            "edges_traversed": E},
            "cpu_baseline": {"value": v, "unit": "GTEPS", "cores": oracle.threads(),
                             "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "GTEPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _barrier_sweep() -> int:
    from gpu_workgroup_managment_gb300 import Runtime
    kinds = {0: "sense", 1: "xf", 2: "tree", 3: "count", 4: "spread", 5: "auto"}
    with Runtime() as rt:
        for threads in (128, 256, 512, 1024):
            for kind, name in kinds.items():
                r = rt.barrier_bench(iterations=20000, threads_per_wg=threads, barrier_kind=kind)
                print(json.dumps({"barrier": name, "threads_per_cta": threads,
                                  "ctas": r["groups"], "barriers": r["barriers"],
                                  "ns_per_barrier": r["ns_per_barrier"]}))
    return 0


def _sssp_rmat(rt, scale: int, steps: int, warmup: int) -> dict:
    """Persistent Lonestar SSSP on RMAT scale `scale` (edge factor 16, seed 1,
    weights U[1,1000]) from the max-degree vertex: one launch per step."""
    from gpu_workgroup_managment_gb300 import PersistentApp, graphs
    g = graphs.rmat(scale, 16, seed=1)
    src = graphs.max_degree_vertex(g)
    with PersistentApp(rt, "lonestar_sssp", g, source=src) as app:
        st0 = app.run()
        d = app.result()
        reached = d != INF
        et, vr = int(g.degrees()[reached].sum()), int(reached.sum())
        for _ in range(warmup):
            app.launch()
        rt.synchronize()
        rt.timer_start()
        for _ in range(steps):
            app.launch()
        ms = rt.timer_stop() / steps
    return {"gteps": et / (ms * 1e-3) / 1e9, "ms": ms, "levels": st0.rounds,
            "groups": st0.groups, "edges_traversed": et, "vertices_reached": vr,
            "bytes_alg": 12 * et + 36 * vr + 8 * g.num_nodes}


def _octree(rt, n: int = 3_000_000) -> dict:
    """The work-stealing octree build at the reference's defaults
    (octree.h: 3,000,000 particles, maxChildren 5, pool size 50,000):
    standalone persistent launches, CUDA events, best of 3 after a warm-up,
    the reference's check on the last one."""
    from gpu_workgroup_managment_gb300.octree import Octree, clustered_particles
    pts = clustered_particles(n, seed=1)
    with Octree(rt, pts) as oc:
        oc.run()
        runs = [oc.run() for _ in range(3)]
        _, done, tasks = oc.tree()
        return {"particles": oc.n, "ms": min(r.kernel_ms for r in runs), "tasks": tasks,
                "groups": runs[0].groups, "check": oc.check()}


def _best(app, k: int = 5):
    app.run()
    return min((app.run() for _ in range(k)), key=lambda s: s.kernel_ms)


def _c1(rt, barrier_ns) -> dict:
    """C1: plain persistent BFS on the 256x256 4-neighbour grid from vertex 0
    (Lonestar view), one launch per run, CUDA events, best of 5; the grid
    form (discovered groups, a grid barrier per level) and, beside it, the
    one-CTA form.  Bytes_alg
    = 8 E_t + 20 V_r; ns per level and the barrier's share of it.  CPU
    baseline: the oracle's level-synchronous restatement of bfs.cl on every
    host core and on one."""
    from gpu_workgroup_managment_gb300 import PersistentApp, graphs
    from oracle import oracle
    g = graphs.lonestar_view(graphs.grid(256, 256))
    # the configuration as defined: discovered groups, a grid barrier per level
    with PersistentApp(rt, "lonestar_bfs", g, bfs_mode=0) as a:
        st = _best(a)
        d = a.result()
    # the same BFS on one CTA (the default for a graph this small and sparse)
    with PersistentApp(rt, "lonestar_bfs", g, bfs_mode=1) as a:
        st1 = _best(a)
        d1 = a.result()
    if not np.array_equal(d1, d) or st1.rounds != st.rounds:
        raise SystemExit("C1 BFS on one CTA differs from the grid form")
    reached = d != INF
    et, vr = int(np.diff(g.row_ptr)[reached].clip(min=0).sum()), int(reached.sum())
    peak, kind = _peak_hbm()
    s = st.kernel_ms * 1e-3
    if not np.array_equal(d, oracle.lonestar_bfs(g, 0)):
        raise SystemExit("C1 BFS differs from the oracle")
    t_omp = _cpu_best(lambda: oracle.lonestar_bfs(g, 0, omp=True))
    t_one = _cpu_best(lambda: oracle.lonestar_bfs(g, 0))
    out = {"ms": st.kernel_ms, "levels": st.rounds, "groups": st.groups,
           "gteps": et / s / 1e9, "gteps_undirected": et / 2 / s / 1e9,
           "ns_per_level": st.kernel_ms * 1e6 / max(st.rounds, 1),
           "gbs_alg": (8 * et + 20 * vr) / s / 1e9,
           "frac_of_" + kind: (8 * et + 20 * vr) / s / 1e9 / peak,
           "cpu_baseline": {"ms": t_omp * 1e3, "gteps": et / t_omp / 1e9,
                            "cores": oracle.threads(), "ms_1core": t_one * 1e3,
                            "kind": "port", "sample": "the whole BFS, best of 3"},
           "one_cta": {"ms": st1.kernel_ms, "ns_per_level": st1.kernel_ms * 1e6 / max(st1.rounds, 1),
                       "gteps": et / (st1.kernel_ms * 1e-3) / 1e9}}
    if barrier_ns:
        out["barrier_share"] = barrier_ns * st.rounds / (st.kernel_ms * 1e6)
    return out


def _c2(rt, _barrier_ns) -> dict:
    """C2: RMAT-20 (edge factor 16, seed 1) persistent Lonestar SSSP from
    the max-degree vertex, Pannotia colour and MIS with seeded priorities;
    best of 5 launches each, results checked against the oracle.
    Algorithmic bytes: SSSP 12 E_t + 36 V_r + 8 V (the packed-word kernel);
    colour 16 E + 24 V (each edge read twice as a (neighbour, value) pair:
    once to count a vertex's larger neighbours, once to release them; per
    vertex two row-pair reads, the colour write and the pending count); MIS
    12 B per edge scanned and 16 B per active vertex, summed over rounds
    (the oracle counts both).  CPU baselines: the oracle's OpenMP
    restatements of sssp.cl, color.cl and mis.cl on every host core, on the
    whole graph (colour: one run - the reference's rounds rescan every
    uncoloured vertex's edges)."""
    from gpu_workgroup_managment_gb300 import PersistentApp, graphs
    from oracle import oracle
    g = graphs.rmat(20, 16, seed=1)
    nv = graphs.seeded_node_values(g.num_nodes, 1)
    src = graphs.max_degree_vertex(g)
    peak, kind = _peak_hbm()
    V, E = g.num_nodes, g.num_edges
    out = {"vertices": V, "edges": E, "cores": oracle.threads()}
    with PersistentApp(rt, "lonestar_sssp", g, source=src) as a:
        st = _best(a)
        d = a.result()
    want = oracle.lonestar_sssp(g, src, omp=True)
    if not np.array_equal(d, want):
        raise SystemExit("C2 SSSP differs from the oracle")
    reached = d != INF
    et, vr = int(g.degrees()[reached].sum()), int(reached.sum())
    s = st.kernel_ms * 1e-3
    gbs = (12 * et + 36 * vr + 8 * V) / s / 1e9
    t = _cpu_best(lambda: oracle.lonestar_sssp(g, src, omp=True))
    out["lonestar_sssp"] = {"ms": st.kernel_ms, "rounds": st.rounds, "groups": st.groups,
                            "gteps": et / s / 1e9, "gbs_alg": gbs, "frac_of_" + kind: gbs / peak,
                            "cpu_ms": t * 1e3, "cpu_gteps": et / t / 1e9}
    with PersistentApp(rt, "color", g, node_values=nv) as a:
        st = _best(a)
        col = a.result()
    t0 = time.perf_counter()
    want = oracle.color(g, nv, omp=True)
    t = time.perf_counter() - t0
    if not np.array_equal(col, want):
        raise SystemExit("C2 colour differs from the oracle")
    s = st.kernel_ms * 1e-3
    gbs = (16 * E + 24 * V) / s / 1e9
    out["color"] = {"ms": st.kernel_ms, "rounds": st.rounds, "groups": st.groups,
                    "gbs_alg": gbs, "frac_of_" + kind: gbs / peak, "cpu_ms": t * 1e3,
                    "cpu_sample": "one run of the OpenMP restatement of color.cl"}
    with PersistentApp(rt, "mis", g, node_values=nv) as a:
        st = _best(a)
        m = a.result()
    want, e_scan, v_act = oracle.mis_work(g, nv)
    if not np.array_equal(m, want):
        raise SystemExit("C2 MIS differs from the oracle")
    s = st.kernel_ms * 1e-3
    gbs = (12 * e_scan + 16 * v_act) / s / 1e9
    t = _cpu_best(lambda: oracle.mis(g, nv, omp=True))
    out["mis"] = {"ms": st.kernel_ms, "rounds": st.rounds, "groups": st.groups,
                  "edges_scanned": e_scan, "gbs_alg": gbs, "frac_of_" + kind: gbs / peak,
                  "cpu_ms": t * 1e3}
    return out


def _c3(rt, _barrier_ns, scale: int = 22) -> dict:
    """C3: PageRank on RMAT-22 (edge factor 16, seed 1), 20 iterations, best
    of 3; Bytes_alg per iteration = 8 E + 16 V.  `scale` < 22 gives the
    smaller profiling case.  CPU baseline: the oracle's OpenMP FP32 pull
    PageRank (same definition) on every host core; error against the FP64
    oracle."""
    from gpu_workgroup_managment_gb300 import PersistentApp, graphs
    from oracle import oracle
    g = graphs.rmat(scale, 16, seed=1)
    with PersistentApp(rt, "pagerank", g, iterations=20) as a:
        st = _best(a, 3)
        pr = a.result()
    s = st.kernel_ms * 1e-3
    peak, kind = _peak_hbm()
    gbs = 20 * (8 * g.num_edges + 16 * g.num_nodes) / s / 1e9
    ref = oracle.pagerank_f64(g)
    err = float(np.max(np.abs(pr.astype(np.float64) - ref)) / np.max(np.abs(ref)))
    if not err <= 1e-5:
        raise SystemExit(f"C3 PageRank error {err} above 1e-5")
    t = _cpu_best(lambda: oracle.pagerank_f32_omp(g), budget_s=8.0)
    return {"ms": st.kernel_ms, "iterations": 20, "groups": st.groups, "gbs_alg": gbs,
            "frac_of_" + kind: gbs / peak, "rel_linf_vs_f64": err,
            "cpu_ms": t * 1e3, "cpu_cores": oracle.threads(),
            "cpu_gbs_alg": 20 * (8 * g.num_edges + 16 * g.num_nodes) / t / 1e9}


def _bc(rt) -> dict:
    """Pannotia betweenness centrality on RMAT-12 (edge factor 16, seed 1),
    every vertex a source: sources over CTAs (shared-memory state) and one
    source at a time over the grid (bc.cl's shape); best of 3, CUDA events.
    Rate = sources x edges / time (each source walks every reached edge
    twice)."""
    from gpu_workgroup_managment_gb300 import PersistentApp, graphs
    g = graphs.rmat(12, 16, seed=1)
    out = {"vertices": g.num_nodes, "edges": g.num_edges, "sources": g.num_nodes}
    for mode, name in ((1, "sources_over_ctas"), (0, "levels_over_grid")):
        with PersistentApp(rt, "bc", g, bc_mode=mode) as a:
            a.run()
            ms = min(a.run().kernel_ms for _ in range(3 if mode else 1))
        out[name + "_ms"] = ms
        out[name + "_gteps"] = g.num_nodes * g.num_edges / (ms * 1e-3) / 1e9
    return out


def _sssp_kernel_only(args) -> int:
    """The command profiled with ncu for the persistent SSSP kernel."""
    from gpu_workgroup_managment_gb300 import Runtime
    with Runtime() as rt:
        r = _sssp_rmat(rt, args.scale, args.steps, max(args.warmup, 3))
    print(json.dumps({"metric": "SSSP GTEPS", "workload": f"rmat{args.scale}_sssp", **r}))
    return 0


def _served(rt, rates=(1000, 5000, 20000), reps: int = 20, reserve: int = 96) -> dict:
    """Served form: a resident colour+BFS job on RMAT scale 22 (edge factor
    16, seed 1; BFS from the max-degree vertex), `reps` repetitions, alone and
    beside a Poisson request stream at each rate: 40% BFS queries on RMAT
    graphs of scale 12-16, 30% FP32 min reductions of 2^20 elements, 30% FP32
    256x256 products; the stream lasts as long as the persistent job."""
    from gpu_workgroup_managment_gb300 import PersistentApp, graphs
    from gpu_workgroup_managment_gb300.serve import Serve, serve_datasets
    g = graphs.rmat(22, 16, seed=1)
    nv = graphs.seeded_node_values(g.num_nodes, 1)
    src = graphs.max_degree_vertex(g)
    qg, vecs, mats = serve_datasets(seed=7)
    out = {"persistent": "colour + Lonestar BFS, RMAT-22", "reps": reps, "reserve": reserve,
           "mix": "40% BFS (RMAT 12-16), 30% FP32 min 2^20, 30% FP32 256x256 matmul",
           "teams": {"bfs": "ceil(E / 65536), at most 32", "reduce": 4, "matmul": 4}}
    with PersistentApp(rt, "color", g, node_values=nv) as ca, \
            PersistentApp(rt, "lonestar_bfs", g, source=src) as ba, \
            Serve(rt, ca, ba, graphs=qg, vecs=vecs, mats=mats, arena_bytes=1 << 30) as sv:
        # the same job as two standalone persistent launches per repetition
        # (each app on its default group count), the reference's
        # "standalone" run of the persistent app (run_test.py:345-360)
        sc, sb = _best(ca, 3).kernel_ms, _best(ba, 3).kernel_ms
        standalone = reps * (sc + sb)
        out["persist_ms_standalone"] = standalone
        out["standalone_rep_ms"] = {"color": sc, "bfs": sb}
        sv.run(reps=1)
        alone = sv.run(reps=reps)
        out["persist_ms_alone"] = alone["persist_ms"]
        out["alone_kept_vs_standalone"] = standalone / alone["persist_ms"]
        runs = []
        for rate in rates:
            st = sv.run(rate=rate, duration_s=60.0, reps=reps, seed=11, reserve=reserve,
                        bfs_groups=32, bfs_edges_per_group=1 << 16, reduce_groups=4,
                        matmul_groups=4, max_in_flight=512)
            runs.append({"rate_offered": rate, "achieved_rate": st["achieved_rate"],
                         "completed": st["completed"], "p50_us": st["lat_p50_us"],
                         "p99_us": st["lat_p99_us"], "mean_us": st["lat_mean_us"],
                         "max_us": st["lat_max_us"], "exec_p50_us": st["exec_p50_us"],
                         "exec_p99_us": st["exec_p99_us"], "wait_p50_us": st["wait_p50_us"],
                         "wait_p99_us": st["wait_p99_us"], "persist_ms": st["persist_ms"],
                         "persist_kept": alone["persist_ms"] / st["persist_ms"],
                         "kept_vs_standalone": standalone / st["persist_ms"],
                         "kills": st["kills"], "forks": st["forks"],
                         "persist_groups_mean": st["persist_groups_mean"],
                         "persist_groups_min": st["persist_groups_min"],
                         "waited_for_memory": st["waited_for_memory"]})
        out["runs"] = runs
        out["checked"] = _served_check(sv, ca, ba, qg, vecs, mats, g, src, nv, reps, reserve,
                                       rates[-1])
        # requests alone (no persistent job) at the lowest rate, for context
        st = sv.run(rate=rates[0], duration_s=0.5, seed=11, bfs_groups=32,
                    bfs_edges_per_group=1 << 16, reduce_groups=4, matmul_groups=4)
        out["requests_only"] = {"rate_offered": rates[0], "p50_us": st["lat_p50_us"],
                                "p99_us": st["lat_p99_us"], "completed": st["completed"]}
    return out


def _r(x, n=3):
    """Round for the summary (None and strings pass through)."""
    if isinstance(x, float):
        return float(f"{x:.{n}g}")
    return x


def _summary(ex: dict) -> dict:
    """The figures each configuration is judged on, rounded, in one short
    object printed at the end of the JSON line."""
    out = {}
    out["per_graph"] = {"all_ctas_ms": _r(ex.get("per_graph_ms")),
                        "x_all": _r(ex.get("speedup_vs_per_graph")),
                        "default_groups_ms": _r(ex.get("per_graph_default_groups_ms")),
                        "x_default": _r(ex.get("speedup_vs_per_graph_default_groups"))}
    out["barrier_ns"] = {"256t": _r(ex.get("barrier_ns")), "ctas": ex.get("barrier_ctas"),
                         "1024t": _r(ex.get("barrier_ns_1024_threads")),
                         "ctas_1024t": ex.get("barrier_ctas_1024_threads")}
    c1 = ex.get("c1_bfs_grid256", {})
    out["c1"] = {"ms": _r(c1.get("ms")), "ns_per_level": _r(c1.get("ns_per_level")),
                 "one_cta_ms": _r(c1.get("one_cta", {}).get("ms")),
                 "cpu_ms": _r(c1.get("cpu_baseline", {}).get("ms")),
                 "cpu_1core_ms": _r(c1.get("cpu_baseline", {}).get("ms_1core"))}
    c2 = ex.get("c2_rmat20", {})
    out["c2"] = {k: {"ms": _r(c2.get(k, {}).get("ms")), "cpu_ms": _r(c2.get(k, {}).get("cpu_ms"))}
                 for k in ("lonestar_sssp", "color", "mis")}
    c3 = ex.get("c3_pagerank_rmat22", {})
    out["c3"] = {"ms": _r(c3.get("ms")), "frac": _r(c3.get("frac_of_measured")),
                 "cpu_ms": _r(c3.get("cpu_ms"))}
    sv = ex.get("served", {})
    out["c5"] = [{"rate": r.get("rate_offered"), "p99_us": _r(r.get("p99_us")),
                  "kept_sa": _r(r.get("kept_vs_standalone")), "kills": r.get("kills")}
                 for r in sv.get("runs", [])]
    out["c5_checked"] = sv.get("checked", {}).get("ok")
    return out


def _served_check(sv, ca, ba, qg, vecs, mats, g, src, nv, reps, reserve, rate) -> dict:
    """Correctness at the benchmarked configuration: one more run at `rate`
    with every request's output kept.  The resident job's colours and BFS
    levels must equal its standalone launches' (bit for bit); every reduce
    must equal the vector's minimum; up to 200 BFS queries must equal the
    oracle's levels; every product must be within 1e-4 (relative L-inf) of a
    float64 product."""
    from oracle import oracle
    ca.run()
    ba.run()
    want_c, want_b = ca.result().copy(), ba.result().copy()
    sv.run(rate=rate, duration_s=60.0, reps=reps, seed=23, reserve=reserve, bfs_groups=32,
           bfs_edges_per_group=1 << 16, reduce_groups=4, matmul_groups=4, max_in_flight=512,
           keep_results=True)
    ok_job = bool(np.array_equal(ca.result(), want_c) and np.array_equal(ba.result(), want_b))
    rq = sv.requests()
    n_bfs = n_red = n_mm = bad = 0
    worst = 0.0
    for i, (k, a0, a1) in enumerate(zip(rq["kind"], rq["arg0"], rq["arg1"])):
        if rq["latency_ns"][i] < 0:
            bad += 1
            continue
        r = sv.result(i, int(k), int(a0))
        if k == 1 and n_bfs < 200:
            n_bfs += 1
            bad += not np.array_equal(r, oracle.lonestar_bfs(qg[a0], int(a1)))
        elif k == 2:
            n_red += 1
            bad += float(r[0]) != float(vecs[a0].min())
        elif k == 3:
            n_mm += 1
            ref = mats[a0, 0].astype(np.float64) @ mats[a0, 1].astype(np.float64)
            err = float(np.max(np.abs(r - ref)) / np.max(np.abs(ref)))
            worst = max(worst, err)
            bad += err > 1e-4
    return {"requests": int(len(rq["kind"])), "bfs_checked": n_bfs, "reduce_checked": n_red,
            "matmul_checked": n_mm, "matmul_rel_linf_max": worst, "mismatches": int(bad),
            "persistent_job_equal_to_standalone": ok_job,
            "ok": bool(ok_job and bad == 0)}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="wgm", choices=["wgm", "reference"])
    ap.add_argument("--no-extra", action="store_true", help="skip the extra measurements")
    ap.add_argument("--kernel-only", action="store_true",
                    help="batched launches only (the command profiled with ncu)")
    ap.add_argument("--sssp-kernel-only", action="store_true",
                    help="persistent SSSP on RMAT --scale only (profiled with ncu)")
    ap.add_argument("--no-tune", action="store_true",
                    help="fixed shape (256 threads, teams of 50000 edges) instead of the autotuner")
    ap.add_argument("--scale", type=int, default=20)
    ap.add_argument("--barrier-sweep", action="store_true",
                    help="ns per barrier for every barrier kind and CTA size")
    ap.add_argument("--served", action="store_true", help="served-form measurement only")
    ap.add_argument("--only", choices=["octree", "bc", "c1", "c2", "c3"],
                    help="one extra measurement alone (the commands profiled with ncu)")
    ap.add_argument("--particles", type=int, default=3_000_000, help="octree size for --only")
    ap.add_argument("--pr-scale", type=int, default=22, help="RMAT scale of --only c3")
    args = ap.parse_args()
    if args.barrier_sweep:
        return _barrier_sweep()
    if args.only:
        from gpu_workgroup_managment_gb300 import Runtime
        with Runtime() as rt:
            if args.only == "octree":
                r = _octree(rt, args.particles)
            elif args.only == "bc":
                r = _bc(rt)
            elif args.only == "c3":
                r = _c3(rt, None, args.pr_scale)
            elif args.only == "c2":
                r = _c2(rt, None)
            else:
                r = _c1(rt, None)
        print(json.dumps({"only": args.only, **r}))
        return 0
    if args.sssp_kernel_only:
        return _sssp_kernel_only(args)
    ws, rank, local = _dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as td
        td.init_process_group("gloo")
        dist = td
    if args.impl == "reference":
        rc = _reference_arm(args, ws, rank)
        if dist:
            dist.destroy_process_group()
        return rc
    if args.served:
        from gpu_workgroup_managment_gb300 import Runtime
        with Runtime(device=local) as rt:
            print(json.dumps(_served(rt)))
        return 0
    warmup = max(args.warmup, 3)

    from gpu_workgroup_managment_gb300 import Runtime
    from gpu_workgroup_managment_gb300._lib import lib
    from gpu_workgroup_managment_gb300.batch import Batch
    from gpu_workgroup_managment_gb300.runtime import pinned_copy
    from gpu_workgroup_managment_gb300 import graphs as G

    gs, jobs, meta = _batch_inputs()
    rt = Runtime(device=local)
    b = Batch(rt, gs, jobs)
    b.run(use_cuda_graph=False)
    res = b.results()
    et, vr = _job_edges(gs, jobs, res, b.offsets)
    E = int(et.sum())
    if args.no_tune:
        b.configure(256, 0, 0)
        b.configure_teams(50000, 0)
        b.run()
        b.reorder_by_last_run()
        tuned = {"threads": 256, "ctas_per_sm": 0, "piece": 0, "team_edges": 50000}
    else:
        tuned = b.autotune(reps=3)
    for _ in range(warmup):
        b.launch(True)
    rt.synchronize()
    if dist:
        dist.barrier()
    if args.kernel_only:
        lib.wgm_profiler_start(rt.handle)  # ncu --profile-from-start off sees these
    with Clocks(local) as clk:
        rt.timer_start()
        for _ in range(args.steps):
            b.launch(True)
        ms_total = rt.timer_stop()
    if args.kernel_only:
        lib.wgm_profiler_stop(rt.handle)
    ms_step = _max_over_ranks(dist, ms_total / args.steps)
    value = E * ws / (ms_step * 1e-3) / 1e9
    if not np.array_equal(b.results(), res):
        raise SystemExit("batched results changed between launches")
    if args.kernel_only:
        if rank == 0:
            print(json.dumps({"metric": "batched GTEPS", "value": value, "ms_per_step": ms_step,
                              "edges_traversed": E, "tuned": tuned}))
        b.close()
        rt.close()
        return 0

    # e2e through the public API: pinned host graphs up, batched launch, results down
    rows, cols, wts = b.pack(gs)
    rows, p1 = pinned_copy(rows)
    cols, p2 = pinned_copy(cols)
    wts, p3 = pinned_copy(wts)
    out, p4 = pinned_copy(np.empty(int(b.offsets[-1]), np.uint32))
    out2, p5 = pinned_copy(np.empty(int(b.offsets[-1]), np.uint32))
    keep = [p1, p2, p3, p4, p5]
    # serial: each step uploads, launches and reads back before the next starts
    for _ in range(2):
        b.upload_packed(rows, cols, wts)
        b.launch(True)
        b.results(out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b.upload_packed(rows, cols, wts)
        b.launch(True)
        b.results(out)
    serial_s = _max_over_ranks(dist, (time.perf_counter() - t0) / args.steps)
    if not np.array_equal(out, res):
        raise SystemExit("e2e results differ")
    # pipelined (the public submit/wait API): step k+1's upload and step k-1's
    # read-back run under step k's kernel; every step still moves all its bytes
    for k in range(2):
        b.submit_packed(rows, cols, wts, out if k % 2 == 0 else out2)
    b.wait()
    out.fill(0)
    out2.fill(0)
    t0 = time.perf_counter()
    for k in range(args.steps):
        b.submit_packed(rows, cols, wts, out if k % 2 == 0 else out2)
    b.wait()
    e2e_s = _max_over_ranks(dist, (time.perf_counter() - t0) / args.steps)
    if not np.array_equal(out, res) or (args.steps > 1 and not np.array_equal(out2, res)):
        raise SystemExit("pipelined e2e results differ")
    h2d = rows.nbytes + cols.nbytes + wts.nbytes
    d2h = out.nbytes
    for p in keep:
        lib.wgm_host_free(p)

    bytes_alg = _alg_bytes(gs, jobs, et, vr)
    peak, peak_kind = _peak_hbm()
    achieved = bytes_alg / (ms_step * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "jobs": len(jobs), "graphs": meta["graphs"],
                   "nodes_total": meta["nodes_total"], "edges_total": meta["edges_total"],
                   "edges_traversed": E, "parallelism": f"replicas{args.gpus}",
                   "cuda_graph": True, "tuned": tuned,
                   "l2": "inputs larger than L2 (1.4 GB CSR + weights), no flush"},
        "e2e": {"value": E * ws / e2e_s / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                "api": "wgm_batch_submit_packed per step (pipelined, two device copies), "
                       "wgm_batch_wait at the end",
                "serial_value": E * ws / serial_s / 1e9, "serial_ms_per_step": serial_s * 1e3},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": _traffic("wgm_k_batch", "batch512"),
                     "bytes_alg_per_launch": bytes_alg, "kernel": "wgm_k_batch"},
        "clocks": clk.summary(),
        "gpu_launches": args.steps,
    }
    if rank == 0 and not args.no_extra:
        extra = {}
        pg = b.run_per_graph()
        pg = min(pg, b.run_per_graph())
        if not np.array_equal(b.results(), res):
            raise SystemExit("per-graph results differ from the batched ones")
        extra["per_graph_ms"] = pg
        extra["per_graph_gteps"] = E / (pg * 1e-3) / 1e9
        extra["speedup_vs_per_graph"] = pg / ms_step
        pgd = b.run_per_graph(default_groups=True)
        pgd = min(pgd, b.run_per_graph(default_groups=True))
        if not np.array_equal(b.results(), res):
            raise SystemExit("per-graph (default groups) results differ from the batched ones")
        extra["per_graph_default_groups_ms"] = pgd
        extra["per_graph_default_groups_gteps"] = E / (pgd * 1e-3) / 1e9
        extra["speedup_vs_per_graph_default_groups"] = pgd / ms_step
        st = b.job_stats()
        extra["makespan_ms"] = float(st["end_ns"].max()) / 1e6
        extra["max_team"] = int(st["team"].max())
        # the default barrier (automatic kind: counting up to 384 CTAs, sense above)
        # os_freq's default block (256 threads, os_freq.cpp:38) on every
        # co-resident CTA, then 1024-thread CTAs
        bb = rt.barrier_bench(iterations=100000, threads_per_wg=256)
        extra["barrier_ns"] = bb["ns_per_barrier"]
        extra["barrier_ctas"] = bb["groups"]
        extra["barrier_count"] = bb["barriers"]
        extra["barrier_kind"] = "sense" if bb["groups"] > 384 else "count"
        bb = rt.barrier_bench(iterations=100000, threads_per_wg=1024)
        extra["barrier_ns_1024_threads"] = bb["ns_per_barrier"]
        extra["barrier_ctas_1024_threads"] = bb["groups"]
        extra["barrier_kind_1024_threads"] = "sense" if bb["groups"] > 384 else "count"
        extra["sssp_rmat20"] = _sssp_rmat(rt, 20, 5, 3)
        try:
            extra["octree"] = _octree(rt)
        except Exception as exc:  # reported, not hidden
            extra["octree"] = {"error": repr(exc)}
        try:
            extra["bc_rmat12"] = _bc(rt)
        except Exception as exc:  # reported, not hidden
            extra["bc_rmat12"] = {"error": repr(exc)}
        for key, fn in (("c1_bfs_grid256", _c1), ("c2_rmat20", _c2), ("c3_pagerank_rmat22", _c3)):
            try:
                extra[key] = fn(rt, extra.get("barrier_ns_1024_threads"))
            except Exception as exc:  # reported, not hidden
                extra[key] = {"error": repr(exc)}
        try:
            extra["served"] = _served(rt)
        except Exception as exc:  # reported, not hidden
            extra["served"] = {"error": repr(exc)}
        line["extra"] = extra
    b.close()
    if rank == 0 and "extra" in line:
        line["summary"] = _summary(line["extra"])
    if rank == 0:
        from oracle import oracle
        arena = oracle.BatchArena(gs, jobs)
        d = arena.run()
        if not np.array_equal(d, res):
            raise SystemExit("batched results differ from the oracle")
        line["config"]["oracle_checked"] = True
        runs, t_tot = 0, 0.0
        while runs < 20 and t_tot < 12.0:
            t0 = time.perf_counter()
            arena.run()
            t_tot += time.perf_counter() - t0
            runs += 1
        line["cpu_baseline"] = {
            "value": E * runs / t_tot / 1e9, "unit": "GTEPS", "cores": oracle.threads(),
            "kind": "port",
            "sample": f"{runs} runs of all {len(jobs)} jobs, jobs spread over the host "
                      "threads, each the serial restatement of lonestar bfs.cl/sssp.cl"}
        if "summary" in line:  # keep the compact figures at the end of the line
            line["summary"] = line.pop("summary")
        print(json.dumps(line))
    rt.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
