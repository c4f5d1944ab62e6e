"""Benchmark of the persistent graph path on one GB300 (or N replicas).

Default workload: persistent Lonestar SSSP on RMAT scale 20 (edge factor 16,
(a,b,c) = (0.57,0.19,0.19), seeded, symmetrised, uint32 weights in [1,1000]),
source = the highest-degree vertex.  A step = one persistent launch (discovery,
device-side init, worklist levels) over the graph resident in HBM.

JSON line keys (one line, rank 0):
  value        GTEPS = traversed edges / device time per step (CUDA events on
               the launching stream; inputs larger than L2)
  e2e          the same metric through the public API with host buffers:
               per step pinned H2D of the CSR + weights, the run, D2H of dist
  roofline     achieved algorithmic GB/s of the SSSP kernel vs the HBM peak
  cpu_baseline the OpenMP oracle (a restatement of the reference's kernel) on
               the machine's host cores, on a bounded sample
  extra        barrier ns (10^6 barriers over every co-resident CTA), grid BFS
`--impl reference` times the reference's algorithm on the host cores (the
oracle port: the reference's OpenCL 2.0 program needs fine-grained SVM atomics,
which no runtime on the box provides).
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
RMAT_SCALE, RMAT_EF, RMAT_SEED = 20, 16, 1
HBM_FALLBACK_GBS = 6800.0


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

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
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


def _traversed(g, dist) -> tuple[int, int]:
    """E_t = out-degree summed over reached vertices, V_r = reached vertices."""
    reached = dist != INF
    return int(g.degrees()[reached].sum()), int(reached.sum())


def _cpu_baseline(g, src, budget_s: float = 12.0) -> dict:
    from oracle import oracle
    runs, t_tot, et = 0, 0.0, 0
    while runs < 50 and t_tot < budget_s:
        t0 = time.perf_counter()
        d = oracle.lonestar_sssp(g, src, omp=True)
        t_tot += time.perf_counter() - t0
        runs += 1
        if runs == 1:
            et, _ = _traversed(g, d)
    return {"value": et * runs / t_tot / 1e9, "unit": "GTEPS", "cores": oracle.threads(),
            "kind": "port",
            "sample": f"{runs} full SSSP runs on the same RMAT graph from the max-degree vertex "
                      f"(OpenMP restatement of lonestar sssp.cl)"}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="wgm", choices=["wgm", "reference"])
    ap.add_argument("--no-extra", action="store_true")
    ap.add_argument("--scale", type=int, default=RMAT_SCALE)
    ap.add_argument("--kernel-only", action="store_true",
                    help="time the device steps only (no e2e, extras or CPU baseline); "
                         "the command profiled with ncu")
    ap.add_argument("--barrier-sweep", action="store_true",
                    help="ns per barrier for every barrier kind and CTA size, one JSON line each")
    args = ap.parse_args()
    scale = args.scale
    if args.barrier_sweep:
        from gpu_workgroup_managment_gb300 import Runtime
        kinds = {0: "sense", 1: "xf", 2: "tree", 3: "count"}
        with Runtime() as rt:
            for threads in (128, 256, 512, 1024):
                for kind, name in kinds.items():
                    r = rt.barrier_bench(iterations=20000, threads_per_wg=threads,
                                         barrier_kind=kind)
                    print(json.dumps({"barrier": name, "threads_per_cta": threads,
                                      "ctas": r["groups"], "barriers": r["barriers"],
                                      "ns_per_barrier": r["ns_per_barrier"]}))
        return 0
    warmup = max(args.warmup, 3)
    ws, rank, local = _dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as td
        td.init_process_group("gloo")
        dist = td

    from gpu_workgroup_managment_gb300 import graphs

    workload = f"rmat{scale}_sssp"
    config = {"workload": f"persistent Lonestar SSSP, RMAT scale {scale} edge factor "
                          f"{RMAT_EF} (0.57,0.19,0.19) seed {RMAT_SEED}, weights U[1,1000], "
                          f"source = max-degree vertex",
              "graph": f"rmat{scale}", "parallelism": f"replicas{args.gpus}",
              "l2": "inputs larger than L2 (CSR+weights > 129 MB), no flush"}

    if args.impl == "reference":
        if rank != 0:
            return 0
        g = graphs.rmat(scale, RMAT_EF, seed=RMAT_SEED)
        src = graphs.max_degree_vertex(g)
        from oracle import oracle
        for _ in range(1):
            oracle.lonestar_sssp(g, src, omp=True)
        times, et = [], 0
        for i in range(args.steps):
            t0 = time.perf_counter()
            d = oracle.lonestar_sssp(g, src, omp=True)
            times.append(time.perf_counter() - t0)
            if i == 0:
                et, _ = _traversed(g, d)
        mean = sum(times) / len(times)
        v = et / mean / 1e9
        line = {"impl": "reference", "metric": "SSSP GTEPS (persistent Lonestar, RMAT-20)",
                "value": v, "unit": "GTEPS", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": 1, "ms_per_step": mean * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
                "config": config,
                "cpu_baseline": {"value": v, "unit": "GTEPS", "cores": oracle.threads(),
                                 "kind": "port",
                                 "sample": f"{args.steps} full SSSP runs (OpenMP restatement "
                                           "of the reference's sssp.cl; the reference's OpenCL "
                                           "2.0 SVM program cannot run here)"},
                "e2e": {"value": v, "unit": "GTEPS", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    from gpu_workgroup_managment_gb300 import PersistentApp, Runtime
    from gpu_workgroup_managment_gb300._lib import lib
    from gpu_workgroup_managment_gb300.runtime import pinned_copy

    g = graphs.rmat(scale, RMAT_EF, seed=RMAT_SEED)
    src = graphs.max_degree_vertex(g)
    rt = Runtime(device=local)
    app = PersistentApp(rt, "lonestar_sssp", g, source=src)
    # correctness of the benchmarked kernel (checked once, outside the timing)
    st0 = app.run()
    d = app.result()
    et, vr = _traversed(g, d)

    for _ in range(warmup):
        app.launch()
    rt.synchronize()
    if dist:
        dist.barrier()
    with Clocks(local) as clk:
        rt.timer_start()
        for _ in range(args.steps):
            app.launch()
        ms_total = rt.timer_stop()
    ms_step = ms_total / args.steps
    if dist:
        import torch
        t = torch.tensor([ms_step], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    value = et * ws / (ms_step * 1e-3) / 1e9
    if args.kernel_only:
        if rank == 0:
            print(json.dumps({"metric": "SSSP GTEPS", "value": value, "ms_per_step": ms_step,
                              "levels": st0.rounds, "groups": st0.groups,
                              "edges_traversed": et, "workload": workload}))
        app.close()
        rt.close()
        return 0

    # e2e through the public API with pinned host buffers
    rp, p1 = pinned_copy(g.row_ptr)
    cl, p2 = pinned_copy(g.col)
    wt, p3 = pinned_copy(g.weights)
    out, p4 = pinned_copy(np.empty(g.num_nodes, np.uint32))
    hg = graphs.Graph(rp, cl, wt)
    for _ in range(2):
        app.upload(hg)
        app.launch()
        app.result(out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        app.upload(hg)
        app.launch()
        app.result(out)
    e2e_s = (time.perf_counter() - t0) / args.steps
    assert np.array_equal(out, d)
    h2d = rp.nbytes + cl.nbytes + wt.nbytes
    d2h = out.nbytes

    bytes_alg = 12 * et + 20 * vr  # SSSP algorithmic bytes per launch
    peak, peak_kind = _peak_hbm()
    achieved = bytes_alg / (ms_step * 1e-3) / 1e9
    line = {
        "metric": "SSSP GTEPS (persistent Lonestar, RMAT-20)", "value": value, "unit": "GTEPS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic", "config": config,
        "e2e": {"value": et / e2e_s / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": _traffic("wgm_k_sssp", workload),
                     "bytes_alg_per_launch": bytes_alg, "edges_traversed": et,
                     "vertices_reached": vr, "levels": st0.rounds, "groups": st0.groups},
        "clocks": clk.summary(),
        "gpu_launches": args.steps,
    }
    for ptr in (p1, p2, p3, p4):
        lib.wgm_host_free(ptr)

    if rank == 0 and not args.no_extra:
        extra = {}
        bb = rt.barrier_bench(iterations=100000, threads_per_wg=256)
        extra["barrier_ns"] = bb["ns_per_barrier"]
        extra["barrier_groups"] = bb["groups"]
        gg = graphs.lonestar_view(graphs.grid(256, 256))
        with PersistentApp(rt, "lonestar_bfs", gg) as ga:
            ga.run()
            rt.timer_start()
            for _ in range(5):
                ga.launch()
            ms = rt.timer_stop() / 5
            lv = ga.result()
        extra["grid256_bfs_ms"] = ms
        extra["grid256_bfs_levels"] = int(lv.max())
        extra["grid256_ns_per_level"] = ms * 1e6 / int(lv.max())
        line["extra"] = extra
    if rank == 0:
        line["cpu_baseline"] = _cpu_baseline(g, src)
        print(json.dumps(line))
    app.close()
    rt.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
