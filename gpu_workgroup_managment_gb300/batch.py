"""Batched form: many graphs and (graph, algorithm, source) jobs in one
persistent launch fed by a device work queue (wgm_batch_* in include/wgm.h).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import graphs as G
from ._lib import WgmGraphDesc, check, lib

ALGOS = {"bfs": 0, "sssp": 1}


class Batch:
    def __init__(self, rt, graphs: list, jobs: list):
        """jobs: (graph index, "bfs" | "sssp", source) per job."""
        self.rt = rt
        self.graphs = graphs
        self.jobs = jobs
        self._descs = (WgmGraphDesc * len(graphs))()
        self._fill(graphs)
        jg = np.array([j[0] for j in jobs], np.int32)
        ja = np.array([ALGOS[j[1]] for j in jobs], np.int32)
        js = np.array([j[2] for j in jobs], np.int32)
        h = C.c_void_p()
        check(lib.wgm_batch_create(rt.handle, len(graphs), self._descs, len(jobs),
                                   jg.ctypes.data, ja.ctypes.data, js.ctypes.data, C.byref(h)),
              "wgm_batch_create")
        self._h = h
        self.sizes = np.array([graphs[j[0]].num_nodes for j in jobs], np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)])

    def _fill(self, graphs):
        self._keep = []
        for i, g in enumerate(graphs):
            d = self._descs[i]
            d.num_nodes = g.num_nodes
            d.num_edges = g.num_edges
            d.row_ptr = g.row_ptr.ctypes.data
            d.col = g.col.ctypes.data if g.num_edges else None
            d.weights = None if g.weights is None else g.weights.ctypes.data
            self._keep.append((g.row_ptr, g.col, g.weights))

    def upload(self, graphs: list) -> None:
        self._fill(graphs)
        check(lib.wgm_batch_upload(self._h, self._descs), "wgm_batch_upload")

    def graph_offsets(self) -> tuple[np.ndarray, np.ndarray]:
        """Where each graph's rows and cols/weights sit in the packed layout."""
        ro = np.empty(len(self.graphs), np.int64)
        co = np.empty(len(self.graphs), np.int64)
        check(lib.wgm_batch_graph_offsets(self._h, ro.ctypes.data, co.ctypes.data))
        return ro, co

    def pack(self, graphs: list, out: tuple | None = None) -> tuple:
        """Concatenate graphs' rows, cols and weights in the packed layout
        (into `out` = (rows, cols, weights) arrays when given)."""
        ro, co = self.graph_offsets()
        nr = int(ro[-1] + graphs[-1].num_nodes + 1)
        ne = int(co[-1] + graphs[-1].num_edges)
        rows, cols, wts = out if out is not None else (
            np.empty(nr, np.int32), np.empty(max(ne, 1), np.int32), np.empty(max(ne, 1), np.uint32))
        for g, r0, c0 in zip(graphs, ro, co):
            rows[r0:r0 + g.num_nodes + 1] = g.row_ptr
            cols[c0:c0 + g.num_edges] = g.col
            if g.weights is not None:
                wts[c0:c0 + g.num_edges] = g.weights
        return rows, cols, wts

    def upload_packed(self, rows: np.ndarray, cols: np.ndarray, wts: np.ndarray) -> None:
        check(lib.wgm_batch_upload_packed(self._h, rows.ctypes.data, cols.ctypes.data,
                                          wts.ctypes.data), "wgm_batch_upload_packed")

    def submit_packed(self, rows: np.ndarray, cols: np.ndarray, wts: np.ndarray,
                      out: np.ndarray) -> None:
        """Queue one pipelined step (upload, launch, read-back into `out`);
        the arrays must stay alive and untouched until wait()."""
        if out.dtype != np.uint32 or out.shape[0] < int(self.offsets[-1]):
            raise ValueError("out must hold every job's distances (uint32)")
        check(lib.wgm_batch_submit_packed(self._h, rows.ctypes.data, cols.ctypes.data,
                                          wts.ctypes.data, out.ctypes.data),
              "wgm_batch_submit_packed")

    def wait(self) -> None:
        check(lib.wgm_batch_wait(self._h), "wgm_batch_wait")

    def configure(self, threads: int = 256, ctas_per_sm: int = 0, piece: int = 0) -> None:
        check(lib.wgm_batch_configure(self._h, threads, ctas_per_sm, piece), "batch_configure")

    def configure_kernel(self, max_regs: int) -> None:
        """Register budget of the batched kernel: 64, 80 or 96 per thread."""
        check(lib.wgm_batch_configure_kernel(self._h, int(max_regs)), "configure_kernel")

    def configure_teams(self, team_edges: int = 0, max_team: int = 0) -> None:
        """A job of E edges runs on ceil(E / team_edges) CTAs, at most max_team
        (0 = defaults: total edges / grid, a quarter of the grid)."""
        check(lib.wgm_batch_configure_teams(self._h, team_edges, max_team), "configure_teams")

    def configure_local(self, rounds: int) -> None:
        """Warp-local continuation rounds per level (0 = plain levels)."""
        check(lib.wgm_batch_configure_local(self._h, rounds), "configure_local")

    def configure_sssp(self, delta_mult: float = 20.0, far_cap: int = 0) -> None:
        """Near-far SSSP buckets of delta_mult x the mean edge weight (0 = the
        Bellman-Ford worklist); far lists of far_cap entries (0 = 2V + 64)."""
        check(lib.wgm_batch_configure_sssp(self._h, float(delta_mult), int(far_cap)),
              "configure_sssp")

    def configure_bfs_one_cta(self, max_avg_degree: float = 5.0) -> None:
        """BFS jobs on graphs of average degree <= max_avg_degree run on one
        CTA whatever their size (0: teams by edges for every job)."""
        check(lib.wgm_batch_configure_bfs_one_cta(self._h, float(max_avg_degree)),
              "wgm_batch_configure_bfs_one_cta")

    def configure_sssp_dense(self, light_mult: float = 0.0) -> None:
        """SSSP jobs on graphs of average degree >= 6: buckets of light_mult x
        the mean weight, heavy edges relaxed once per bucket (0: off)."""
        check(lib.wgm_batch_configure_sssp_dense(self._h, float(light_mult)),
              "configure_sssp_dense")

    def launch(self, use_cuda_graph: bool = True) -> None:
        check(lib.wgm_batch_launch(self._h, int(use_cuda_graph)), "wgm_batch_launch")

    def launch_per_graph(self) -> None:
        check(lib.wgm_batch_launch_per_graph(self._h), "wgm_batch_launch_per_graph")

    def run(self, use_cuda_graph: bool = True) -> float:
        ms = C.c_double()
        check(lib.wgm_batch_run(self._h, int(use_cuda_graph), C.byref(ms)), "wgm_batch_run")
        return ms.value

    def run_per_graph(self, default_groups: bool = False) -> float:
        """One standalone persistent launch per job on every co-resident CTA,
        or (default_groups) on the group count wgm_run_persistent picks."""
        ms = C.c_double()
        check(lib.wgm_batch_run_per_graph_sized(self._h, int(default_groups), C.byref(ms)),
              "wgm_batch_run_per_graph_sized")
        return ms.value

    def result(self, job: int) -> np.ndarray:
        out = np.empty(int(self.sizes[job]), np.uint32)
        check(lib.wgm_batch_read(self._h, job, out.ctypes.data, out.shape[0]))
        return out

    def results(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(int(self.offsets[-1]), np.uint32)
        check(lib.wgm_batch_read_all(self._h, out.ctypes.data, out.shape[0]))
        return out

    def info(self) -> dict:
        n, e, t, c, p = C.c_int64(), C.c_int64(), C.c_int(), C.c_int(), C.c_int()
        check(lib.wgm_batch_info(self._h, C.byref(n), C.byref(e), C.byref(t), C.byref(c),
                                 C.byref(p)))
        return {"total_nodes": n.value, "total_edges": e.value, "threads": t.value,
                "ctas_per_sm": c.value, "piece": p.value}

    def job_stats(self) -> dict:
        """Per job of the last batched launch (caller's order): device start and
        end in ns from the earliest start, team size, levels run."""
        n = len(self.jobs)
        st, en = np.empty(n, np.int64), np.empty(n, np.int64)
        tm, lv = np.empty(n, np.int32), np.empty(n, np.int32)
        check(lib.wgm_batch_job_stats(self._h, st.ctypes.data, en.ctypes.data, tm.ctypes.data,
                                      lv.ctypes.data), "wgm_batch_job_stats")
        return {"start_ns": st, "end_ns": en, "team": tm, "levels": lv}

    def job_work(self) -> np.ndarray:
        """Edges each job of the last batched launch walked (caller's order);
        a vertex visited again counts its edges again."""
        w = np.empty(len(self.jobs), np.int64)
        check(lib.wgm_batch_job_work(self._h, w.ctypes.data), "wgm_batch_job_work")
        return w

    def reorder_by_last_run(self) -> None:
        """Queue the jobs longest first by their device time in the last
        batched launch."""
        check(lib.wgm_batch_reorder_by_last_run(self._h), "wgm_batch_reorder_by_last_run")

    def autotune(self, reps: int = 3) -> dict:
        t, c, p, ms = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        check(lib.wgm_batch_autotune(self._h, reps, C.byref(t), C.byref(c), C.byref(p),
                                     C.byref(ms)), "wgm_batch_autotune")
        te, mt = C.c_int64(), C.c_int()
        check(lib.wgm_batch_team_info(self._h, C.byref(te), C.byref(mt)))
        dm, fc, rg = C.c_double(), C.c_int(), C.c_int()
        check(lib.wgm_batch_sssp_info(self._h, C.byref(dm), C.byref(fc)))
        check(lib.wgm_batch_kernel_info(self._h, C.byref(rg)))
        lm = C.c_double()
        check(lib.wgm_batch_sssp_dense_info(self._h, C.byref(lm)))
        return {"threads": t.value, "ctas_per_sm": c.value, "piece": p.value, "ms": ms.value,
                "team_edges": te.value, "max_team": mt.value, "sssp_delta_mult": dm.value,
                "sssp_dense_mult": lm.value, "max_regs": rg.value}

    def close(self):
        if self._h:
            lib.wgm_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def traversed_edges(g, dist: np.ndarray) -> int:
    """E_t: out-degree summed over the reached vertices (INF = 1e9)."""
    return int(g.degrees()[dist != 1000000000].sum())


def batch_workload(n_graphs: int = 512, seed: int = 2024, mu: float = 13.0, sigma: float = 2.5,
                   lo: int = 8, hi: int = 18) -> tuple[list, list, dict]:
    """Seeded batch: log2(V) ~ Normal(mu, sigma) clamped to [lo, hi]; even
    graphs RMAT (a,b,c)=(0.57,0.19,0.19) with average degree U{8..32}, odd
    graphs near-square 2D grids; weights U[1,1000] per undirected edge; one
    BFS and one SSSP job per graph from seeded sources."""
    rng = np.random.default_rng(seed)
    graphs, jobs = [], []
    for i in range(n_graphs):
        x = float(np.clip(rng.normal(mu, sigma), lo, hi))
        if i % 2 == 0:
            scale = int(round(x))
            deg = int(rng.integers(8, 33))
            g = G.rmat(scale, max(1, deg // 2), seed=seed * 1000 + i)
        else:
            v = int(round(2 ** x))
            rows = max(1, int(round(v ** 0.5)))
            cols = max(1, int(round(v / rows)))
            g = G.grid(rows, cols)
            g.weights = G.uniform_weights(g, seed * 1000 + i)
        graphs.append(g)
        jobs.append((i, "bfs", int(rng.integers(0, g.num_nodes))))
        jobs.append((i, "sssp", int(rng.integers(0, g.num_nodes))))
    meta = {"graphs": n_graphs, "seed": seed, "log2_nodes_mu": mu, "log2_nodes_sigma": sigma,
            "log2_nodes_range": [lo, hi], "jobs": len(jobs),
            "nodes_total": int(sum(g.num_nodes for g in graphs)),
            "edges_total": int(sum(g.num_edges for g in graphs))}
    return graphs, jobs, meta
