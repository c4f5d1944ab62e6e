"""Seeded benchmark inputs built without the product library.

TEST INFRASTRUCTURE ONLY: bench.py's reference arm and CPU baselines build
their graphs here (liboracle.so + numpy), so a CPU arm never maps libwgm.so.
The definitions (grid layout, RMAT sampling, weights, the batched workload's
draws) are the ones the product's generators implement; tests/test_bench_cpu.py
checks that both produce identical arrays.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import oracle


@dataclass
class HostGraph:
    """0-based CSR: row_ptr[V+1] int32, col[E] int32, weights[E] uint32 or None."""
    row_ptr: np.ndarray
    col: np.ndarray
    weights: np.ndarray | None = None
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def num_nodes(self) -> int:
        return int(self.row_ptr.shape[0] - 1)

    @property
    def num_edges(self) -> int:
        return int(self.col.shape[0])

    def degrees(self) -> np.ndarray:
        return np.maximum(np.diff(self.row_ptr.astype(np.int64)), 0)


def grid(rows: int, cols: int | None = None) -> HostGraph:
    """4-connected grid, node r*cols+c, neighbours (up, left, right, down)."""
    cols = rows if cols is None else cols
    lib = oracle.lib()
    E = int(lib.oracle_grid_edges(rows, cols))
    rp = np.empty(rows * cols + 1, np.int32)
    cl = np.empty(max(E, 1), np.int32)
    if lib.oracle_gen_grid(rows, cols, rp.ctypes.data, cl.ctypes.data) != 0:
        raise ValueError(f"grid {rows}x{cols}")
    return HostGraph(rp, cl[:E].copy(), None, f"grid{rows}x{cols}")


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 1, permute: bool = True, wmin: int = 1, wmax: int = 1000) -> HostGraph:
    """RMAT, symmetrised, self loops and duplicates removed, rows sorted,
    weights U[wmin, wmax] per undirected edge (wmax = 0: none)."""
    lib = oracle.lib()
    rp, cl, wt = C.c_void_p(), C.c_void_p(), C.c_void_p()
    ne = C.c_int64()
    if lib.oracle_gen_rmat(scale, edge_factor, a, b, c, seed, int(permute), wmin, wmax,
                           C.byref(rp), C.byref(cl), C.byref(wt), C.byref(ne)) != 0:
        raise MemoryError(f"rmat scale {scale}")
    V, E = 1 << scale, ne.value
    try:
        row_ptr = np.ctypeslib.as_array(C.cast(rp, C.POINTER(C.c_int32)), (V + 1,)).copy()
        col = (np.ctypeslib.as_array(C.cast(cl, C.POINTER(C.c_int32)), (E,)).copy()
               if E else np.zeros(0, np.int32))
        w = None
        if wmax > 0 and E:
            w = np.ctypeslib.as_array(C.cast(wt, C.POINTER(C.c_uint32)), (E,)).copy()
    finally:
        for p in (rp, cl, wt):
            if p.value:
                lib.oracle_free(p)
    return HostGraph(row_ptr, col, w, f"rmat{scale}")


def uniform_weights(g: HostGraph, seed: int, wmin: int = 1, wmax: int = 1000) -> np.ndarray:
    """Weight of {u, v}: wmin + splitmix((min << 32 | max) ^ (seed * golden
    mod 2^64)) mod (wmax - wmin + 1), without SplitMix64's initial increment;
    equal in both directions."""
    src = np.repeat(np.arange(g.num_nodes, dtype=np.uint64), g.degrees())
    dst = g.col[: src.shape[0]].astype(np.uint64)
    key = (np.minimum(src, dst) << np.uint64(32)) | np.maximum(src, dst)
    key ^= np.uint64((seed * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF)
    key = (key ^ (key >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    key = (key ^ (key >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    key ^= key >> np.uint64(31)
    w = np.zeros(g.num_edges, np.uint32)
    w[: src.shape[0]] = (np.uint64(wmin) + key % np.uint64(wmax - wmin + 1)).astype(np.uint32)
    return w


def batch_workload(n_graphs: int = 512, seed: int = 2024, mu: float = 13.0, sigma: float = 2.5,
                   lo: int = 8, hi: int = 18) -> tuple[list, list, dict]:
    """The batched benchmark: log2(V) ~ Normal(mu, sigma) clamped to [lo, hi]
    (numpy default_rng(seed)); even graphs RMAT (0.57, 0.19, 0.19) of scale
    round(x) and edge factor max(1, U{8..32} // 2), seed seed*1000+i; odd
    graphs grids of round(sqrt(round(2^x))) rows, weights seeded the same
    way; one BFS then one SSSP job per graph from U{0..V-1} sources."""
    rng = np.random.default_rng(seed)
    graphs, jobs = [], []
    for i in range(n_graphs):
        x = float(np.clip(rng.normal(mu, sigma), lo, hi))
        if i % 2 == 0:
            scale = int(round(x))
            deg = int(rng.integers(8, 33))
            g = rmat(scale, max(1, deg // 2), seed=seed * 1000 + i)
        else:
            v = int(round(2 ** x))
            rows = max(1, int(round(v ** 0.5)))
            cols = max(1, int(round(v / rows)))
            g = grid(rows, cols)
            g.weights = uniform_weights(g, seed * 1000 + i)
        graphs.append(g)
        jobs.append((i, "bfs", int(rng.integers(0, g.num_nodes))))
        jobs.append((i, "sssp", int(rng.integers(0, g.num_nodes))))
    meta = {"graphs": n_graphs, "seed": seed, "log2_nodes_mu": mu, "log2_nodes_sigma": sigma,
            "log2_nodes_range": [lo, hi], "jobs": len(jobs),
            "nodes_total": int(sum(g.num_nodes for g in graphs)),
            "edges_total": int(sum(g.num_edges for g in graphs))}
    return graphs, jobs, meta
