"""Graphs for the persistent apps: seeded generators (through libwgm), the
reference loaders' CSR semantics, priorities, and on-disk formats.

A Graph is a 0-based CSR: row_ptr[V+1] (int32), col[E] (int32) and optional
weights[E] (uint32).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._lib import check, lib


@dataclass
class Graph:
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


def _as_graph(row_ptr, col, weights=None, name="", **meta) -> Graph:
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    wt = None if weights is None else np.ascontiguousarray(weights, dtype=np.uint32)
    return Graph(rp, cl, wt, name, dict(meta))


def grid(rows: int, cols: int | None = None) -> Graph:
    """4-connected grid, node id r*cols+c, neighbours (up, left, right, down)."""
    cols = rows if cols is None else cols
    V = rows * cols
    E = 4 * V - 2 * rows - 2 * cols
    rp = np.empty(V + 1, np.int32)
    cl = np.empty(max(E, 1), np.int32)
    ne = C.c_int64()
    check(lib.wgm_gen_grid(rows, cols, rp.ctypes.data, cl.ctypes.data, C.byref(ne)), "gen_grid")
    return Graph(rp, cl[: ne.value].copy(), None, f"grid{rows}x{cols}", {"rows": rows, "cols": cols})


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
         c: float = 0.19, seed: int = 1, permute: bool = True, wmin: int = 1,
         wmax: int = 1000) -> Graph:
    """RMAT graph: symmetrised, self loops and duplicates removed, rows sorted,
    weights uniform in [wmin, wmax] per undirected edge (wmax=0: none)."""
    h = C.c_void_p()
    check(lib.wgm_gen_rmat(scale, edge_factor, a, b, c, seed, int(permute), wmin, wmax,
                           C.byref(h)), "gen_rmat")
    try:
        V, E = C.c_int32(), C.c_int64()
        lib.wgm_host_graph_info(h, C.byref(V), C.byref(E))
        rp, cl, wt = C.c_void_p(), C.c_void_p(), C.c_void_p()
        lib.wgm_host_graph_arrays(h, C.byref(rp), C.byref(cl), C.byref(wt))
        row_ptr = np.ctypeslib.as_array(C.cast(rp, C.POINTER(C.c_int32)), (V.value + 1,)).copy()
        col = (np.ctypeslib.as_array(C.cast(cl, C.POINTER(C.c_int32)), (E.value,)).copy()
               if E.value else np.zeros(0, np.int32))
        weights = None
        if wt.value and E.value:
            weights = np.ctypeslib.as_array(C.cast(wt, C.POINTER(C.c_uint32)), (E.value,)).copy()
    finally:
        lib.wgm_host_graph_free(h)
    return Graph(row_ptr, col, weights, f"rmat{scale}",
                 {"scale": scale, "edge_factor": edge_factor, "a": a, "b": b, "c": c,
                  "seed": seed, "permute": permute})


def uniform_weights(g: Graph, seed: int, wmin: int = 1, wmax: int = 1000) -> np.ndarray:
    """Symmetric weights in [wmin, wmax]: one value per undirected edge."""
    V = g.num_nodes
    src = np.repeat(np.arange(V, dtype=np.int64), g.degrees())
    lo = np.minimum(src, g.col[: src.shape[0]]).astype(np.uint64)
    hi = np.maximum(src, g.col[: src.shape[0]]).astype(np.uint64)
    x = (lo << np.uint64(32)) | hi
    x ^= np.uint64(seed * 0x9E3779B97F4A7C15 % (1 << 64))
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    x ^= x >> np.uint64(31)
    w = np.zeros(g.num_edges, np.uint32)
    w[: src.shape[0]] = (np.uint64(wmin) + x % np.uint64(wmax - wmin + 1)).astype(np.uint32)
    return w


def max_degree_vertex(g: Graph) -> int:
    """Highest-degree vertex, lowest id on ties."""
    return int(np.argmax(g.degrees()))


def swap_labels(g: Graph, s: int) -> Graph:
    """Relabel vertices 0 and s (the reference hard-wires source 0, bfs.cl:236-240,
    pannotia sssp.h:21): the returned graph's vertex 0 is g's vertex s."""
    if s == 0:
        return g
    V = g.num_nodes
    perm = np.arange(V, dtype=np.int64)
    perm[0], perm[s] = s, 0  # new id -> old id
    inv = np.argsort(perm)   # old id -> new id
    deg = g.degrees()[perm]
    rp = np.zeros(V + 1, np.int64)
    rp[1:] = np.cumsum(deg)
    col = np.empty(int(rp[-1]), np.int32)
    wt = None if g.weights is None else np.empty(int(rp[-1]), np.uint32)
    for new in range(V):
        old = perm[new]
        a, b = g.row_ptr[old], g.row_ptr[old] + deg[new]
        seg = inv[g.col[a:b]]
        order = np.argsort(seg, kind="stable")
        col[rp[new]:rp[new + 1]] = seg[order]
        if wt is not None:
            wt[rp[new]:rp[new + 1]] = g.weights[a:b][order]
    return Graph(rp.astype(np.int32), col, wt, g.name + f"_swap{s}", dict(g.meta, swapped=s))


def lonestar_view(g: Graph) -> Graph:
    """The CSR the Lonestar kernels walk after readFromGR: the `.gr` loader sets
    psrc[nnodes] = nedges with 1-based psrc (lonestar/graph_apps/bfs/bfs.h:41-43,
    141-146), so the last vertex loses its last out-edge: row_ptr[V] = E - 1."""
    rp = g.row_ptr.copy()
    if g.num_edges > 0:
        rp[-1] = g.num_edges - 1
    return Graph(rp, g.col, g.weights, g.name + "_lonestar", dict(g.meta, lonestar_view=True))


def reference_node_values(V: int) -> np.ndarray:
    """node_value[i] = i/(float)(V+1) (pannotia color.h:53, mis.h:55)."""
    return (np.arange(V, dtype=np.float32) / np.float32(V + 1)).astype(np.float32)


def seeded_node_values(V: int, seed: int) -> np.ndarray:
    """A seeded permutation p of 0..V-1 mapped to p/(float)(V+1): distinct
    priorities with the same float arithmetic as the reference rule."""
    p = np.random.default_rng(seed).permutation(V).astype(np.float32)
    return (p / np.float32(V + 1)).astype(np.float32)


# ---- Galois .gr v1 (read by lonestar/graph_apps/bfs/bfs.h:95-169) ----------

def write_gr(path: str, g: Graph) -> None:
    V, E = g.num_nodes, g.num_edges
    with open(path, "wb") as f:
        hdr = np.array([1, 4 if g.weights is not None else 0, V, E], dtype="<u8")
        f.write(hdr.tobytes())
        f.write(g.row_ptr[1:].astype("<u8").tobytes())
        f.write(g.col.astype("<u4").tobytes())
        if g.weights is not None:
            if E % 2:
                f.write(b"\0\0\0\0")
            f.write(g.weights.astype("<u4").tobytes())


def read_gr(path: str) -> Graph:
    raw = np.fromfile(path, dtype=np.uint8)
    hdr = raw[:32].view("<u8")
    version, size_edge, V, E = (int(x) for x in hdr)
    if version != 1:
        raise ValueError(f"{path}: .gr version {version} (expected 1)")
    off = 32
    out_idx = raw[off:off + 8 * V].view("<u8").astype(np.int64)
    off += 8 * V
    col = raw[off:off + 4 * E].view("<u4").astype(np.int32)
    off += 4 * E
    wt = None
    if size_edge:
        off += 4 * (E % 2)
        wt = raw[off:off + 4 * E].view("<u4").astype(np.uint32)
    rp = np.zeros(V + 1, np.int32)
    rp[1:] = out_idx
    return Graph(rp, col, wt, path)
