"""Python access to the CPU oracle (liboracle.so) and to the reference's own
kernels compiled under the one-work-group shim (oracle/_ref/libref_*.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arms, always as the checker or the timed
CPU baseline, never on the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


SOURCES = ("wgm_oracle.c", "oracle_inputs.c")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    newest = max(os.path.getmtime(s) for s in srcs + [os.path.join(HERE, "wgm_oracle.h")])
    if force or not os.path.exists(LIB) or newest > os.path.getmtime(LIB):
        tmp = LIB + ".tmp"
        subprocess.run(["gcc", "-O2", "-fPIC", "-fopenmp", "-shared", "-o", tmp, *srcs],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        P, I = C.c_void_p, C.c_int32
        protos = {
            "oracle_lonestar_bfs": [I, P, P, I, P],
            "oracle_lonestar_sssp": [I, P, P, P, I, P],
            "oracle_pannotia_color": [I, P, P, P, P],
            "oracle_pannotia_mis": [I, P, P, P, P],
            "oracle_pannotia_mis_work": [I, P, P, P, P, P],
            "oracle_pannotia_sssp": [I, P, P, P, I, P],
            "oracle_lonestar_bfs_omp": [I, P, P, I, P, P],
            "oracle_lonestar_sssp_omp": [I, P, P, P, I, P, P],
            "oracle_pannotia_color_omp": [I, P, P, P, P, P],
            "oracle_pannotia_mis_omp": [I, P, P, P, P, P, P],
            "oracle_omp_threads": [],
            "oracle_matmult_rand_fill": [P, I, I, I],
            "oracle_matmult_i32": [P, I, I, P, I, P],
            "oracle_hash_diag": [P, I, I],
            "oracle_matmult_f32": [P, I, I, P, I, P],
            "oracle_batch_lonestar": [I, P, P, P, P, P, P, P, P, P, P],
            "oracle_connect_four": [P, I, P],
            "oracle_pannotia_bc_f64": [I, P, P, I, P],
        }
        for name, args in protos.items():
            fn = getattr(_lib, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _lib.oracle_hash_diag.restype = C.c_int32
        _lib.oracle_matmult_rand_fill.restype = C.c_int32
        _lib.oracle_reduce_min_i32.restype = C.c_int32
        _lib.oracle_reduce_min_f32.restype = C.c_float
        _lib.oracle_pagerank_f64.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_double,
                                             C.c_int, C.c_void_p]
        _lib.oracle_pagerank_f32_omp.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_float,
                                                 C.c_int, C.c_void_p, C.c_void_p]
        _lib.oracle_reduce_min_i32.argtypes = [C.c_void_p, C.c_int64]
        _lib.oracle_grid_edges.argtypes = [I, I]
        _lib.oracle_grid_edges.restype = C.c_int64
        _lib.oracle_gen_grid.argtypes = [I, I, P, P]
        _lib.oracle_gen_grid.restype = C.c_int
        _lib.oracle_gen_rmat.argtypes = [I, I, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                         I, C.c_uint32, C.c_uint32, P, P, P, P]
        _lib.oracle_gen_rmat.restype = C.c_int
        _lib.oracle_free.argtypes = [P]
        _lib.oracle_free.restype = None
        _lib.oracle_reduce_min_f32.argtypes = [C.c_void_p, C.c_int64]
    return _lib


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def threads() -> int:
    return lib().oracle_omp_threads()


class BatchArena:
    """Graphs and jobs of a batch packed for oracle_batch_lonestar."""

    def __init__(self, graphs: list, jobs: list):
        rows, cols, wts, roff, coff = [], [], [], [], []
        r = c = 0
        for g in graphs:
            roff.append(r)
            coff.append(c)
            rows.append(g.row_ptr)
            cols.append(g.col)
            wts.append(g.weights if g.weights is not None else np.zeros(g.num_edges, np.uint32))
            r += g.num_nodes + 1
            c += g.num_edges
        self.rows = np.concatenate(rows).astype(np.int32)
        self.cols = np.concatenate(cols).astype(np.int32) if c else np.zeros(1, np.int32)
        self.wts = np.concatenate(wts).astype(np.uint32) if c else np.zeros(1, np.uint32)
        self.graph_roff = np.array(roff, np.int64)
        self.graph_coff = np.array(coff, np.int64)
        self.graphs = graphs
        self.set_jobs(jobs)

    def set_jobs(self, jobs: list) -> None:
        gi = np.array([j[0] for j in jobs], np.int64)
        self.V = np.array([self.graphs[i].num_nodes for i in gi], np.int32)
        self.row_off = self.graph_roff[gi]
        self.col_off = self.graph_coff[gi]
        self.dist_off = np.concatenate([[0], np.cumsum(self.V.astype(np.int64))[:-1]])
        self.algo = np.array([0 if j[1] == "bfs" else 1 for j in jobs], np.int32)
        self.source = np.array([j[2] for j in jobs], np.int32)
        self.dist = np.empty(int(self.V.astype(np.int64).sum()), np.uint32)

    def run(self) -> np.ndarray:
        lib().oracle_batch_lonestar(len(self.V), _p(self.V), _p(self.row_off), _p(self.col_off),
                                    _p(self.dist_off), _p(self.algo), _p(self.source),
                                    _p(self.rows), _p(self.cols), _p(self.wts), _p(self.dist))
        return self.dist


def pannotia_bc_f64(g, num_sources: int | None = None) -> np.ndarray:
    """Betweenness centrality of pannotia bc.cl in float64, sources
    0 .. num_sources-1 (all by default)."""
    V = g.num_nodes
    out = np.empty(V, np.float64)
    n = V if num_sources is None else num_sources
    if lib().oracle_pannotia_bc_f64(V, _p(g.row_ptr), _p(g.col), n, _p(out)) != 0:
        raise MemoryError("oracle_pannotia_bc_f64")
    return out


def connect_four(board: np.ndarray, maxlevel: int = 6) -> np.ndarray:
    """next_move_value[7] of the reference's connect-four look-ahead
    (test_suite/connect_four/device/connect_four.cl) from a 42-cell board."""
    b = np.ascontiguousarray(board, dtype=np.uint8).reshape(42)
    out = np.empty(7, np.int32)
    if lib().oracle_connect_four(_p(b), maxlevel, _p(out)) != 0:
        raise ValueError("maxlevel must be 1..7")
    return out


def lonestar_bfs(g, source: int = 0, omp: bool = False) -> np.ndarray:
    V = g.num_nodes
    d = np.empty(V, np.uint32)
    if omp:
        scratch = np.empty(2 * V, np.int32)
        lib().oracle_lonestar_bfs_omp(V, _p(g.row_ptr), _p(g.col), source, _p(d), _p(scratch))
    else:
        lib().oracle_lonestar_bfs(V, _p(g.row_ptr), _p(g.col), source, _p(d))
    return d


def lonestar_sssp(g, source: int = 0, omp: bool = False) -> np.ndarray:
    V = g.num_nodes
    d = np.empty(V, np.uint32)
    if omp:
        scratch = np.empty(3 * V, np.int32)
        lib().oracle_lonestar_sssp_omp(V, _p(g.row_ptr), _p(g.col), _p(g.weights), source, _p(d),
                                       _p(scratch))
    else:
        lib().oracle_lonestar_sssp(V, _p(g.row_ptr), _p(g.col), _p(g.weights), source, _p(d))
    return d


def color(g, node_value: np.ndarray, omp: bool = False) -> np.ndarray:
    V = g.num_nodes
    out = np.empty(V, np.int32)
    nv = np.ascontiguousarray(node_value, np.float32)
    if omp:
        md = np.empty(V, np.float32)
        lib().oracle_pannotia_color_omp(V, _p(g.row_ptr), _p(g.col), _p(nv), _p(out), _p(md))
    else:
        lib().oracle_pannotia_color(V, _p(g.row_ptr), _p(g.col), _p(nv), _p(out))
    return out


def mis(g, node_value: np.ndarray, omp: bool = False) -> np.ndarray:
    V = g.num_nodes
    out = np.empty(V, np.int32)
    nv = np.ascontiguousarray(node_value, np.float32)
    if omp:
        scratch = np.empty(2 * V, np.int32)
        mn = np.empty(V, np.float32)
        lib().oracle_pannotia_mis_omp(V, _p(g.row_ptr), _p(g.col), _p(nv), _p(out), _p(scratch),
                                      _p(mn))
    else:
        lib().oracle_pannotia_mis(V, _p(g.row_ptr), _p(g.col), _p(nv), _p(out))
    return out


def mis_work(g, node_value: np.ndarray) -> tuple[np.ndarray, int, int]:
    """MIS membership plus its work: edges scanned by the minimum phase and
    active vertices, each summed over rounds."""
    V = g.num_nodes
    out = np.empty(V, np.int32)
    work = np.zeros(2, np.int64)
    nv = np.ascontiguousarray(node_value, np.float32)
    lib().oracle_pannotia_mis_work(V, _p(g.row_ptr), _p(g.col), _p(nv), _p(out), _p(work))
    return out, int(work[0]), int(work[1])


def pannotia_sssp(g, source: int = 0) -> np.ndarray:
    V = g.num_nodes
    out = np.empty(V, np.int32)
    data = np.ascontiguousarray(g.weights.view(np.int32))
    lib().oracle_pannotia_sssp(V, _p(g.row_ptr), _p(g.col), _p(data), source, _p(out))
    return out


def pagerank_f64(g, damping: float = 0.85, iterations: int = 20) -> np.ndarray:
    pr = np.empty(g.num_nodes, np.float64)
    lib().oracle_pagerank_f64(g.num_nodes, _p(g.row_ptr), _p(g.col), damping, iterations, _p(pr))
    return pr


def pagerank_f32_omp(g, damping: float = 0.85, iterations: int = 20) -> np.ndarray:
    V = g.num_nodes
    pr = np.empty(V, np.float32)
    scratch = np.empty(2 * V, np.float32)
    lib().oracle_pagerank_f32_omp(V, _p(g.row_ptr), _p(g.col), damping, iterations, _p(pr),
                                  _p(scratch))
    return pr


def matmult_inputs(n: int, seed: int = 1234) -> tuple[np.ndarray, np.ndarray]:
    """matmult.h:163-203: A then B filled by the middle-square generator."""
    A = np.empty((n, n), np.int32)
    B = np.empty((n, n), np.int32)
    s = lib().oracle_matmult_rand_fill(_p(A), n, n, seed)
    lib().oracle_matmult_rand_fill(_p(B), n, n, s)
    return A, B


def matmult_i32(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    Cm = np.empty((A.shape[0], B.shape[1]), np.int32)
    lib().oracle_matmult_i32(_p(A), A.shape[0], A.shape[1], _p(B), B.shape[1], _p(Cm))
    return Cm


def hash_diag(M: np.ndarray) -> int:
    return int(lib().oracle_hash_diag(_p(np.ascontiguousarray(M, np.int32)), M.shape[0],
                                      M.shape[1]))


def reduce_min_i32(buf: np.ndarray) -> int:
    return int(lib().oracle_reduce_min_i32(_p(buf), buf.shape[0]))


# ---- the reference's own kernels under the shim (built by build_ref.py) ----

def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libref_lonestar_bfs.so"))


_REF_PROTOS = {
    "ref_run_lonestar": [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int],
    "ref_run_color": [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int],
    "ref_run_mis": [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int],
    "ref_run_pannotia_sssp": [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int],
    "ref_run_matmult": [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                        C.c_int],
    "ref_run_reduce": [C.c_void_p, C.c_int, C.c_int],
}
_ref_libs: dict = {}


def _ref(name: str) -> C.CDLL:
    if name not in _ref_libs:
        lib_ = C.CDLL(os.path.join(REF_DIR, f"libref_{name}.so"))
        for fn, args in _REF_PROTOS.items():
            if hasattr(lib_, fn):
                getattr(lib_, fn).argtypes = args
                getattr(lib_, fn).restype = C.c_int
        _ref_libs[name] = lib_
    return _ref_libs[name]


def ref_lonestar_bfs(g, wgs: int = 128) -> np.ndarray:
    d = np.empty(g.num_nodes, np.uint32)
    _ref("lonestar_bfs").ref_run_lonestar(g.num_nodes, _p(g.row_ptr), _p(g.col), None, _p(d), wgs)
    return d


def ref_lonestar_sssp(g, wgs: int = 128) -> np.ndarray:
    d = np.empty(g.num_nodes, np.uint32)
    _ref("lonestar_sssp").ref_run_lonestar(g.num_nodes, _p(g.row_ptr), _p(g.col), _p(g.weights),
                                           _p(d), wgs)
    return d


def ref_color(g, node_value: np.ndarray, wgs: int = 128) -> np.ndarray:
    out = np.empty(g.num_nodes, np.int32)
    nv = np.ascontiguousarray(node_value, np.float32)
    _ref("pannotia_color").ref_run_color(g.num_nodes, _p(g.row_ptr), _p(g.col), _p(nv), _p(out),
                                         wgs)
    return out


def ref_mis(g, node_value: np.ndarray, wgs: int = 128) -> np.ndarray:
    out = np.empty(g.num_nodes, np.int32)
    nv = np.ascontiguousarray(node_value, np.float32)
    _ref("pannotia_mis").ref_run_mis(g.num_nodes, _p(g.row_ptr), _p(g.col), _p(nv), _p(out), wgs)
    return out


def ref_pannotia_sssp(g, wgs: int = 128) -> np.ndarray:
    out = np.empty(g.num_nodes, np.int32)
    data = np.ascontiguousarray(g.weights.view(np.int32))
    _ref("pannotia_sssp").ref_run_pannotia_sssp(g.num_nodes, _p(g.row_ptr), _p(g.col), _p(data),
                                                _p(out), wgs)
    return out


def ref_matmult(A: np.ndarray, B: np.ndarray, wgs: int = 128) -> tuple[np.ndarray, int]:
    Cm = np.empty((A.shape[0], B.shape[1]), np.int32)
    h = _ref("matmult").ref_run_matmult(_p(A), A.shape[0], A.shape[1], _p(B), B.shape[0],
                                        B.shape[1], _p(Cm), wgs)
    return Cm, int(h)


def ref_reduce(buf: np.ndarray, wgs: int = 256) -> int:
    return int(_ref("reduce").ref_run_reduce(_p(buf), buf.shape[0], wgs))
