"""Served form: a resident persistent job (colour then BFS, repeated) beside a
Poisson stream of requests in one serving megakernel (wgm_serve_* in
include/wgm.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import WgmGraphDesc, WgmServeConfig, WgmServeStats, check, lib

KINDS = {1: "bfs", 2: "reduce", 3: "matmul", 4: "reduce_i32", 5: "matmul_i32"}


class Serve:
    def __init__(self, rt, color_app=None, bfs_app=None, graphs: list | None = None,
                 vecs: np.ndarray | None = None, mats: np.ndarray | None = None,
                 arena_bytes: int = 256 << 20):
        """color_app/bfs_app: PersistentApp handles of the resident job (both
        or neither); graphs: BFS query graphs; vecs: (n, len) float32 >= 0;
        mats: (n, 2, m, m) float32 operand pairs."""
        self.rt = rt
        graphs = graphs or []
        self.graphs = graphs
        descs = (WgmGraphDesc * max(1, len(graphs)))()
        self._keep = []
        for i, g in enumerate(graphs):
            d = descs[i]
            d.num_nodes, d.num_edges = g.num_nodes, g.num_edges
            d.row_ptr = g.row_ptr.ctypes.data
            d.col = g.col.ctypes.data if g.num_edges else None
            d.weights = None
            self._keep.append(g)
        self.vecs = None if vecs is None else np.ascontiguousarray(vecs, np.float32)
        self.mats = None if mats is None else np.ascontiguousarray(mats, np.float32)
        nv, vl = (0, 1) if self.vecs is None else self.vecs.shape
        nm, mn = (0, 32) if self.mats is None else (self.mats.shape[0], self.mats.shape[-1])
        h = C.c_void_p()
        check(lib.wgm_serve_create(
            rt.handle, color_app._h if color_app else None, bfs_app._h if bfs_app else None,
            len(graphs), descs, nv, vl, None if self.vecs is None else self.vecs.ctypes.data,
            nm, mn, None if self.mats is None else self.mats.ctypes.data, arena_bytes,
            C.byref(h)), "wgm_serve_create")
        self._h = h
        self.mat_n = mn

    def set_int_data(self, ivecs: np.ndarray, imats: np.ndarray) -> None:
        """int32 reduce inputs (n, len) and operand pairs (n, 2, m, m)."""
        self.ivecs = np.ascontiguousarray(ivecs, np.int32)
        self.imats = np.ascontiguousarray(imats, np.int32)
        check(lib.wgm_serve_set_int_data(self._h, self.ivecs.shape[0], self.ivecs.shape[1],
                                         self.ivecs.ctypes.data, self.imats.shape[0],
                                         self.imats.shape[-1], self.imats.ctypes.data),
              "wgm_serve_set_int_data")
        self.imat_n = self.imats.shape[-1]

    def run(self, rate: float = 0.0, duration_s: float = 0.0, seed: int = 1,
            frac_bfs: float = 0.4, frac_reduce: float = 0.3, reps: int = 0,
            persist_groups: int = 0, reserve: int = 0, bfs_groups: int = 4,
            reduce_groups: int = 4, matmul_groups: int = 4, max_in_flight: int = 256,
            keep_results: bool = False, threads_per_wg: int = 0,
            bfs_edges_per_group: int = 0, frac_int: float = 0.0,
            persist_max_groups: int = 0) -> dict:
        c = WgmServeConfig(rate, duration_s, seed, frac_bfs, frac_reduce, reps, persist_groups,
                           reserve, bfs_groups, reduce_groups, matmul_groups, max_in_flight,
                           int(keep_results), threads_per_wg, bfs_edges_per_group, frac_int,
                           persist_max_groups)
        st = WgmServeStats()
        rc = lib.wgm_serve_run(self._h, C.byref(c), C.byref(st))
        if rc:
            buf = C.create_string_buffer(1024)
            lib.wgm_serve_diag(self._h, buf, 1024)
            check(rc, "wgm_serve_run (" + buf.value.decode() + ")")
        return {k: getattr(st, k) for k, _ in WgmServeStats._fields_}

    def groups_trace(self) -> tuple[np.ndarray, np.ndarray]:
        """(t_ns, groups): the persistent job's group count every 1 ms of the
        last run."""
        n = C.c_int64(0)
        check(lib.wgm_serve_groups_trace(self._h, None, None, 0, C.byref(n)))
        t = np.zeros(n.value, np.int64)
        g = np.zeros(n.value, np.int32)
        if n.value:
            check(lib.wgm_serve_groups_trace(self._h, t.ctypes.data, g.ctypes.data, n.value,
                                             C.byref(n)))
        return t, g

    def requests(self) -> dict:
        n = C.c_int64(0)
        check(lib.wgm_serve_requests(self._h, C.byref(n), None, None, None, None, None))
        k = np.empty(n.value, np.int32)
        a0, a1, g = np.empty_like(k), np.empty_like(k), np.empty_like(k)
        lat = np.empty(n.value, np.int64)
        check(lib.wgm_serve_requests(self._h, C.byref(n), k.ctypes.data, a0.ctypes.data,
                                     a1.ctypes.data, lat.ctypes.data, g.ctypes.data))
        ex = np.empty(n.value, np.int64)
        check(lib.wgm_serve_exec_times(self._h, n.value, ex.ctypes.data))
        return {"kind": k, "arg0": a0, "arg1": a1, "latency_ns": lat, "groups": g, "exec_ns": ex}

    def result(self, i: int, kind: int, arg0: int) -> np.ndarray:
        if kind == 1:
            out = np.empty(self.graphs[arg0].num_nodes, np.uint32)
        elif kind == 2:
            out = np.empty(1, np.float32)
        elif kind == 3:
            out = np.empty((self.mat_n, self.mat_n), np.float32)
        elif kind == 4:
            out = np.empty(1, np.int32)
        else:
            out = np.empty(1 + self.imat_n * self.imat_n, np.int32)  # hash, then C
        check(lib.wgm_serve_result(self._h, i, out.ctypes.data, out.nbytes), "wgm_serve_result")
        return out

    def close(self):
        if self._h:
            lib.wgm_serve_destroy(self._h)
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


def serve_datasets(seed: int = 7, scales=(12, 13, 14, 15, 16), graphs_per_scale: int = 2,
                   n_vecs: int = 4, vec_len: int = 1 << 20, n_mats: int = 4, mat_n: int = 256):
    """Resident request datasets: RMAT query graphs of the given scales (edge
    factor 16, symmetrised), non-negative FP32 vectors, FP32 operand pairs."""
    from . import graphs as G
    gs = [G.rmat(s, 16, seed=seed * 100 + s * 10 + k) for s in scales
          for k in range(graphs_per_scale)]
    rng = np.random.default_rng(seed)
    vecs = rng.random((n_vecs, vec_len), dtype=np.float32) * 1000.0 + 1.0
    mats = (rng.random((n_mats, 2, mat_n, mat_n), dtype=np.float32) - 0.5).astype(np.float32)
    return gs, vecs, mats
