"""Host mirror of the reference's scheduler_rt host API and app plugins.

Python names follow the reference's host interface
(src/scheduler_rt/rt_host/cl_scheduler.h, cl_communicator.h, the app plugin
headers); every call goes straight to libwgm's C-ABI.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from ._lib import WgmConfig, WgmError, WgmGraphDesc, WgmRunStats, check, lib
from .graphs import Graph

APPS = {
    "lonestar_bfs": L.APP_LONESTAR_BFS,
    "lonestar_sssp": L.APP_LONESTAR_SSSP,
    "color": L.APP_PANNOTIA_COLOR,
    "mis": L.APP_PANNOTIA_MIS,
    "sssp": L.APP_PANNOTIA_SSSP,
    "pagerank": L.APP_PAGERANK,
    "bc": L.APP_PANNOTIA_BC,
}
_RESULT_DTYPE = {
    L.APP_LONESTAR_BFS: np.uint32, L.APP_LONESTAR_SSSP: np.uint32,
    L.APP_PANNOTIA_COLOR: np.int32, L.APP_PANNOTIA_MIS: np.int32,
    L.APP_PANNOTIA_SSSP: np.int32, L.APP_PAGERANK: np.float32,
    L.APP_PANNOTIA_BC: np.float32,
}


def default_config(**overrides) -> WgmConfig:
    cfg = WgmConfig()
    lib.wgm_config_default(C.byref(cfg))
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise AttributeError(f"wgm_config has no field {k}")
        setattr(cfg, k, v)
    return cfg


@dataclass
class RunStats:
    groups: int
    rounds: int
    device_status: int
    device_site: int
    kernel_ms: float
    host_ms: float


class Runtime:
    """One runtime = one device's discovery/barrier/scheduler state, one
    stream (mk_init_scheduler_ctx + mk_init_discovery_ctx + IW_barrier)."""

    def __init__(self, **config):
        self.cfg = default_config(**config)
        h = C.c_void_p()
        check(lib.wgm_runtime_create(C.byref(self.cfg), C.byref(h)), "wgm_runtime_create")
        self._h = h

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self) -> None:
        if self._h:
            lib.wgm_runtime_destroy(self._h)
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

    def reset(self) -> None:
        check(lib.wgm_reset(self._h), "wgm_reset")

    def sm_count(self) -> int:
        n = C.c_int()
        check(lib.wgm_sm_count(self._h, C.byref(n)))
        return n.value

    def last_failure(self) -> str:
        s, site, det = self.device_status()
        return f"device status {s} at site {site} (detail {det})" if s else "no device failure"

    def device_status(self) -> tuple[int, int, int]:
        s, site, det = C.c_int(), C.c_int(), C.c_int()
        check(lib.wgm_device_status(self._h, C.byref(s), C.byref(site), C.byref(det)))
        return s.value, site.value, det.value

    def get_occupancy_bound(self, threads_per_wg: int = 256) -> int:
        """CL_Communicator::get_occupancy_bound (cl_communicator.h:350-374)."""
        g = C.c_int()
        check(lib.wgm_get_occupancy_bound(self._h, threads_per_wg, C.byref(g)),
              "get_occupancy_bound")
        return g.value

    def hw_occupancy_bound(self, app: str | int, threads_per_wg: int = 256) -> int:
        kind = APPS[app] if isinstance(app, str) else app
        g = C.c_int()
        check(lib.wgm_hw_occupancy_bound(self._h, kind, threads_per_wg, C.byref(g)))
        return g.value

    def barrier_bench(self, iterations: int = 1000, threads_per_wg: int = 256,
                      num_wgs: int = 0, barrier_kind: int = L.BARRIER_AUTO) -> dict:
        """os_freq (test_suite/os_freq): iterations x 10 barriers."""
        ns, ms, g = C.c_double(), C.c_double(), C.c_int()
        check(lib.wgm_barrier_bench(self._h, threads_per_wg, num_wgs, iterations, barrier_kind,
                                    C.byref(ns), C.byref(ms), C.byref(g)), "barrier_bench")
        return {"ns_per_barrier": ns.value, "kernel_ms": ms.value, "groups": g.value,
                "barriers": iterations * 10}

    def barrier_bench_cluster(self, iterations: int = 1000, threads_per_wg: int = 256,
                              cluster_size: int = 8, num_clusters: int = 0) -> dict:
        """os_freq over every co-resident cluster of cluster_size CTAs, with the
        cluster barrier (hardware cluster barrier + one leader per cluster)."""
        ns, ms, g = C.c_double(), C.c_double(), C.c_int()
        check(lib.wgm_barrier_bench_cluster(self._h, threads_per_wg, cluster_size, num_clusters,
                                            iterations, C.byref(ns), C.byref(ms), C.byref(g)),
              "barrier_bench_cluster")
        return {"ns_per_barrier": ns.value, "kernel_ms": ms.value, "groups": g.value,
                "barriers": iterations * 10, "cluster_size": cluster_size}

    def synchronize(self) -> None:
        check(lib.wgm_synchronize(self._h), "wgm_synchronize")

    def set_abort(self, value: int) -> None:
        check(lib.wgm_set_abort(self._h, value))

    def timer_start(self) -> None:
        check(lib.wgm_timer_start(self._h), "wgm_timer_start")

    def timer_stop(self) -> float:
        """Milliseconds of device time since timer_start (CUDA events on the
        runtime's stream); waits for the stream."""
        ms = C.c_double()
        check(lib.wgm_timer_stop(self._h, C.byref(ms)), "wgm_timer_stop")
        return ms.value


def pinned_copy(a: np.ndarray) -> tuple[np.ndarray, int]:
    """Copy `a` into pinned host memory (wgm_host_alloc); returns the view and
    the raw pointer to release with lib.wgm_host_free."""
    ptr = lib.wgm_host_alloc(max(a.nbytes, 1))
    if not ptr:
        raise MemoryError("wgm_host_alloc failed")
    buf = (C.c_char * max(a.nbytes, 1)).from_address(ptr)
    view = np.frombuffer(buf, dtype=a.dtype, count=a.size).reshape(a.shape)
    view[...] = a
    return view, ptr


def _desc(g: Graph) -> tuple[WgmGraphDesc, tuple]:
    keep = (g.row_ptr, g.col, g.weights)
    d = WgmGraphDesc()
    d.num_nodes = g.num_nodes
    d.num_edges = g.num_edges
    d.row_ptr = g.row_ptr.ctypes.data
    d.col = g.col.ctypes.data if g.num_edges else None
    d.weights = None if g.weights is None else g.weights.ctypes.data
    return d, keep


class PersistentApp:
    """One persistent task: the app plugin interface of the reference
    (init_persistent_app_for_occupancy / reset_persistent_task /
    check_persistent_task / clean_persistent_task)."""

    def __init__(self, rt: Runtime, app: str | int, graph: Graph, source: int = 0,
                 node_values: np.ndarray | None = None, damping: float = 0.85,
                 iterations: int = 20, bc_sources: int | None = None,
                 bc_mode: int | None = None, color_mode: int | None = None,
                 bfs_mode: int | None = None):
        self.rt = rt
        self.kind = APPS[app] if isinstance(app, str) else app
        self.graph = graph
        d, _keep = _desc(graph)
        h = C.c_void_p()
        check(lib.wgm_app_create(rt.handle, self.kind, C.byref(d), C.byref(h)), "wgm_app_create")
        self._h = h
        self.V = graph.num_nodes
        if source:
            self.set_source(source)
        if node_values is not None:
            self.set_node_values(node_values)
        if self.kind == L.APP_PAGERANK:
            check(lib.wgm_app_set_pagerank(self._h, damping, iterations))
        if self.kind == L.APP_PANNOTIA_BC and bc_sources is not None:
            check(lib.wgm_app_set_bc_sources(self._h, bc_sources))
        if self.kind == L.APP_PANNOTIA_BC and bc_mode is not None:
            check(lib.wgm_app_set_bc_mode(self._h, bc_mode))
        if self.kind == L.APP_PANNOTIA_COLOR and color_mode is not None:
            check(lib.wgm_app_set_color_mode(self._h, color_mode))
        if self.kind == L.APP_LONESTAR_BFS and bfs_mode is not None:
            check(lib.wgm_app_set_bfs_mode(self._h, bfs_mode))

    @property
    def name(self) -> str:
        return lib.wgm_persistent_app_name(self.kind).decode()

    @property
    def kernel_name(self) -> str:
        return lib.wgm_persistent_kernel_name(self.kind).decode()

    def set_source(self, s: int) -> None:
        check(lib.wgm_app_set_source(self._h, s), "set_source")

    def set_node_values(self, nv: np.ndarray) -> None:
        nv = np.ascontiguousarray(nv, dtype=np.float32)
        if nv.shape != (self.V,):
            raise ValueError("node_values must have one float per vertex")
        check(lib.wgm_app_set_node_values(self._h, nv.ctypes.data), "set_node_values")

    def upload(self, g: Graph) -> None:
        d, _keep = _desc(g)
        check(lib.wgm_app_upload(self._h, C.byref(d)), "wgm_app_upload")

    def run(self, num_wgs: int = 0) -> RunStats:
        """One iteration of run_persistent (skel.cpp:316-355)."""
        st = WgmRunStats()
        check(lib.wgm_run_persistent(self.rt.handle, self._h, num_wgs, C.byref(st)),
              f"run_persistent({self.name})")
        return RunStats(st.groups, st.rounds, st.device_status, st.device_site,
                        st.kernel_ms, st.host_ms)

    def launch(self, num_wgs: int = 0, stream: int | None = None) -> None:
        check(lib.wgm_launch_persistent(self.rt.handle, self._h, num_wgs, stream),
              f"launch_persistent({self.name})")

    def result(self, out: np.ndarray | None = None) -> np.ndarray:
        dt = _RESULT_DTYPE[self.kind]
        if out is None:
            out = np.empty(self.V, dt)
        check(lib.wgm_app_read_result(self._h, out.ctypes.data, out.nbytes), "read_result")
        return out

    def rounds(self) -> int:
        r = C.c_int()
        check(lib.wgm_app_rounds(self._h, C.byref(r)))
        return r.value

    def close(self) -> None:
        if self._h:
            lib.wgm_app_destroy(self._h)
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


def solve(rt: Runtime, app: str, graph: Graph, **kw) -> tuple[np.ndarray, RunStats]:
    """Create, run once, read back, destroy."""
    with PersistentApp(rt, app, graph, **kw) as a:
        st = a.run()
        return a.result(), st


__all__ = ["Runtime", "PersistentApp", "RunStats", "WgmError", "default_config", "solve", "APPS"]
