"""ctypes binding of libwgm.so (the C-ABI declared in include/wgm.h).

The product path has no CPU fallback: if the extension has not been built,
importing this module raises, naming the build step.
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libwgm.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "wgm.h")

WGM_OK = 0
STATUS = {
    0: "WGM_OK", -1: "WGM_ERR_INVALID", -2: "WGM_ERR_TOO_MANY_GROUPS", -3: "WGM_ERR_TIMEOUT",
    -4: "WGM_ERR_OOM", -5: "WGM_ERR_CUDA", -6: "WGM_ERR_OVERFLOW", -7: "WGM_ERR_NO_DEVICE",
    -8: "WGM_ERR_ABORTED", -9: "WGM_ERR_STATE",
}
STATUS_CODE = {v: k for k, v in STATUS.items()}

APP_LONESTAR_BFS, APP_LONESTAR_SSSP, APP_PANNOTIA_COLOR = 1, 2, 3
APP_PANNOTIA_MIS, APP_PANNOTIA_SSSP, APP_PAGERANK = 4, 5, 6
APP_OCTREE = 7
APP_CONNECT_FOUR = 8
APP_PANNOTIA_BC = 9
DISCOVERY_TICKET, DISCOVERY_REFERENCE = 0, 1
BARRIER_SENSE, BARRIER_XF, BARRIER_TREE, BARRIER_COUNT, BARRIER_SPREAD, BARRIER_AUTO = 0, 1, 2, 3, 4, 5
NP_NONE, NP_MATMULT_I32, NP_REDUCE_I32, NP_MATMULT_F32, NP_REDUCE_F32 = 0, 1, 2, 3, 4


class WgmConfig(C.Structure):
    _fields_ = [
        ("device", C.c_int), ("threads_per_wg", C.c_int), ("num_wgs", C.c_int),
        ("use_query_barrier", C.c_int), ("non_persistent_wgs", C.c_int),
        ("non_persistent_frequency_ms", C.c_int), ("skip_tasks", C.c_int),
        ("host_handshake", C.c_int), ("discovery_mode", C.c_int),
        ("discovery_extra_rounds", C.c_int), ("barrier_kind", C.c_int),
        ("tree_fanin", C.c_int), ("hub_threshold", C.c_int),
        ("spin_timeout_ns", C.c_uint64), ("run_timeout_ns", C.c_uint64),
        ("discovery_window_ns", C.c_uint64),
    ]


class WgmRunStats(C.Structure):
    _fields_ = [("groups", C.c_int), ("rounds", C.c_int), ("device_status", C.c_int),
                ("device_site", C.c_int), ("kernel_ms", C.c_double), ("host_ms", C.c_double)]


class WgmServeConfig(C.Structure):
    _fields_ = [("rate_per_s", C.c_double), ("duration_s", C.c_double), ("seed", C.c_uint64),
                ("frac_bfs", C.c_double), ("frac_reduce", C.c_double), ("reps", C.c_int),
                ("persist_groups", C.c_int), ("reserve", C.c_int), ("bfs_groups", C.c_int),
                ("reduce_groups", C.c_int), ("matmul_groups", C.c_int),
                ("max_in_flight", C.c_int), ("keep_results", C.c_int),
                ("threads_per_wg", C.c_int), ("bfs_edges_per_group", C.c_int64),
                ("frac_int", C.c_double), ("persist_max_groups", C.c_int)]


class WgmServeStats(C.Structure):
    _fields_ = [("arrived", C.c_int64), ("completed", C.c_int64),
                ("waited_for_memory", C.c_int64), ("stream_s", C.c_double),
                ("achieved_rate", C.c_double), ("lat_p50_us", C.c_double),
                ("lat_p99_us", C.c_double), ("lat_mean_us", C.c_double),
                ("lat_max_us", C.c_double), ("persist_ms", C.c_double),
                ("persist_reps", C.c_int), ("kills", C.c_int), ("forks", C.c_int),
                ("groups", C.c_int), ("run_ms", C.c_double), ("exec_p50_us", C.c_double),
                ("exec_p99_us", C.c_double), ("wait_p50_us", C.c_double),
                ("wait_p99_us", C.c_double), ("persist_groups_mean", C.c_double),
                ("persist_groups_min", C.c_int)]


class WgmGraphDesc(C.Structure):
    _fields_ = [("num_nodes", C.c_int32), ("num_edges", C.c_int64),
                ("row_ptr", C.c_void_p), ("col", C.c_void_p), ("weights", C.c_void_p)]


class WgmAppVtable(C.Structure):
    """wgm_app_vtable (include/wgm.h): a registered app's table; the entry
    points are filled by the app's own library, so they stay plain
    pointers here."""
    _fields_ = [("version", C.c_int), ("user", C.c_void_p), ("app_name", C.c_char_p),
                ("kernel_name", C.c_char_p), ("init", C.c_void_p), ("reset", C.c_void_p),
                ("check", C.c_void_p), ("read_result", C.c_void_p), ("rounds", C.c_void_p),
                ("clean", C.c_void_p), ("occupancy", C.c_void_p), ("launch", C.c_void_p),
                ("launch_mega", C.c_void_p)]


APP_PLUGIN = 100
APP_VTABLE_VERSION = 1

_P = C.c_void_p
_I = C.c_int
_PROTOS = {
    "wgm_app_register": (_I, [_P, C.POINTER(WgmAppVtable), C.POINTER(_P)]),
    "wgm_batch_configure_sssp_dense": (_I, [_P, C.c_double]),
    "wgm_batch_sssp_dense_info": (_I, [_P, C.POINTER(C.c_double)]),
    "wgm_barrier_bench_cluster": (_I, [_P, _I, _I, _I, _I, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.POINTER(_I)]),
    "wgm_serve_groups_trace": (_I, [_P, _P, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "wgm_app_set_color_mode": (_I, [_P, C.c_int32]),
    "wgm_app_set_bfs_mode": (_I, [_P, C.c_int32]),
    "wgm_profiler_start": (_I, [_P]),
    "wgm_profiler_stop": (_I, [_P]),
    "wgm_app_check": (_I, [_P, C.POINTER(_I)]),
    "wgm_config_default": (None, [C.POINTER(WgmConfig)]),
    "wgm_status_string": (C.c_char_p, [_I]),
    "wgm_runtime_create": (_I, [C.POINTER(WgmConfig), C.POINTER(_P)]),
    "wgm_runtime_destroy": (_I, [_P]),
    "wgm_reset": (_I, [_P]),
    "wgm_last_cuda_error": (_I, [_P]),
    "wgm_device_status": (_I, [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)]),
    "wgm_set_abort": (_I, [_P, _I]),
    "wgm_sm_count": (_I, [_P, C.POINTER(_I)]),
    "wgm_get_occupancy_bound": (_I, [_P, _I, C.POINTER(_I)]),
    "wgm_hw_occupancy_bound": (_I, [_P, _I, _I, C.POINTER(_I)]),
    "wgm_barrier_bench": (_I, [_P, _I, _I, _I, _I, C.POINTER(C.c_double),
                               C.POINTER(C.c_double), C.POINTER(_I)]),
    "wgm_persistent_app_name": (C.c_char_p, [_I]),
    "wgm_persistent_kernel_name": (C.c_char_p, [_I]),
    "wgm_app_create": (_I, [_P, _I, C.POINTER(WgmGraphDesc), C.POINTER(_P)]),
    "wgm_octree_create": (_I, [_P, C.c_int32, _P, C.c_int32, C.c_int32, C.c_int64, C.POINTER(_P)]),
    "wgm_octree_read": (_I, [_P, _P, C.c_int64, _P, _P, _P]),
    "wgm_octree_check": (_I, [_P, _P]),
    "wgm_c4_create": (_I, [_P, _P, C.c_int32, C.c_int32, C.POINTER(_P)]),
    "wgm_app_set_bc_sources": (_I, [_P, C.c_int32]),
    "wgm_app_set_bc_mode": (_I, [_P, C.c_int32]),
    "wgm_app_upload": (_I, [_P, C.POINTER(WgmGraphDesc)]),
    "wgm_app_set_source": (_I, [_P, C.c_int32]),
    "wgm_app_set_node_values": (_I, [_P, _P]),
    "wgm_app_set_pagerank": (_I, [_P, C.c_float, _I]),
    "wgm_run_persistent": (_I, [_P, _P, _I, C.POINTER(WgmRunStats)]),
    "wgm_launch_persistent": (_I, [_P, _P, _I, _P]),
    "wgm_synchronize": (_I, [_P]),
    "wgm_app_read_result": (_I, [_P, _P, C.c_size_t]),
    "wgm_app_result_device_ptr": (_I, [_P, C.POINTER(_P), C.POINTER(C.c_size_t)]),
    "wgm_app_rounds": (_I, [_P, C.POINTER(_I)]),
    "wgm_app_destroy": (_I, [_P]),
    "wgm_comm_create": (_I, [_P, _P, _I, _I, C.POINTER(_P)]),
    "wgm_comm_destroy": (_I, [_P]),
    "wgm_comm_launch_mega_kernel": (_I, [_P, _I]),
    "wgm_comm_number_of_discovered_groups": (_I, [_P, C.POINTER(_I)]),
    "wgm_comm_send_persistent_task": (_I, [_P, _I]),
    "wgm_comm_send_task_synchronous": (_I, [_P, _I, C.POINTER(C.c_uint64),
                                            C.POINTER(C.c_uint64)]),
    "wgm_comm_is_executing_persistent": (_I, [_P, C.POINTER(_I)]),
    "wgm_comm_get_persistent_time": (_I, [_P, C.POINTER(C.c_uint64)]),
    "wgm_comm_send_quit": (_I, [_P]),
    "wgm_comm_finish": (_I, [_P]),
    "wgm_comm_reset": (_I, [_P]),
    "wgm_comm_add_redline": (_I, [_P]),
    "wgm_comm_summary": (_I, [_P, C.c_char_p, C.c_size_t]),
    "wgm_comm_task_times": (_I, [_P, _P, _P, _I, C.POINTER(_I)]),
    "wgm_comm_average_persistent_groups": (_I, [_P, C.POINTER(C.c_double)]),
    "wgm_comm_reset_non_persistent": (_I, [_P]),
    "wgm_comm_check_non_persistent": (_I, [_P, C.POINTER(_I)]),
    "wgm_comm_get_occupancy_bound": (_I, [_P, C.POINTER(_I)]),
    "wgm_run_merged_iteration": (_I, [_P, _I, _I, _I, _I, C.POINTER(_I), C.POINTER(_I)]),
    "wgm_batch_create": (_I, [_P, _I, _P, _I, _P, _P, _P, C.POINTER(_P)]),
    "wgm_batch_upload": (_I, [_P, _P]),
    "wgm_batch_configure": (_I, [_P, _I, _I, _I]),
    "wgm_batch_configure_teams": (_I, [_P, C.c_int64, _I]),
    "wgm_batch_team_info": (_I, [_P, _P, _P]),
    "wgm_batch_configure_local": (_I, [_P, _I]),
    "wgm_batch_configure_sssp": (_I, [_P, C.c_double, _I]),
    "wgm_batch_sssp_info": (_I, [_P, _P, _P]),
    "wgm_batch_configure_kernel": (_I, [_P, _I]),
    "wgm_batch_kernel_info": (_I, [_P, _P]),
    "wgm_batch_submit_packed": (_I, [_P, _P, _P, _P, _P]),
    "wgm_batch_wait": (_I, [_P]),
    "wgm_batch_upload_packed": (_I, [_P, _P, _P, _P]),
    "wgm_batch_graph_offsets": (_I, [_P, _P, _P]),
    "wgm_batch_job_stats": (_I, [_P, _P, _P, _P, _P]),
    "wgm_batch_job_work": (_I, [_P, _P]),
    "wgm_batch_configure_bfs_one_cta": (_I, [_P, C.c_double]),
    "wgm_batch_reorder_by_last_run": (_I, [_P]),
    "wgm_serve_create": (_I, [_P, _P, _P, _I, _P, _I, _I, _P, _I, _I, _P, C.c_int64, _P]),
    "wgm_serve_run": (_I, [_P, _P, _P]),
    "wgm_serve_requests": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "wgm_serve_result": (_I, [_P, C.c_int64, _P, C.c_int64]),
    "wgm_serve_destroy": (_I, [_P]),
    "wgm_serve_set_int_data": (_I, [_P, _I, _I, _P, _I, _I, _P]),
    "wgm_serve_exec_times": (_I, [_P, C.c_int64, _P]),
    "wgm_serve_diag": (_I, [_P, C.c_char_p, C.c_size_t]),
    "wgm_batch_launch": (_I, [_P, _I]),
    "wgm_batch_run": (_I, [_P, _I, C.POINTER(C.c_double)]),
    "wgm_batch_launch_per_graph": (_I, [_P]),
    "wgm_batch_run_per_graph": (_I, [_P, C.POINTER(C.c_double)]),
    "wgm_batch_launch_per_graph_sized": (_I, [_P, _I]),
    "wgm_batch_run_per_graph_sized": (_I, [_P, _I, C.POINTER(C.c_double)]),
    "wgm_batch_read": (_I, [_P, _I, _P, C.c_int64]),
    "wgm_batch_read_all": (_I, [_P, _P, C.c_int64]),
    "wgm_batch_info": (_I, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(_I),
                            C.POINTER(_I), C.POINTER(_I)]),
    "wgm_batch_autotune": (_I, [_P, _I, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I),
                                C.POINTER(C.c_double)]),
    "wgm_batch_destroy": (_I, [_P]),
    "wgm_timer_start": (_I, [_P]),
    "wgm_timer_stop": (_I, [_P, C.POINTER(C.c_double)]),
    "wgm_bfs_noalloc": (_I, [_P, _P, C.c_int32, C.c_int64, C.c_int32, _P, _P]),
    "wgm_host_alloc": (_P, [C.c_size_t]),
    "wgm_host_free": (None, [_P]),
    "wgm_gen_grid": (_I, [C.c_int32, C.c_int32, _P, _P, C.POINTER(C.c_int64)]),
    "wgm_gen_rmat": (_I, [_I, _I, C.c_double, C.c_double, C.c_double, C.c_uint64, _I,
                          C.c_uint32, C.c_uint32, C.POINTER(_P)]),
    "wgm_host_graph_info": (_I, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
    "wgm_host_graph_arrays": (_I, [_P, C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]),
    "wgm_host_graph_free": (None, [_P]),
}


def header_functions() -> list[str]:
    """Names of every function include/wgm.h declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wgm_[a-z0-9_]+)\s*\(", text)))


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


class WgmError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        self.name = STATUS.get(status, str(status))
        msg = lib.wgm_status_string(status).decode()
        super().__init__(f"{what}: {self.name} ({msg})" if what else f"{self.name} ({msg})")


def check(status: int, what: str = "") -> None:
    if status != WGM_OK:
        raise WgmError(status, what)
