"""Host side of the megakernel: the reference's CL_Communicator
(src/scheduler_rt/rt_host/cl_communicator.h) over libwgm's C-ABI."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import check, lib

NP_TASKS = {
    "none": L.NP_NONE, "matmult": L.NP_MATMULT_I32, "reduce": L.NP_REDUCE_I32,
    "matmult_f32": L.NP_MATMULT_F32, "reduce_f32": L.NP_REDUCE_F32,
}


class Communicator:
    """One megakernel host: a resident persistent app (optional) plus one
    non-persistent task kind (matmult: n x n; reduce: n elements)."""

    def __init__(self, rt, persistent=None, np_task: str = "matmult", np_size: int = 256):
        self.rt = rt
        self.persistent = persistent
        h = C.c_void_p()
        papp = persistent._h if persistent is not None else None
        check(lib.wgm_comm_create(rt.handle, papp, NP_TASKS[np_task], np_size, C.byref(h)),
              "wgm_comm_create")
        self._h = h

    def close(self):
        if self._h:
            lib.wgm_comm_destroy(self._h)
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

    def launch_mega_kernel(self, num_wgs: int = 0) -> None:
        check(lib.wgm_comm_launch_mega_kernel(self._h, num_wgs), "launch_mega_kernel")

    def number_of_discovered_groups(self) -> int:
        g = C.c_int()
        check(lib.wgm_comm_number_of_discovered_groups(self._h, C.byref(g)))
        return g.value

    def send_persistent_task(self, groups: int) -> None:
        check(lib.wgm_comm_send_persistent_task(self._h, groups), "send_persistent_task")

    def send_task_synchronous(self, groups: int) -> tuple[int, int]:
        """Returns (execution_ns, response_ns) like the reference's time_ret."""
        e, r = C.c_uint64(), C.c_uint64()
        check(lib.wgm_comm_send_task_synchronous(self._h, groups, C.byref(e), C.byref(r)),
              "send_task_synchronous")
        return e.value, r.value

    def is_executing_persistent(self) -> bool:
        x = C.c_int()
        check(lib.wgm_comm_is_executing_persistent(self._h, C.byref(x)))
        return bool(x.value)

    def get_persistent_time(self) -> int:
        ns = C.c_uint64()
        check(lib.wgm_comm_get_persistent_time(self._h, C.byref(ns)), "get_persistent_time")
        return ns.value

    def send_quit_signal(self) -> None:
        check(lib.wgm_comm_send_quit(self._h))

    def finish(self) -> None:
        check(lib.wgm_comm_finish(self._h), "finish")

    def reset_communicator(self) -> None:
        check(lib.wgm_comm_reset(self._h), "reset_communicator")

    def add_redline(self) -> None:
        check(lib.wgm_comm_add_redline(self._h))

    def summary_str(self) -> str:
        buf = C.create_string_buffer(8192)
        check(lib.wgm_comm_summary(self._h, buf, len(buf)))
        return buf.value.decode()

    def task_times(self) -> tuple[np.ndarray, np.ndarray]:
        n = C.c_int()
        check(lib.wgm_comm_task_times(self._h, None, None, 0, C.byref(n)))
        r = np.zeros(max(n.value, 1), np.uint64)
        e = np.zeros(max(n.value, 1), np.uint64)
        check(lib.wgm_comm_task_times(self._h, r.ctypes.data, e.ctypes.data, n.value,
                                      C.byref(n)))
        return r[: n.value], e[: n.value]

    def average_persistent_groups(self) -> float:
        a = C.c_double()
        check(lib.wgm_comm_average_persistent_groups(self._h, C.byref(a)))
        return a.value

    def reset_non_persistent(self) -> None:
        check(lib.wgm_comm_reset_non_persistent(self._h))

    def check_non_persistent_task(self) -> bool:
        ok = C.c_int()
        check(lib.wgm_comm_check_non_persistent(self._h, C.byref(ok)))
        return bool(ok.value)

    def get_occupancy_bound(self) -> int:
        g = C.c_int()
        check(lib.wgm_comm_get_occupancy_bound(self._h, C.byref(g)), "get_occupancy_bound")
        return g.value

    def run_merged_iteration(self, num_wgs: int = 0, np_groups: int = 1,
                             frequency_ms: int = 2, skip_tasks: bool = False) -> dict:
        """execute_merged_iteration (skel.cpp:405-463)."""
        err, tasks = C.c_int(), C.c_int()
        check(lib.wgm_run_merged_iteration(self._h, num_wgs, np_groups, frequency_ms,
                                           int(skip_tasks), C.byref(err), C.byref(tasks)),
              "run_merged_iteration")
        return {"np_errors": err.value, "np_tasks": tasks.value}
