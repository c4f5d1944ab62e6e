"""Connect-four look-ahead as a persistent app: the reference's second
work-stealing stress test of offer_kill / offer_fork
(src/test_suite/connect_four: device kernel connect_four.cl, host plugin
connect_four.h) over libwgm's C-ABI.  Runs standalone (`run`) or as the
megakernel's persistent app through a `Communicator`."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import WgmRunStats, check, lib
from .runtime import RunStats

EMPTY, HUMAN, COMPUTER = 0, 1, 2
PLUS_INF, MINUS_INF = 666, -666


def parse_board(text: str) -> np.ndarray:
    """A board as connect_four.h:89-104 reads it: '.' empty, 'o' human,
    'x' computer, other characters skipped; 42 cells, top row first."""
    cells = [".ox".index(ch) for ch in text if ch in ".ox"][:42]
    if len(cells) < 42:
        raise ValueError("not enough valid characters in the board")
    return np.array(cells, np.uint8)


class ConnectFour:
    """maxlevel = FLAGS_maxlevel (6), pool_size = FLAGS_pool_size (10000)."""

    def __init__(self, rt, board: np.ndarray, maxlevel: int = 6, pool_size: int = 10000):
        self.rt = rt
        b = np.ascontiguousarray(board, dtype=np.uint8).reshape(42)
        h = C.c_void_p()
        check(lib.wgm_c4_create(rt.handle, b.ctypes.data, maxlevel, pool_size, C.byref(h)),
              "wgm_c4_create")
        self._h = h
        self.maxlevel = maxlevel

    def run(self, num_wgs: int = 0) -> RunStats:
        st = WgmRunStats()
        check(lib.wgm_run_persistent(self.rt.handle, self._h, num_wgs, C.byref(st)),
              "run_persistent(connect_four)")
        return RunStats(st.groups, st.rounds, st.device_status, st.device_site,
                        st.kernel_ms, st.host_ms)

    def result(self) -> np.ndarray:
        """next_move_value[7]: the value of each first move."""
        out = np.empty(7, np.int32)
        check(lib.wgm_app_read_result(self._h, out.ctypes.data, out.nbytes), "read_result")
        return out

    def tasks(self) -> int:
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
