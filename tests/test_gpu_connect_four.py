"""Connect-four look-ahead on the GPU (src/test_suite/connect_four): the
reference's own known answer on its committed board (tests/golden/
connect_four.json), the oracle on other boards and look-ahead depths, any
group count, and inside the megakernel while non-persistent tasks make
groups leave and come back mid-search.  min/max answers make the result
independent of the schedule, so it is compared exactly."""
import json
import os

import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import Runtime, WgmError
from gpu_workgroup_managment_gb300.communicator import Communicator
from gpu_workgroup_managment_gb300.connect_four import ConnectFour
from oracle import oracle

pytestmark = pytest.mark.gpu

FAST = dict(run_timeout_ns=20_000_000_000)
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "connect_four.json")


def _golden():
    with open(GOLDEN) as f:
        d = json.load(f)
    return np.array(d["board"], np.uint8), d["maxlevel"], np.array(d["next_move_value"])


def _boards():
    rng = np.random.default_rng(3)
    out = [np.zeros(42, np.uint8)]
    for k in range(3):
        b = np.zeros((6, 7), np.uint8)
        for m in range(6 + 4 * k):  # legal random plays from the bottom
            c = int(rng.integers(0, 7))
            col = b[:, c]
            empty = np.nonzero(col == 0)[0]
            if len(empty):
                col[empty[-1]] = 2 if m % 2 == 0 else 1
        out.append(b.reshape(42))
    return out


@pytest.mark.parametrize("num_wgs", [0, 1, 5])
def test_reference_board_known_answer(num_wgs):
    board, maxlevel, want = _golden()
    with Runtime(**FAST) as rt, ConnectFour(rt, board, maxlevel) as c4:
        for _ in range(2):  # every run starts afresh
            st = c4.run(num_wgs)
            assert np.array_equal(c4.result(), want)
            assert c4.tasks() == st.rounds > 7


@pytest.mark.parametrize("maxlevel", [1, 3, 5])
def test_other_boards_match_oracle(maxlevel):
    with Runtime(**FAST) as rt:
        for b in _boards():
            with ConnectFour(rt, b, maxlevel) as c4:
                c4.run()
                assert np.array_equal(c4.result(), oracle.connect_four(b, maxlevel))


def test_full_pools_are_reported():
    board, maxlevel, _ = _golden()
    with Runtime(**FAST) as rt:
        with ConnectFour(rt, board, maxlevel, pool_size=1) as c4:
            with pytest.raises(WgmError):
                c4.run(1)  # one group pushes 7 children per node: 1-node pools fill
        with ConnectFour(rt, board, maxlevel) as c4:
            c4.run()


def test_in_megakernel_with_kills_and_forks():
    board, _, _ = _golden()
    want7 = oracle.connect_four(board, 7)
    with Runtime(**FAST) as rt, ConnectFour(rt, board, 7) as c4:
        with Communicator(rt, c4, "matmult", 64) as cm:
            cm.launch_mega_kernel()
            n = cm.number_of_discovered_groups()
            cm.send_persistent_task(n)
            sent = 0
            while cm.is_executing_persistent() and sent < 40:
                cm.reset_non_persistent()
                cm.send_task_synchronous(max(1, n // 2))
                assert cm.check_non_persistent_task()
                sent += 1
            cm.get_persistent_time()
            avg = cm.average_persistent_groups()
            cm.send_quit_signal()
            cm.finish()
        assert np.array_equal(c4.result(), want7)
        assert sent > 0 and avg < n
        with Communicator(rt, c4, "reduce", 1 << 16) as cm:
            r = cm.run_merged_iteration(np_groups=8, frequency_ms=0)
            assert r["np_errors"] == 0
        assert np.array_equal(c4.result(), want7)
