"""The offer_kill / groups_to_kill protocol in a CPU-thread model: host
threads run the same protocol code as the kernels (csrc/wgm_protocol.h).

The reference's kill side reads groups_to_kill and stores the value minus
one (src/scheduler_rt/rt_device/scheduler_1.cl:67-71).  With a scheduler that
may clear the word at any time, a clear landing between the two steps is
overwritten by the stale value minus one, and groups nobody asked for leave.
The runtime decrements with a compare-and-swap instead; these tests force
that interleaving, and stress it with threads, against both forms (the racy
one is planted in the test harness only)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def model(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("model") / "libkill_model.so")
    subprocess.run(["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread", "-o", out,
                    os.path.join(HERE, "model", "kill_model.cpp")], check=True)
    lib = C.CDLL(out)
    lib.model_kill_clear_interleaving.argtypes = [C.c_int, C.c_void_p]
    lib.model_kill_stress.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_void_p]
    return lib


def test_clear_between_read_and_decrement_is_not_overwritten(model):
    out = np.zeros(3, np.int32)
    model.model_kill_clear_interleaving(0, out.ctypes.data)
    killed, to_kill, groups = out
    assert killed == 0 and to_kill == 0 and groups == 5


def test_planted_load_then_store_revives_the_cleared_request(model):
    """The same interleaving against the reference's load-then-store form:
    the cleared word comes back as 2, so two more groups would leave."""
    out = np.zeros(3, np.int32)
    model.model_kill_clear_interleaving(1, out.ctypes.data)
    killed, to_kill, groups = out
    assert killed == 1 and to_kill == 2 and groups == 4


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_kill_stress_no_kill_after_the_request_is_withdrawn(model, seed):
    out = np.zeros(6, np.int64)
    model.model_kill_stress(0, 48, 400, seed, out.ctypes.data)
    kills, granted, late, groups, disorder, revived = out
    assert revived == 0, "a withdrawn request came back"
    assert late == 0, "a group left after the scheduler withdrew every request"
    assert kills == granted and groups == 48 - kills
    assert disorder == 0, "only the highest persistent id may leave"
