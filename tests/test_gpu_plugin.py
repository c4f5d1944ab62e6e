"""A persistent app built outside the library, against include/ alone
(tests/plugin_app/level_count.cu: a level-synchronous BFS that counts the
vertices of each level), registered through wgm_app_register and run like a
built-in app: standalone on discovered groups, and inside the megakernel
next to non-persistent tasks, where groups leave it at resizing barriers
(offer_kill) and come back (offer_fork).  The levels and per-level counts
must equal a host BFS exactly.

The reference binds apps the same way in spirit: kernels written against
kernel_merge/stubs/stubs.h:4-7, host plugin functions per app
(src/lonestar/graph_apps/bfs/bfs.h:192-370) chosen at skel.cpp:50-77."""
import collections
import ctypes as C
import os

import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import Runtime, graphs
from gpu_workgroup_managment_gb300._lib import WgmAppVtable, check
from gpu_workgroup_managment_gb300.communicator import Communicator
from gpu_workgroup_managment_gb300.plugin import RegisteredApp, build_app

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
INF = 0xFFFFFFFF


@pytest.fixture(scope="module")
def app_lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("plugin") / "liblevel_count.so")
    build_app(os.path.join(HERE, "plugin_app", "level_count.cu"), out)
    lib = C.CDLL(out)
    lib.level_count_vtable.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                       C.POINTER(WgmAppVtable)]
    return lib


def _table(app_lib, g, source):
    vt = WgmAppVtable()
    check(app_lib.level_count_vtable(g.num_nodes, g.row_ptr.ctypes.data, g.col.ctypes.data,
                                     source, C.byref(vt)), "level_count_vtable")
    return vt


def _host_bfs(g, source):
    dist = np.full(g.num_nodes, INF, np.uint32)
    dist[source] = 0
    q = collections.deque([source])
    while q:
        v = q.popleft()
        for w in g.col[g.row_ptr[v]:g.row_ptr[v + 1]]:
            if dist[w] == INF:
                dist[w] = dist[v] + 1
                q.append(w)
    counts = np.bincount(dist[dist != INF].astype(np.int64), minlength=g.num_nodes + 1)
    return dist, counts.astype(np.int32)


def _result(app, g):
    raw = app.read(4 * g.num_nodes + 4 * (g.num_nodes + 1))
    return raw[: 4 * g.num_nodes].view(np.uint32), raw[4 * g.num_nodes:].view(np.int32)


@pytest.mark.parametrize("which", ["grid", "rmat"])
def test_registered_app_standalone(app_lib, which):
    g = graphs.grid(48, 80) if which == "grid" else graphs.rmat(12, 8, seed=4)
    src = 0 if which == "grid" else graphs.max_degree_vertex(g)
    want_d, want_c = _host_bfs(g, src)
    with Runtime() as rt:
        with RegisteredApp(rt, _table(app_lib, g, src)) as app:
            for num_wgs in (1, 7, 0):
                st = app.run(num_wgs)
                d, c = _result(app, g)
                assert np.array_equal(d, want_d), num_wgs
                assert np.array_equal(c, want_c), num_wgs
                assert app.check()
                assert st.rounds == int(want_d[want_d != INF].max()) + 1
                assert app.rounds() == st.rounds


def test_registered_app_in_the_megakernel_with_kills_and_forks(app_lib):
    """Non-persistent matmults take half the groups again and again while
    the app runs: the persistent group count dips (groups were killed at
    resizing barriers) and the result is still exact."""
    g = graphs.grid(256, 256)
    want_d, want_c = _host_bfs(g, 0)
    with Runtime() as rt:
        with RegisteredApp(rt, _table(app_lib, g, 0)) as app:
            with Communicator(rt, app, "matmult", 96) as cm:
                cm.launch_mega_kernel()
                n = cm.number_of_discovered_groups()
                cm.send_persistent_task(n)
                tasks = 0
                while cm.is_executing_persistent() and tasks < 200:
                    cm.reset_non_persistent()
                    cm.send_task_synchronous(max(1, n // 2))
                    assert cm.check_non_persistent_task()
                    tasks += 1
                cm.get_persistent_time()
                avg = cm.average_persistent_groups()
                cm.send_quit_signal()
                cm.finish()
            d, c = _result(app, g)
            assert np.array_equal(d, want_d)
            assert np.array_equal(c, want_c)
            assert app.check()
    assert tasks > 0
    assert avg < n, "no group ever left the persistent task"


def test_registered_app_merged_iteration(app_lib):
    """execute_merged_iteration (skel.cpp:405-463) with the registered app as
    the persistent task."""
    g = graphs.rmat(13, 8, seed=9)
    src = graphs.max_degree_vertex(g)
    want_d, _ = _host_bfs(g, src)
    with Runtime() as rt:
        with RegisteredApp(rt, _table(app_lib, g, src)) as app:
            with Communicator(rt, app, "reduce", 1 << 16) as cm:
                occ = cm.get_occupancy_bound()
                r = cm.run_merged_iteration(np_groups=max(1, occ // 2), frequency_ms=0)
                assert r["np_errors"] == 0
            d, _ = _result(app, g)
            assert np.array_equal(d, want_d)
