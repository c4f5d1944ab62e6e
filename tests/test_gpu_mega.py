"""The megakernel and its communicator on the GPU.

Mirrors the reference's merged runs (host_skeleton/skel.cpp:405-631,
run_test.py:362-393): a persistent graph app shares the megakernel with
non-persistent tasks sent as often as possible, so persistent groups are
killed at barriers (offer_kill) and forked back (offer_fork) many times.  The
persistent result must equal the oracle bit for bit (PageRank: FP32 within
1e-5 relative L-inf of the FP64 oracle) and every non-persistent result must
pass its check (matmult.h:259-261, reduce.h:368-370).
"""
import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import PersistentApp, Runtime, WgmError, graphs

FAST = dict(run_timeout_ns=20_000_000_000)  # fail in seconds, not minutes
from gpu_workgroup_managment_gb300.communicator import Communicator
from oracle import oracle

pytestmark = pytest.mark.gpu


def _expected(app, g, source, nv):
    if app == "lonestar_bfs":
        return oracle.lonestar_bfs(g, source)
    if app == "lonestar_sssp":
        return oracle.lonestar_sssp(g, source)
    if app == "color":
        return oracle.color(g, nv)
    if app == "mis":
        return oracle.mis(g, nv)
    if app == "sssp":
        return oracle.pannotia_sssp(g, source)
    return oracle.pagerank_f64(g)


def _same(app, got, want):
    if app == "pagerank":
        return np.max(np.abs(got.astype(np.float64) - want)) / np.max(np.abs(want)) <= 1e-5
    return np.array_equal(got, want)


def _graph_for(app):
    if app in ("lonestar_bfs", "lonestar_sssp"):
        g = graphs.grid(128, 128)
        g.weights = graphs.uniform_weights(g, 3)
        return graphs.lonestar_view(g), 0
    g = graphs.rmat(15, 16, seed=6)
    return g, graphs.max_degree_vertex(g)


APPS = ["lonestar_bfs", "lonestar_sssp", "color", "mis", "sssp", "pagerank"]


@pytest.mark.parametrize("app", APPS)
def test_persistent_alone_in_megakernel(app):
    g, src = _graph_for(app)
    nv = graphs.seeded_node_values(g.num_nodes, 2)
    with Runtime(**FAST) as rt:
        kw = {"node_values": nv} if app in ("color", "mis") else {}
        with PersistentApp(rt, app, g, source=src, **kw) as pa:
            with Communicator(rt, pa, "matmult", 64) as cm:
                r = cm.run_merged_iteration(skip_tasks=True)
                assert r["np_tasks"] == 0
            assert _same(app, pa.result(), _expected(app, g, src, nv))


@pytest.mark.parametrize("app,np_task,np_size", [
    ("lonestar_bfs", "matmult", 128), ("lonestar_sssp", "reduce", 1 << 20),
    ("color", "matmult", 96), ("mis", "reduce_f32", 1 << 18),
    ("sssp", "matmult_f32", 64), ("pagerank", "reduce", 1 << 16),
])
def test_merged_resizing_keeps_results(app, np_task, np_size):
    g, src = _graph_for(app)
    nv = graphs.seeded_node_values(g.num_nodes, 2)
    with Runtime(**FAST) as rt:
        kw = {"node_values": nv} if app in ("color", "mis") else {}
        with PersistentApp(rt, app, g, source=src, **kw) as pa:
            with Communicator(rt, pa, np_task, np_size) as cm:
                occ = cm.get_occupancy_bound()
                assert occ >= 2
                try:
                    r = cm.run_merged_iteration(np_groups=max(1, occ // 2), frequency_ms=0)
                except WgmError as e:
                    raise AssertionError(f"{e}; {rt.last_failure()}; {cm.summary_str()}")
                assert r["np_errors"] == 0
                summ = cm.summary_str()
                assert "Number of discovered groups" in summ
            assert _same(app, pa.result(), _expected(app, g, src, nv))


def test_query_barrier_variant():
    g, src = _graph_for("color")
    nv = graphs.seeded_node_values(g.num_nodes, 5)
    with Runtime(use_query_barrier=1, **FAST) as rt:
        with PersistentApp(rt, "color", g, node_values=nv) as pa:
            with Communicator(rt, pa, "matmult", 64) as cm:
                r = cm.run_merged_iteration(np_groups=4, frequency_ms=0)
                assert r["np_errors"] == 0
            assert np.array_equal(pa.result(), oracle.color(g, nv))


def test_resizing_actually_happens():
    """Groups leave the persistent task for the non-persistent tasks and come
    back: the monitor's persistent group count must dip below the start."""
    g = graphs.lonestar_view(graphs.grid(256, 256))
    with Runtime() as rt:
        with PersistentApp(rt, "lonestar_bfs", g) as pa:
            with Communicator(rt, pa, "matmult", 128) as cm:
                cm.launch_mega_kernel()
                n = cm.number_of_discovered_groups()
                cm.send_persistent_task(n)
                done = 0
                while cm.is_executing_persistent() and done < 50:
                    cm.reset_non_persistent()
                    cm.send_task_synchronous(n // 2)
                    assert cm.check_non_persistent_task()
                    done += 1
                cm.get_persistent_time()
                avg = cm.average_persistent_groups()
                cm.send_quit_signal()
                cm.finish()
                resp, exe = cm.task_times()
            assert np.array_equal(pa.result(), oracle.lonestar_bfs(g, 0))
    assert done > 0 and len(resp) == done
    assert avg < n


def test_non_persistent_only():
    with Runtime() as rt:
        for task, size in (("matmult", 100), ("reduce", 123457), ("matmult_f32", 48),
                           ("reduce_f32", 5000)):
            with Communicator(rt, None, task, size) as cm:
                cm.launch_mega_kernel()
                n = cm.number_of_discovered_groups()
                for groups in (1, n // 3, n):
                    cm.reset_non_persistent()
                    e, r = cm.send_task_synchronous(max(groups, 1))
                    assert cm.check_non_persistent_task(), (task, groups)
                    assert e > 0
                cm.send_quit_signal()
                cm.finish()


def test_too_many_groups_is_an_error():
    with Runtime() as rt:
        with Communicator(rt, None, "reduce", 1000) as cm:
            cm.launch_mega_kernel()
            n = cm.number_of_discovered_groups()
            with pytest.raises(WgmError) as e:
                cm.send_task_synchronous(n + 1)
            assert e.value.name == "WGM_ERR_TOO_MANY_GROUPS"
            cm.send_quit_signal()
            cm.finish()
