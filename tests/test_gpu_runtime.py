"""Runtime mechanisms on the GPU: discovery, barriers, the standalone host
handshake, and the failure paths (a wait that runs out, a host abort), which
must end in a recorded status with the context still usable - never a hang.
"""
import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import PersistentApp, Runtime, WgmError, graphs
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_occupancy_bound(rt):
    sms = rt.sm_count()
    hw = rt.hw_occupancy_bound(0, 256)  # the discovery probe's own kernel
    found = rt.get_occupancy_bound(256)
    assert sms >= 1 and hw >= sms
    assert 1 <= found <= hw
    assert rt.hw_occupancy_bound("lonestar_bfs", 256) >= sms


def test_reference_mode_discovery(rt):
    with Runtime(discovery_mode=1, discovery_extra_rounds=10) as r:
        n = r.get_occupancy_bound(128)
        assert n >= 1
        res = r.barrier_bench(iterations=100, threads_per_wg=128)
        assert res["groups"] >= 1


@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4, 5])
def test_barrier_bench(kind):
    with Runtime() as r:
        res = r.barrier_bench(iterations=1000, threads_per_wg=256, barrier_kind=kind)
        assert res["groups"] >= r.sm_count()
        assert 0 < res["ns_per_barrier"] < 100000


@pytest.mark.parametrize("threads,csize", [(256, 8), (256, 2), (1024, 4)])
def test_cluster_barrier_bench(threads, csize):
    """The cluster barrier on a cluster grid: every CTA of every co-resident
    cluster is discovered, and 10,000 barriers complete."""
    with Runtime() as r:
        res = r.barrier_bench_cluster(iterations=1000, threads_per_wg=threads,
                                      cluster_size=csize)
        assert res["groups"] >= r.sm_count() * (1 if threads == 1024 else 2)
        assert res["groups"] % csize == 0
        assert 0 < res["ns_per_barrier"] < 100000


def test_cluster_barrier_kind_on_a_plain_launch():
    """WGM_BARRIER_CLUSTER on a launch without clusters: every CTA is its own
    one-CTA cluster, so it is a counting barrier; a persistent BFS using it
    still equals the oracle."""
    g = graphs.lonestar_view(graphs.grid(40, 40))
    with Runtime(barrier_kind=6) as r:
        with PersistentApp(r, "lonestar_bfs", g) as a:
            a.run()
            assert np.array_equal(a.result(), oracle.lonestar_bfs(g, 0))


def test_handshake_run(rt):
    g = graphs.lonestar_view(graphs.grid(64, 64))
    with Runtime(host_handshake=1) as r:
        with PersistentApp(r, "lonestar_bfs", g) as a:
            st = a.run()
            assert st.host_ms > 0
            assert np.array_equal(a.result(), oracle.lonestar_bfs(g, 0))


def test_wait_runs_out_then_context_usable():
    """The kernel waits for DEVICE_TO_PERSISTENT_TASK, which nothing sends;
    its bounded wait expires and the launch reports a timeout."""
    g = graphs.lonestar_view(graphs.grid(32, 32))
    with Runtime(host_handshake=1, spin_timeout_ns=50_000_000) as r:
        with PersistentApp(r, "lonestar_bfs", g) as a:
            a.launch()
            with pytest.raises(WgmError) as e:
                r.synchronize()
            assert e.value.name == "WGM_ERR_TIMEOUT"
    with Runtime() as r2:
        with PersistentApp(r2, "lonestar_bfs", g) as a:
            a.run()
            assert np.array_equal(a.result(), oracle.lonestar_bfs(g, 0))


def test_host_abort_ends_wait():
    g = graphs.lonestar_view(graphs.grid(32, 32))
    with Runtime(host_handshake=1, spin_timeout_ns=20_000_000_000) as r:
        with PersistentApp(r, "lonestar_bfs", g) as a:
            a.launch()
            r.set_abort(1)
            with pytest.raises(WgmError) as e:
                r.synchronize()
            assert e.value.name in ("WGM_ERR_ABORTED", "WGM_ERR_TIMEOUT")
            r.set_abort(0)


def test_reset_after_failure_allows_runs():
    g = graphs.lonestar_view(graphs.grid(32, 32))
    with Runtime(host_handshake=1, spin_timeout_ns=30_000_000) as r:
        with PersistentApp(r, "lonestar_bfs", g) as a:
            a.launch()
            with pytest.raises(WgmError):
                r.synchronize()
            r.reset()
            st = a.run()  # run() does the host side of the handshake
            assert st.groups >= 1
            assert np.array_equal(a.result(), oracle.lonestar_bfs(g, 0))
