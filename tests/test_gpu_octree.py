"""Work-stealing octree build on the GPU (src/test_suite/final_octree): the
reference's own check (leaf counts and particlesDone equal the particle
count), and against the oracle the same leaves - each leaf's particle range,
parent box and octant - with the same particles in every leaf, whatever the
group count, alone or inside the megakernel while non-persistent tasks make
groups leave (offer_kill) and come back (offer_fork) mid-build."""
import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import Runtime, WgmError
from gpu_workgroup_managment_gb300.communicator import Communicator
from gpu_workgroup_managment_gb300.octree import Octree, clustered_particles, leaves
from oracle import octree_oracle

pytestmark = pytest.mark.gpu

FAST = dict(run_timeout_ns=20_000_000_000)


@pytest.fixture(scope="module")
def cloud():
    p = clustered_particles(60_000, seed=4)
    out, lv = octree_oracle.build(p, 5)
    return p, out, lv


def _matches(oc, want_particles, want_leaves):
    assert oc.check()
    tree, done, tasks = oc.tree()
    assert done == oc.n and tasks > 0
    got = leaves(tree, oc.n)
    assert got == want_leaves
    assert octree_oracle.same_leaf_contents(oc.particles(), want_particles, want_leaves)


@pytest.mark.parametrize("num_wgs", [0, 1, 3, 40])
def test_octree_standalone(cloud, num_wgs):
    p, out, lv = cloud
    with Runtime(**FAST) as rt, Octree(rt, p) as oc:
        for _ in range(2):  # every run starts from the input particles
            st = oc.run(num_wgs)
            assert st.rounds > 0
            _matches(oc, out, lv)


def test_octree_other_shapes():
    """A single cluster (deep boxes), maxchilds 1, blocks of 128 and 1024."""
    p = clustered_particles(3_000, seed=9, cluster=3_000)
    for mc, tpw in ((1, 128), (8, 1024)):
        out, lv = octree_oracle.build(p, mc)
        with Runtime(threads_per_wg=tpw, **FAST) as rt, Octree(rt, p, maxchilds=mc) as oc:
            oc.run()
            _matches(oc, out, lv)


def test_octree_overflows_are_reported(cloud):
    p, _, _ = cloud
    with Runtime(**FAST) as rt:
        with Octree(rt, p, pool_size=1) as oc:
            # one group pushes up to 8 children per task and pops one: the
            # one-task pools fill within a few dozen tasks
            with pytest.raises(WgmError):
                oc.run(1)
            assert not oc.check()
        with Octree(rt, p, tree_cap=200) as oc:  # tree full after a dozen blocks
            with pytest.raises(WgmError):
                oc.run()
            assert not oc.check()
        with Octree(rt, p) as oc:  # the runtime stays usable
            oc.run()
            assert oc.check()


def test_octree_in_megakernel_with_kills_and_forks(cloud):
    p, out, lv = cloud
    big = clustered_particles(400_000, seed=5)
    big_out, big_lv = octree_oracle.build(big, 5)
    with Runtime(**FAST) as rt:
        for pts, want, wl in ((p, out, lv), (big, big_out, big_lv)):
            with Octree(rt, pts) as oc, Communicator(rt, oc, "matmult", 64) as cm:
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
                _matches(oc, want, wl)
                if pts is big:
                    assert sent > 0 and avg < n  # groups left the build and came back
        # the merged-iteration driver of the reference (skel.cpp:387-463)
        with Octree(rt, big) as oc, Communicator(rt, oc, "reduce", 1 << 16) as cm:
            r = cm.run_merged_iteration(np_groups=8, frequency_ms=0)
            assert r["np_errors"] == 0
            _matches(oc, big_out, big_lv)
