"""Pannotia betweenness centrality on the GPU (pannotia/graph_apps/bc):
FP32 with the reference's arithmetic (rho and sigma scaled by 10000, float
atomic adds) against the float64 oracle, relative L-inf error <= 1e-4 of the
largest centrality - standalone, on a directed graph, over a subset of
sources, with few groups, and in the megakernel while non-persistent tasks
resize it at its barriers."""
import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import PersistentApp, Runtime, graphs
from gpu_workgroup_managment_gb300.communicator import Communicator
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-4
FAST = dict(run_timeout_ns=20_000_000_000)


def _err(got, want):
    return float(np.max(np.abs(got.astype(np.float64) - want)) / max(np.max(np.abs(want)), 1e-30))


def _directed(g, keep, seed):
    rng = np.random.default_rng(seed)
    src = np.repeat(np.arange(g.num_nodes), np.diff(g.row_ptr))
    k = rng.random(g.num_edges) < keep
    rp = np.zeros(g.num_nodes + 1, np.int32)
    rp[1:] = np.cumsum(np.bincount(src[k], minlength=g.num_nodes))
    return graphs.Graph(rp, g.col[k].astype(np.int32))


@pytest.mark.parametrize("mode", [0, 1])  # levels over the grid / sources over CTAs
@pytest.mark.parametrize("name", ["rmat10", "grid24", "directed", "subset", "few_groups"])
def test_bc_vs_f64_oracle(name, mode):
    g = graphs.grid(24, 24) if name == "grid24" else graphs.rmat(10, 8, seed=2)
    if name == "directed":
        g = _directed(g, 0.6, 1)
    n_src = 100 if name == "subset" else None
    with Runtime(**FAST) as rt, PersistentApp(rt, "bc", g, bc_sources=n_src, bc_mode=mode) as a:
        for _ in range(2):  # repeat runs start afresh
            st = a.run(3 if name == "few_groups" else 0)
            assert st.rounds == (n_src or g.num_nodes)
            err = _err(a.result(), oracle.pannotia_bc_f64(g, n_src))
            assert err <= TOL, err


def test_bc_cta_mode_limits():
    """Sources over CTAs keep a source's state in shared memory: graphs
    above 10240 vertices must use the level-synchronous form.  (Not a big
    grid: its path counts overflow float, in the reference's arithmetic
    too.)"""
    from gpu_workgroup_managment_gb300 import WgmError
    g = graphs.rmat(14, 8, seed=3)  # 16384 vertices
    with Runtime(**FAST) as rt, PersistentApp(rt, "bc", g, bc_sources=4) as a:
        with pytest.raises(WgmError):
            PersistentApp(rt, "bc", g, bc_sources=4, bc_mode=1)
        a.run()
        assert _err(a.result(), oracle.pannotia_bc_f64(g, 4)) <= TOL


def test_bc_in_megakernel_resized():
    g = graphs.rmat(9, 8, seed=4)
    want = oracle.pannotia_bc_f64(g)
    with Runtime(**FAST) as rt, PersistentApp(rt, "bc", g) as a:
        with Communicator(rt, a, "matmult", 64) as cm:
            r = cm.run_merged_iteration(np_groups=8, frequency_ms=0)
            assert r["np_errors"] == 0
        assert _err(a.result(), want) <= TOL
