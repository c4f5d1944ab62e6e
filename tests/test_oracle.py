"""The CPU oracle pinned to the reference.

1. Against the committed golden fixtures, which the reference's own kernels
   produced (tests/golden/make_golden.py).
2. Against the reference's kernels run live under the shim, on more seeded
   graphs, when the reference checkout is present (this container).
3. The OpenMP variants (the timed CPU baseline) against the sequential oracle.
Mirrors the reference's per-node diff checks (lonestar/graph_apps/bfs/bfs.h:
336-370, pannotia color.h:166-195, mis.h:170-202) and the matmult hash check
(matmult.h:259-261).
"""
import glob
import os

import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import graphs
from oracle import oracle


def _fixtures(golden_dir):
    return sorted(p for p in glob.glob(os.path.join(golden_dir, "*.npz"))
                  if not p.endswith("tasks.npz"))


def _graph(z):
    return graphs.Graph(z["row_ptr"], z["col"], z["weights"])


@pytest.mark.parametrize("name", ["grid32", "rmat10", "ragged"])
def test_oracle_matches_golden(golden_dir, name):
    z = np.load(os.path.join(golden_dir, f"{name}.npz"))
    g = _graph(z)
    lv = graphs.lonestar_view(g)
    assert np.array_equal(oracle.lonestar_bfs(lv), z["bfs"])
    assert np.array_equal(oracle.lonestar_sssp(lv), z["sssp"])
    assert np.array_equal(oracle.color(g, z["node_value_ref"]), z["color_ref"])
    assert np.array_equal(oracle.color(g, z["node_value_seed"]), z["color_seed"])
    assert np.array_equal(oracle.mis(g, z["node_value_ref"]), z["mis_ref"])
    assert np.array_equal(oracle.mis(g, z["node_value_seed"]), z["mis_seed"])
    assert np.array_equal(oracle.pannotia_sssp(g), z["psssp"])


def test_golden_fixtures_are_nontrivial(golden_dir):
    z = np.load(os.path.join(golden_dir, "grid32.npz"))
    assert z["bfs"].max() == 62  # corner to corner: 31 + 31 levels
    assert (z["mis_seed"] == 2).sum() > 100
    assert z["color_seed"].max() > 2


def test_tasks_golden(golden_dir):
    z = np.load(os.path.join(golden_dir, "tasks.npz"))
    A, B = oracle.matmult_inputs(64, 1234)
    assert np.array_equal(A, z["A"]) and np.array_equal(B, z["B"])
    Cm = oracle.matmult_i32(A, B)
    assert np.array_equal(Cm, z["C"])
    assert oracle.hash_diag(Cm) == int(z["hash"])
    assert oracle.reduce_min_i32(z["reduce_in"]) == int(z["reduce_min"])


needs_ref = pytest.mark.skipif(not oracle.ref_available(),
                               reason="reference shim not built (no reference checkout)")


@needs_ref
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_reference_rmat(seed):
    g = graphs.rmat(9, 8, seed=seed)
    g = graphs.swap_labels(g, graphs.max_degree_vertex(g))
    lv = graphs.lonestar_view(g)
    nv = graphs.seeded_node_values(g.num_nodes, seed)
    assert np.array_equal(oracle.lonestar_bfs(lv), oracle.ref_lonestar_bfs(lv))
    assert np.array_equal(oracle.lonestar_sssp(lv), oracle.ref_lonestar_sssp(lv))
    assert np.array_equal(oracle.color(g, nv), oracle.ref_color(g, nv))
    assert np.array_equal(oracle.mis(g, nv), oracle.ref_mis(g, nv))
    assert np.array_equal(oracle.pannotia_sssp(g), oracle.ref_pannotia_sssp(g))


@needs_ref
def test_oracle_matches_reference_grid_rectangular():
    g = graphs.grid(7, 40)
    g.weights = graphs.uniform_weights(g, seed=4)
    lv = graphs.lonestar_view(g)
    nv = graphs.reference_node_values(g.num_nodes)
    assert np.array_equal(oracle.lonestar_bfs(lv), oracle.ref_lonestar_bfs(lv))
    assert np.array_equal(oracle.lonestar_sssp(lv), oracle.ref_lonestar_sssp(lv))
    assert np.array_equal(oracle.color(g, nv), oracle.ref_color(g, nv))
    assert np.array_equal(oracle.mis(g, nv), oracle.ref_mis(g, nv))


@needs_ref
def test_oracle_matches_reference_tasks():
    A, B = oracle.matmult_inputs(40, 77)
    Cm, h = oracle.ref_matmult(A, B)
    assert np.array_equal(oracle.matmult_i32(A, B), Cm)
    assert oracle.hash_diag(Cm) == h
    buf = np.random.default_rng(1).integers(1, 1 << 30, 4096, dtype=np.int32)
    assert oracle.reduce_min_i32(buf) == oracle.ref_reduce(buf)


@pytest.mark.parametrize("seed", [4, 5])
def test_omp_variants_match_sequential(seed):
    g = graphs.rmat(12, 16, seed=seed)
    lv = graphs.lonestar_view(g)
    nv = graphs.seeded_node_values(g.num_nodes, seed)
    s = graphs.max_degree_vertex(g)
    assert np.array_equal(oracle.lonestar_bfs(lv, s), oracle.lonestar_bfs(lv, s, omp=True))
    assert np.array_equal(oracle.lonestar_sssp(lv, s), oracle.lonestar_sssp(lv, s, omp=True))
    assert np.array_equal(oracle.color(g, nv), oracle.color(g, nv, omp=True))
    assert np.array_equal(oracle.mis(g, nv), oracle.mis(g, nv, omp=True))


def test_sssp_oracle_is_shortest_paths():
    scipy = pytest.importorskip("scipy.sparse.csgraph")
    import scipy.sparse as sp
    g = graphs.rmat(10, 8, seed=8)
    src = np.repeat(np.arange(g.num_nodes), g.degrees())
    m = sp.csr_matrix((g.weights.astype(np.float64), (src, g.col)),
                      shape=(g.num_nodes, g.num_nodes))
    ref = scipy.dijkstra(m, indices=0)
    got = oracle.lonestar_sssp(g, 0).astype(np.float64)
    got[got == 1e9] = np.inf
    assert np.array_equal(ref, got)
    hops = scipy.shortest_path(m, unweighted=True, indices=0)
    b = oracle.lonestar_bfs(g, 0).astype(np.float64)
    b[b == 1e9] = np.inf
    assert np.array_equal(hops, b)


def test_pagerank_f32_close_to_f64():
    g = graphs.rmat(12, 16, seed=2)
    p64 = oracle.pagerank_f64(g)
    p32 = oracle.pagerank_f32_omp(g)
    assert abs(p64.sum() - 1.0) < 1e-9
    assert np.max(np.abs(p32 - p64)) / np.max(np.abs(p64)) < 1e-5


def test_octree_oracle_properties():
    """The octree restatement: leaves tile [0, n) in order, every leaf holds
    at most maxchilds particles (a box is split above that), every particle
    of a leaf lies in its octant of the parent box, and the output is a
    permutation of the input."""
    from gpu_workgroup_managment_gb300.octree import clustered_particles
    from oracle import octree_oracle
    p = clustered_particles(20_000, seed=2)
    out, lv = octree_oracle.build(p, 5)
    pos = 0
    for beg, end, (mx, my, mz, _w), o in lv:
        if end == beg:
            continue
        assert beg == pos and end - beg <= 5
        pts = out[beg:end]
        assert np.all((pts[:, 0] >= np.float32(mx)) == bool(o & 1))
        assert np.all((pts[:, 1] >= np.float32(my)) == bool(o & 2))
        assert np.all((pts[:, 2] >= np.float32(mz)) == bool(o & 4))
        pos = end
    assert pos == len(p)
    a = np.sort(p.view(np.uint32).reshape(-1, 4), axis=0)
    b = np.sort(out.view(np.uint32).reshape(-1, 4), axis=0)
    assert np.array_equal(a, b)


def test_connect_four_oracle_known_answer():
    """The restatement reproduces the reference's own check values on its
    committed board (connect_four.h:344-351, via tests/golden)."""
    import json
    with open(os.path.join(os.path.dirname(__file__), "golden", "connect_four.json")) as f:
        d = json.load(f)
    got = oracle.connect_four(np.array(d["board"], np.uint8), d["maxlevel"])
    assert got.tolist() == d["next_move_value"]


def test_bc_oracle_matches_networkx():
    """The float64 restatement of bc.cl is Brandes' betweenness over ordered
    pairs: networkx on the same directed graph agrees."""
    nx = pytest.importorskip("networkx")
    for g in (graphs.rmat(7, 4, seed=3), graphs.grid(6, 9)):
        G = nx.DiGraph()
        G.add_nodes_from(range(g.num_nodes))
        src = np.repeat(np.arange(g.num_nodes), np.diff(g.row_ptr))
        G.add_edges_from(zip(src.tolist(), g.col.tolist()))
        want = nx.betweenness_centrality(G, normalized=False)
        got = oracle.pannotia_bc_f64(g)
        assert np.allclose(got, [want[v] for v in range(g.num_nodes)], rtol=1e-9, atol=1e-9)
        part = oracle.pannotia_bc_f64(g, 5)  # the first 5 sources only
        assert np.all(part <= got + 1e-9)
