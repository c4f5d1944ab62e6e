"""GPU parity of the persistent kernels, through the C-ABI (libwgm.so).

Bit-exact against (a) the golden fixtures the reference's own kernels
produced, (b) the CPU oracle on seeded graphs, across barrier kinds,
discovery modes, block sizes, grid sizes and hub thresholds, and (c) at the
full sizes of the benchmark configurations, the OpenMP oracle plus
size-independent properties (shortest-path optimality, independence and
maximality).  PageRank: FP32 within 1e-5 relative L-inf (||x-x64||/||x64||)
of the FP64 oracle.
"""
import os

import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import PersistentApp, Runtime, WgmError, graphs
from oracle import oracle

pytestmark = pytest.mark.gpu

PR_TOL = 1e-5


def _run(rt, app, g, **kw):
    with PersistentApp(rt, app, g, **kw) as a:
        st = a.run()
        return a.result(), st


@pytest.mark.parametrize("name", ["grid32", "rmat10", "ragged"])
def test_golden_fixtures(rt, golden_dir, name):
    z = np.load(os.path.join(golden_dir, f"{name}.npz"))
    g = graphs.Graph(z["row_ptr"], z["col"], z["weights"])
    lv = graphs.lonestar_view(g)
    assert np.array_equal(_run(rt, "lonestar_bfs", lv)[0], z["bfs"])
    assert np.array_equal(_run(rt, "lonestar_sssp", lv)[0], z["sssp"])
    for tag in ("ref", "seed"):
        nv = z[f"node_value_{tag}"]
        assert np.array_equal(_run(rt, "color", g, node_values=nv)[0], z[f"color_{tag}"])
        assert np.array_equal(_run(rt, "mis", g, node_values=nv)[0], z[f"mis_{tag}"])
    assert np.array_equal(_run(rt, "sssp", g)[0], z["psssp"])


def _all_apps_vs_oracle(rt, g, source, seed, num_wgs=0):
    lv = graphs.lonestar_view(g)
    nv = graphs.seeded_node_values(g.num_nodes, seed)
    with PersistentApp(rt, "lonestar_bfs", lv, source=source) as a:
        a.run(num_wgs)
        assert np.array_equal(a.result(), oracle.lonestar_bfs(lv, source)), "bfs"
    with PersistentApp(rt, "lonestar_sssp", lv, source=source) as a:
        a.run(num_wgs)
        assert np.array_equal(a.result(), oracle.lonestar_sssp(lv, source)), "sssp"
    with PersistentApp(rt, "color", g, node_values=nv) as a:
        a.run(num_wgs)
        assert np.array_equal(a.result(), oracle.color(g, nv)), "color"
    with PersistentApp(rt, "mis", g, node_values=nv) as a:
        a.run(num_wgs)
        assert np.array_equal(a.result(), oracle.mis(g, nv)), "mis"
    with PersistentApp(rt, "sssp", g, source=source) as a:
        a.run(num_wgs)
        assert np.array_equal(a.result(), oracle.pannotia_sssp(g, source)), "pannotia sssp"
    with PersistentApp(rt, "pagerank", g) as a:
        a.run(num_wgs)
        p64 = oracle.pagerank_f64(g)
        err = np.max(np.abs(a.result().astype(np.float64) - p64)) / np.max(np.abs(p64))
        assert err <= PR_TOL, f"pagerank rel Linf {err}"


@pytest.mark.parametrize("seed", [1, 2])
def test_rmat_all_apps(rt, seed):
    g = graphs.rmat(14, 16, seed=seed)
    _all_apps_vs_oracle(rt, g, graphs.max_degree_vertex(g), seed)


def test_grid_all_apps(rt):
    g = graphs.grid(96, 70)
    g.weights = graphs.uniform_weights(g, seed=5)
    _all_apps_vs_oracle(rt, g, 0, 3)


@pytest.mark.parametrize("num_wgs", [1, 2, 7, 61])
def test_few_groups(rt, num_wgs):
    g = graphs.rmat(12, 8, seed=4)
    _all_apps_vs_oracle(rt, g, graphs.max_degree_vertex(g), 4, num_wgs=num_wgs)


@pytest.mark.parametrize("cfg", [
    dict(barrier_kind=0), dict(barrier_kind=0, threads_per_wg=1024),
    dict(barrier_kind=5, threads_per_wg=1024),
    dict(barrier_kind=1), dict(barrier_kind=2), dict(barrier_kind=2, tree_fanin=3),
    dict(barrier_kind=3), dict(barrier_kind=3, threads_per_wg=128),
    dict(barrier_kind=4), dict(barrier_kind=4, threads_per_wg=1024),
    dict(discovery_mode=1, discovery_extra_rounds=2), dict(threads_per_wg=128),
    dict(threads_per_wg=512), dict(threads_per_wg=1024), dict(hub_threshold=32),
    dict(hub_threshold=63),
    dict(hub_threshold=127), dict(hub_threshold=100000), dict(host_handshake=1),
])
def test_runtime_variants(cfg):
    g = graphs.rmat(13, 16, seed=9)
    with Runtime(**cfg) as r:
        _all_apps_vs_oracle(r, g, graphs.max_degree_vertex(g), 9)


def test_star_and_edge_cases(rt):
    # star: one hub with every other vertex as a leaf, plus isolated vertices
    V = 3000
    leaves = np.arange(1, 2500, dtype=np.int32)
    rows = [leaves.tolist()] + [[0]] * 2499 + [[]] * (V - 2500)
    rp = np.zeros(V + 1, np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    col = np.array([c for r in rows for c in r], np.int32)
    g = graphs.Graph(rp, col, graphs.uniform_weights(graphs.Graph(rp, col), 1))
    _all_apps_vs_oracle(rt, g, 0, 1)
    _all_apps_vs_oracle(rt, g, 2999, 2)   # isolated source
    _all_apps_vs_oracle(rt, g, 17, 3)     # leaf source


def test_color_default_groups():
    """Colour in rounds on the default group count takes 512 threads per SM
    (two 256-thread CTAs); an explicit count is honoured; the colours are the
    oracle's either way."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    g = graphs.rmat(12, 16, seed=3)
    nv = graphs.seeded_node_values(g.num_nodes, 3)
    want = oracle.color(g, nv)
    for tpw, groups in ((256, 2 * sms), (128, 4 * sms), (1024, sms)):
        with Runtime(threads_per_wg=tpw) as r, \
                PersistentApp(r, "color", g, node_values=nv, color_mode=0) as a:
            st = a.run()
            assert st.groups == groups, (tpw, st.groups)
            assert np.array_equal(a.result(), want)
            st = a.run(7)
            assert st.groups == 7
            assert np.array_equal(a.result(), want)


def test_lonestar_default_groups():
    """Lonestar BFS/SSSP on the default group count: one group per 8192
    edges rounded up to the SM count (the 256x256 grid: one CTA per SM),
    every co-resident CTA on large graphs; same distances as on all CTAs."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    gg, gr = graphs.grid(256, 256), graphs.rmat(18, 16, seed=2)  # 262K / 7.5M edges
    gg.weights = graphs.uniform_weights(gg, 1)
    gr.weights = graphs.uniform_weights(gr, 2)
    grid, big = graphs.lonestar_view(gg), graphs.lonestar_view(gr)
    with Runtime() as r:
        for g, small in ((grid, True), (big, False)):
            for app, ref in (("lonestar_bfs", oracle.lonestar_bfs),
                             ("lonestar_sssp", oracle.lonestar_sssp)):
                src = graphs.max_degree_vertex(g)
                want = ref(g, src)
                with PersistentApp(r, app, g, source=src) as a:
                    st = a.run()
                    assert np.array_equal(a.result(), want), app
                    full = a.run(1 << 20).groups
                    assert np.array_equal(a.result(), want), app
                    # the small grid's BFS runs on one CTA (bfs_mode -1 picks it)
                    expect = (1 if app == "lonestar_bfs" else sms) if small else full
                    assert st.groups == expect, (app, st.groups, full)
        # Pannotia SSSP: 1024 threads per SM on the grid
        with PersistentApp(r, "sssp", gg, source=0) as a:
            st = a.run()
            assert st.groups == min(4 * sms, a.run(1 << 20).groups)
            assert np.array_equal(a.result(), oracle.pannotia_sssp(gg, 0))


def test_single_vertex(rt):
    g = graphs.Graph(np.array([0, 0], np.int32), np.zeros(0, np.int32), np.zeros(0, np.uint32))
    for app in ("lonestar_bfs", "lonestar_sssp", "color", "mis", "sssp", "pagerank"):
        out, _ = _run(rt, app, g)
        want = {"lonestar_bfs": 0, "lonestar_sssp": 0, "color": 1, "mis": 2, "sssp": 0,
                "pagerank": 1.0}[app]
        assert out[0] == pytest.approx(want), app


def test_lonestar_quirk_isolated_last_vertex(rt):
    # The last vertex has no edges: with the loader's psrc[V] = E its degree
    # reads -1; the kernels walk nothing for it (like the reference's gather).
    rows = [[1], [0, 2], [1], []]
    rp = np.array([0, 1, 3, 4, 4], np.int32)
    col = np.array([1, 0, 2, 1], np.int32)
    g = graphs.Graph(rp, col, np.ones(4, np.uint32))
    lv = graphs.lonestar_view(g)
    assert lv.row_ptr[-1] == 3 and lv.row_ptr[-2] == 4
    for src in range(4):
        with PersistentApp(rt, "lonestar_bfs", lv, source=src) as a:
            a.run()
            assert np.array_equal(a.result(), oracle.lonestar_bfs(lv, src))


def test_repeated_runs_and_reupload(rt):
    g = graphs.rmat(12, 16, seed=11)
    h = graphs.rmat(12, 16, seed=12)
    lv = graphs.lonestar_view(g)
    with PersistentApp(rt, "lonestar_bfs", lv, source=3) as a:
        first = None
        for _ in range(5):
            a.run()
            r = a.result()
            first = r if first is None else first
            assert np.array_equal(r, first)
        if h.num_edges == g.num_edges:
            a.upload(graphs.lonestar_view(h))
            a.run()
            assert np.array_equal(a.result(), oracle.lonestar_bfs(graphs.lonestar_view(h), 3))


@pytest.mark.parametrize("which", ["grid", "lonestar_grid", "rmat", "star", "isolated",
                                   "path"])
def test_bfs_one_cta(which):
    """Lonestar BFS on one CTA against the oracle and the grid form: same
    levels, same level count, on grids (with the loader's last-edge quirk),
    a small RMAT graph with hubs, a star of degree-1 leaves, an isolated
    source and a long path whose frontier is one vertex for 20,000 levels;
    the automatic mode picks one CTA only for small sparse graphs."""
    src = 0
    if which == "grid":
        g = graphs.grid(120, 200)
    elif which == "lonestar_grid":
        g = graphs.lonestar_view(graphs.grid(256, 256))
    elif which == "rmat":
        g = graphs.rmat(13, 16, seed=6)
        src = graphs.max_degree_vertex(g)
    elif which == "star":
        g = _star_of_leaves(5000)
        src = 17
    elif which == "isolated":
        g = graphs.rmat(10, 4, seed=3)
        src = int(np.flatnonzero(g.degrees() == 0)[0])
    else:
        V = 20000
        rp = np.concatenate([[0, 1], np.arange(3, 2 * V - 1, 2), [2 * V - 2]]).astype(np.int32)
        col = np.empty(2 * V - 2, np.int32)
        col[0] = 1
        for v in range(1, V - 1):
            col[rp[v]], col[rp[v] + 1] = v - 1, v + 1
        col[-1] = V - 2
        g = graphs.Graph(rp, col)
    want = oracle.lonestar_bfs(g, src)
    with Runtime() as r:
        out = {}
        for mode in (-1, 0, 1):
            with PersistentApp(r, "lonestar_bfs", g, source=src, bfs_mode=mode) as a:
                st = a.run()
                out[mode] = (a.result(), st.rounds, st.groups)
        assert np.array_equal(out[1][0], want) and np.array_equal(out[0][0], want)
        assert np.array_equal(out[-1][0], want)
        assert out[1][1] == out[0][1] == out[-1][1]
        assert out[1][2] == 1 and out[0][2] > 1
        sparse_small = g.num_nodes <= 65536 and g.num_edges <= 8 * g.num_nodes
        assert (out[-1][2] == 1) == sparse_small


def test_c1_grid_256_bfs_full_size(rt):
    """Configuration 1: 256x256 grid, source 0, bit-exact levels."""
    g = graphs.lonestar_view(graphs.grid(256, 256))
    with PersistentApp(rt, "lonestar_bfs", g) as a:
        st = a.run()
        d = a.result()
    assert np.array_equal(d, oracle.lonestar_bfs(g, 0))
    assert d.max() == 510 and st.groups > 0


@pytest.fixture(scope="module")
def rmat20():
    g = graphs.rmat(20, 16, seed=1)
    return g, graphs.max_degree_vertex(g)


def _check_sssp_optimal(g, src, dist, inf):
    V = g.num_nodes
    s = np.repeat(np.arange(V), g.degrees())
    d = dist.astype(np.int64)
    w = g.weights.astype(np.int64)
    fin = d[s] != inf
    # no edge can improve a distance
    assert np.all(d[g.col[fin]] <= d[s[fin]] + w[fin])
    # every reached vertex but the source is tight on some in-edge
    tight = np.zeros(V, bool)
    ok = fin & (d[g.col] == d[s] + w)
    tight[g.col[ok]] = True
    reached = d != inf
    reached[src] = False
    assert np.all(tight[reached])


def test_c2_rmat20_sssp_color_mis_full_size(rt, rmat20):
    """Configuration 2 at full size: RMAT-20, source = max-degree vertex."""
    g, src = rmat20
    with PersistentApp(rt, "lonestar_sssp", g, source=src) as a:
        a.run()
        d = a.result()
    assert np.array_equal(d, oracle.lonestar_sssp(g, src, omp=True))
    _check_sssp_optimal(g, src, d, 1000000000)
    nv = graphs.seeded_node_values(g.num_nodes, 1)
    with PersistentApp(rt, "color", g, node_values=nv) as a:
        a.run()
        c = a.result()
    assert np.array_equal(c, oracle.color(g, nv, omp=True))
    assert c.min() >= 1
    with PersistentApp(rt, "mis", g, node_values=nv) as a:
        a.run()
        m = a.result()
    assert np.array_equal(m, oracle.mis(g, nv, omp=True))
    s = np.repeat(np.arange(g.num_nodes), g.degrees())
    member = m == 2
    assert not np.any(member[s] & member[g.col])             # independent
    covered = member.copy()
    covered[g.col[member[s]]] = True
    assert np.all(covered)                                    # maximal


def test_c2_rmat20_bfs_full_size(rt, rmat20):
    g, src = rmat20
    with PersistentApp(rt, "lonestar_bfs", g, source=src) as a:
        a.run()
        d = a.result()
    assert np.array_equal(d, oracle.lonestar_bfs(g, src, omp=True))


def test_c3_rmat22_pagerank_full_size(rt):
    """Configuration 3: FP32 pull PageRank on RMAT-22, damping 0.85, 20
    iterations, within 1e-5 relative L-inf of the FP64 oracle; and the colour
    of the same graph (the served form's resident job) against the oracle."""
    g = graphs.rmat(22, 16, seed=1)
    with PersistentApp(rt, "pagerank", g) as a:
        a.run()
        p = a.result()
    p64 = oracle.pagerank_f64(g)
    err = np.max(np.abs(p.astype(np.float64) - p64)) / np.max(np.abs(p64))
    assert err <= PR_TOL, f"pagerank rel Linf {err}"
    nv = graphs.seeded_node_values(g.num_nodes, 1)
    with PersistentApp(rt, "color", g, node_values=nv) as a:
        a.run()
        c = a.result()
    assert np.array_equal(c, oracle.color(g, nv, omp=True))


def test_invalid_inputs_rejected(rt):
    g = graphs.rmat(8, 8, seed=1)
    bad = graphs.Graph(g.row_ptr.copy(), g.col.copy(), g.weights)
    bad.col[5] = g.num_nodes + 3
    with pytest.raises(WgmError) as e:
        PersistentApp(rt, "color", bad)
    assert e.value.name == "WGM_ERR_INVALID"
    loop = graphs.Graph(np.array([0, 1, 2], np.int32), np.array([0, 0], np.int32))
    with pytest.raises(WgmError):
        PersistentApp(rt, "mis", loop)
    with PersistentApp(rt, "color", g) as a:
        with pytest.raises(WgmError):
            a.set_node_values(np.zeros(g.num_nodes, np.float32))
    with PersistentApp(rt, "lonestar_bfs", g) as a:
        with pytest.raises(WgmError):
            a.set_source(g.num_nodes)
    with pytest.raises(WgmError):
        PersistentApp(rt, "lonestar_sssp", graphs.Graph(g.row_ptr, g.col, None))


def _drop_edges(g, keep_frac, seed):
    """A directed graph: every edge of g kept with probability keep_frac."""
    rng = np.random.default_rng(seed)
    src = np.repeat(np.arange(g.num_nodes), np.diff(g.row_ptr))
    keep = rng.random(g.num_edges) < keep_frac
    rp = np.zeros(g.num_nodes + 1, np.int32)
    rp[1:] = np.cumsum(np.bincount(src[keep], minlength=g.num_nodes))
    return graphs.Graph(rp, g.col[keep].astype(np.int32))


def _star_of_leaves(n):
    """Vertex 0 joined to n leaves (every leaf has degree 1), plus a path
    0-n+1-n+2 so the hub also has higher-degree neighbours."""
    rows = [list(range(1, n + 1)) + [n + 1]] + [[0]] * n + [[0, n + 2], [n + 1]]
    rp = np.zeros(len(rows) + 1, np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    return graphs.Graph(rp, np.array([c for r in rows for c in r], np.int32))


@pytest.mark.parametrize("which", ["rmat", "grid", "star", "directed", "hubs"])
def test_color_without_rounds(which):
    """Colour without rounds (the option of standalone runs) against the oracle and
    against the round form: same colours, same round count (the largest
    colour), on a small graph count, a high-diameter grid, degree-1 leaves
    (color.cl:46), a directed subgraph and a low hub threshold."""
    cfg = {}
    if which == "rmat":
        g = graphs.rmat(14, 16, seed=31)
    elif which == "grid":
        g = graphs.grid(90, 70)
    elif which == "star":
        g = _star_of_leaves(3000)
    elif which == "directed":
        g = _drop_edges(graphs.rmat(12, 8, seed=8), 0.6, 9)
    else:
        g = graphs.rmat(12, 16, seed=4)
        cfg = dict(hub_threshold=8)
    nv = graphs.seeded_node_values(g.num_nodes, 23)
    want = oracle.color(g, nv)
    with Runtime(**cfg) as r:
        with PersistentApp(r, "color", g, node_values=nv, color_mode=1) as a:
            s1 = [a.run(), a.run(13)]
            c1 = a.result()
        with PersistentApp(r, "color", g, node_values=nv, color_mode=0) as a:
            s0 = a.run()
            c0 = a.result()
    assert np.array_equal(c1, want) and np.array_equal(c0, want)
    assert all(s.rounds == s0.rounds == int(want.max()) for s in s1)
    assert s1[1].groups == 13


@pytest.mark.parametrize("kind", ["symmetric", "directed", "unsorted"])
def test_color_graph_shapes(kind):
    """Colour on a symmetric RMAT with hubs, on a directed subgraph (the
    in-edge transpose differs from the rows) and on the symmetric graph with
    shuffled rows (its transpose is uploaded instead of shared): the
    oracle's colours, with and without the hub pass."""
    g = graphs.rmat(13, 8, seed=21)
    if kind == "directed":
        g = _drop_edges(g, 0.7, 4)
    elif kind == "unsorted":
        rng = np.random.default_rng(5)
        col = g.col.copy()
        for v in range(g.num_nodes):
            seg = col[g.row_ptr[v]:g.row_ptr[v + 1]]
            rng.shuffle(seg)
        g = graphs.Graph(g.row_ptr, col)
    nv = graphs.seeded_node_values(g.num_nodes, 17)
    for cfg in (dict(), dict(hub_threshold=16)):
        for mode in (0, 1):
            with Runtime(**cfg) as r, \
                    PersistentApp(r, "color", g, node_values=nv, color_mode=mode) as a:
                a.run()
                assert np.array_equal(a.result(), oracle.color(g, nv)), (kind, cfg, mode)
