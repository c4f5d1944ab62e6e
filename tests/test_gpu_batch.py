"""Batched form on the GPU: every job's result must equal the plain per-graph
launch and the oracle, bit for bit, whatever the block size, CTAs per SM,
worklist piece size, and whether the launch is replayed from a CUDA graph."""
import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import Runtime, graphs
from gpu_workgroup_managment_gb300.batch import Batch, batch_workload
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_batch():
    gs, jobs, _ = batch_workload(n_graphs=40, seed=7, mu=10.0, sigma=2.0, lo=8, hi=13)
    return gs, jobs


def _oracle(gs, jobs):
    out = []
    for gi, algo, src in jobs:
        g = gs[gi]
        out.append(oracle.lonestar_bfs(g, src) if algo == "bfs" else oracle.lonestar_sssp(g, src))
    return out


def test_batch_matches_oracle_and_per_graph(small_batch):
    gs, jobs = small_batch
    want = _oracle(gs, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        b.run(use_cuda_graph=False)
        got = [b.result(k) for k in range(len(jobs))]
        for k in range(len(jobs)):
            assert np.array_equal(got[k], want[k]), k
        b.run_per_graph()
        for k in range(len(jobs)):
            assert np.array_equal(b.result(k), want[k]), ("per-graph", k)
        b.run(use_cuda_graph=True)
        b.run(use_cuda_graph=True)  # replay of the captured graph
        allres = b.results()
        for k in range(len(jobs)):
            assert np.array_equal(allres[b.offsets[k]:b.offsets[k + 1]], want[k])


@pytest.mark.parametrize("threads,ctas,piece", [(128, 1, 16), (512, 2, 64), (1024, 0, 32),
                                                (256, 3, 0)])
def test_batch_configurations(small_batch, threads, ctas, piece):
    gs, jobs = small_batch
    want = _oracle(gs, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        b.configure(threads, ctas, piece)
        b.configure_local(ctas % 3 * 4)  # 0, 4, 8 local rounds across the cases
        b.run(use_cuda_graph=True)
        for k in range(len(jobs)):
            assert np.array_equal(b.result(k), want[k]), k


@pytest.mark.parametrize("team_edges,max_team,threads", [(2000, 8, 256), (500, 64, 128),
                                                         (4000, 3, 512)])
def test_batch_teams(small_batch, team_edges, max_team, threads):
    """Large jobs on teams of CTAs (team counting barrier, global level
    counters): results stay identical, across replays of the CUDA graph."""
    gs, jobs = small_batch
    want = _oracle(gs, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        b.configure(threads, 0, 0)
        b.configure_teams(team_edges, max_team)
        b.configure_local(4 if threads == 256 else 12)  # warp-local continuation
        for rep in range(4):
            b.run(use_cuda_graph=rep > 0)
            allres = b.results()
            for k in range(len(jobs)):
                assert np.array_equal(allres[b.offsets[k]:b.offsets[k + 1]], want[k]), (rep, k)
            if rep == 1:
                b.reorder_by_last_run()  # profile-guided queue order
        st = b.job_stats()
        assert np.all(st["end_ns"] >= st["start_ns"]) and st["team"].max() > 1
        assert np.all(st["levels"] >= 1)


@pytest.mark.parametrize("mult,far_cap,team_edges", [(0, 0, 0), (20, 0, 0), (2, 0, 1500),
                                                     (20, 3, 0), (5, 1, 800), (1e5, 0, 0)])
def test_batch_sssp_schedules(small_batch, mult, far_cap, team_edges):
    """Near-far SSSP (buckets of mult x the mean weight; 0 = the worklist),
    on single CTAs and on teams, with far lists so small that most parked
    vertices take the full-list path: every distance equals the oracle's,
    across replays of the CUDA graph."""
    gs, jobs = small_batch
    want = _oracle(gs, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        b.configure(256, 0, 0)
        b.configure_local(0)
        b.configure_teams(team_edges, 0)
        b.configure_sssp(mult, far_cap)
        for rep in range(3):
            b.run(use_cuda_graph=rep > 0)
            allres = b.results()
            for k in range(len(jobs)):
                assert np.array_equal(allres[b.offsets[k]:b.offsets[k + 1]], want[k]), (rep, k)
        if team_edges:
            assert b.job_stats()["team"].max() > 1


@pytest.mark.parametrize("light,far_cap,team_edges", [(0.05, 0, 0), (0.2, 0, 0), (0.2, 2, 1500),
                                                      (1.0, 0, 800), (3.0, 1, 0), (0.2, 0, 400)])
def test_batch_sssp_heavy_deferral(small_batch, light, far_cap, team_edges):
    """SSSP on the dense (RMAT) graphs with heavy edges deferred to once per
    bucket (buckets of `light` x the mean weight), on single CTAs and teams,
    with far lists so small that parked vertices take the full-list path:
    every distance equals the oracle's, across CUDA-graph replays, and the
    sparse (grid) jobs keep their own schedule."""
    gs, jobs = small_batch
    want = _oracle(gs, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        b.configure(256, 0, 0)
        b.configure_local(0)
        b.configure_teams(team_edges, 0)
        b.configure_sssp(20.0, far_cap)
        b.configure_sssp_dense(light)
        for rep in range(3):
            b.run(use_cuda_graph=rep > 0)
            allres = b.results()
            for k in range(len(jobs)):
                assert np.array_equal(allres[b.offsets[k]:b.offsets[k + 1]], want[k]), (rep, k)
        if team_edges:
            assert b.job_stats()["team"].max() > 1


def test_batch_heavy_deferral_dense_edge_cases():
    """A dense graph whose weights span [1, 10^6] (most edges heavy at every
    bucket width tried) and a clique, from several sources, on single CTAs
    and teams."""
    rng = np.random.default_rng(5)
    V = 600
    rows = [sorted(set(rng.integers(0, V, 24).tolist()) - {v}) for v in range(V)]
    adj = {v: set(r) for v, r in enumerate(rows)}
    for v, r in enumerate(rows):
        for u in r:
            adj[u].add(v)
    rp = np.zeros(V + 1, np.int32)
    rp[1:] = np.cumsum([len(adj[v]) for v in range(V)])
    col = np.array([u for v in range(V) for u in sorted(adj[v])], np.int32)
    g = graphs.Graph(rp, col)
    lo = np.minimum(np.repeat(np.arange(V), np.diff(rp)), col)
    hi = np.maximum(np.repeat(np.arange(V), np.diff(rp)), col)
    g.weights = (1 + (lo * 7919 + hi * 104729) % 1000000).astype(np.uint32)
    K = 40
    kr = np.arange(0, K * (K - 1) + 1, K - 1, dtype=np.int32)
    kc = np.array([u for v in range(K) for u in range(K) if u != v], np.int32)
    clique = graphs.Graph(kr, kc)
    clique.weights = graphs.uniform_weights(clique, 9)
    gs = [g, clique]
    jobs = [(0, "sssp", 0), (0, "sssp", 599), (1, "sssp", 3), (0, "bfs", 5)]
    want = _oracle(gs, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        for light, cap, te in ((0.2, 0, 0), (0.01, 3, 0), (0.001, 0, 2000), (0.5, 1, 500)):
            b.configure_teams(te, 0)
            b.configure_sssp(20.0, cap)
            b.configure_sssp_dense(light)
            b.run()
            for k in range(len(jobs)):
                assert np.array_equal(b.result(k), want[k]), (light, cap, te, k)


@pytest.mark.parametrize("regs,threads", [(64, 1024), (80, 768), (96, 640), (96, 128)])
def test_batch_register_budgets(small_batch, regs, threads):
    """The kernel built for 64, 80 and 96 registers per thread, at the
    largest block each allows: identical results."""
    gs, jobs = small_batch
    want = _oracle(gs, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        b.configure(threads, 0, 0)
        b.configure_kernel(regs)
        b.configure_local(0)
        b.configure_teams(3000, 0)
        for rep in range(2):
            b.run(use_cuda_graph=rep > 0)
            for k in range(len(jobs)):
                assert np.array_equal(b.result(k), want[k]), (rep, k)


def test_batch_edge_cases():
    # single vertex, isolated source, star hub, the Lonestar loader view
    one = graphs.Graph(np.array([0, 0], np.int32), np.zeros(0, np.int32), np.zeros(0, np.uint32))
    rows = [list(range(1, 3000))] + [[0]] * 2999
    rp = np.zeros(3001, np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    star = graphs.Graph(rp, np.array([c for r in rows for c in r], np.int32))
    star.weights = graphs.uniform_weights(star, 1)
    gridv = graphs.grid(20, 30)
    gridv.weights = graphs.uniform_weights(gridv, 2)
    lv = graphs.lonestar_view(gridv)
    gs = [one, star, lv]
    jobs = [(0, "bfs", 0), (0, "sssp", 0), (1, "bfs", 0), (1, "sssp", 17), (2, "bfs", 599),
            (2, "sssp", 0), (1, "bfs", 2999)]
    want = _oracle(gs, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        b.run()
        for k in range(len(jobs)):
            assert np.array_equal(b.result(k), want[k]), k
        b.configure_bfs_one_cta(0)  # BFS on the star and the grid on teams too
        b.configure_teams(100, 4)  # the star and the grid on teams
        b.run()
        for k in range(len(jobs)):
            assert np.array_equal(b.result(k), want[k]), ("teams", k)
        for mult, cap in ((0.5, 2), (0, 0)):  # near-far with tiny buckets and far lists
            b.configure_sssp(mult, cap)
            b.run()
            for k in range(len(jobs)):
                assert np.array_equal(b.result(k), want[k]), ("near-far", mult, k)


LONESTAR_INF = 1000000000  # MYINFINITY of the Lonestar kernels: unreached


@pytest.mark.parametrize("team_edges,threads", [(0, 512), (1500, 256), (300, 128)])
def test_batch_job_work(small_batch, team_edges, threads):
    """Edges walked per job: a BFS job visits every reached vertex once, so
    it walks exactly their edges; an SSSP job walks them at least once (more
    where distances are lowered again), on single CTAs and teams."""
    gs, jobs = small_batch
    want = _oracle(gs, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        b.configure(threads, 0, 0)
        b.configure_teams(team_edges, 0)
        b.configure_bfs_one_cta(0 if team_edges == 300 else 5.0)
        b.run()
        work = b.job_work()
        teams = b.job_stats()["team"]
        for k, (gi, algo, _) in enumerate(jobs):
            g = gs[gi]
            deg = np.maximum(np.diff(g.row_ptr.astype(np.int64)), 0)
            reached = int(deg[want[k] != LONESTAR_INF].sum())
            if algo == "bfs":
                assert work[k] == reached, (k, work[k], reached)
                if team_edges != 300 and g.num_edges <= 5 * g.num_nodes:
                    assert teams[k] == 1, k  # low-degree BFS on one CTA
            else:
                assert work[k] >= reached, (k, work[k], reached)
        if team_edges:
            assert teams.max() > 1


def test_batch_autotune_picks_a_valid_config(small_batch):
    gs, jobs = small_batch
    gs, jobs = gs[:12], [j for j in jobs if j[0] < 12]
    want = _oracle(gs, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        best = b.autotune(reps=1)
        # piece 0 = each graph's own max(32, E/V)
        assert best["threads"] in (128, 256, 512) and best["piece"] in (0, 16, 32, 64)
        assert best["max_regs"] in (64, 80, 96)
        b.run()
        for k in range(len(jobs)):
            assert np.array_equal(b.result(k), want[k]), k


def test_batch_pipelined_submits(small_batch):
    """submit_packed/wait: steps alternate between two device copies; each
    step's distances land in its own host buffer and equal the oracle's for
    the weights that step uploaded (two weight sets, interleaved)."""
    from gpu_workgroup_managment_gb300.runtime import pinned_copy
    from gpu_workgroup_managment_gb300._lib import lib
    gs, jobs = small_batch
    want_a = _oracle(gs, jobs)
    gs_b = []
    for i, g in enumerate(gs):
        h = graphs.Graph(g.row_ptr, g.col, graphs.uniform_weights(g, 900 + i))
        gs_b.append(h)
    want_b = _oracle(gs_b, jobs)
    with Runtime() as rt, Batch(rt, gs, jobs) as b:
        ra, ca, wa = b.pack(gs)
        rb, cb, wb = b.pack(gs_b)
        bufs, keep = [], []
        for arr in (ra, ca, wa, rb, cb, wb):
            x, p = pinned_copy(arr)
            bufs.append(x)
            keep.append(p)
        outs = []
        for k in range(5):
            o, p = pinned_copy(np.zeros(int(b.offsets[-1]), np.uint32))
            outs.append(o)
            keep.append(p)
        for k in range(5):
            src = bufs[:3] if k % 2 == 0 else bufs[3:]
            b.submit_packed(*src, outs[k])
        b.wait()
        for k in range(5):
            want = want_a if k % 2 == 0 else want_b
            for j in range(len(jobs)):
                assert np.array_equal(outs[k][b.offsets[j]:b.offsets[j + 1]], want[j]), (k, j)
        # a plain launch after pipelined steps uses the first copy again
        b.upload(gs_b)
        b.run()
        for j in range(len(jobs)):
            assert np.array_equal(b.result(j), want_b[j]), ("plain", j)
        for p in keep:
            lib.wgm_host_free(p)
