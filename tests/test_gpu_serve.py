"""Served form on the GPU: a Poisson stream of requests (BFS queries, FP32
reductions, FP32 matrix products) admitted by device memory and run
concurrently on teams of groups, beside a resident persistent colour+BFS job
that cedes groups at its resizing barriers.  Every request's result must be
the same alone and in the mix (bit for bit), BFS results must equal the
oracle, reductions the exact minimum, products a float64 reference within
1e-5 relative, and the persistent job's colours and levels the oracle's."""
import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import PersistentApp, Runtime, graphs
from gpu_workgroup_managment_gb300.serve import Serve, serve_datasets
from oracle import oracle

pytestmark = pytest.mark.gpu

FAST = dict(run_timeout_ns=10_000_000_000)


@pytest.fixture(scope="module")
def data():
    gs, vecs, mats = serve_datasets(seed=3, scales=(9, 10, 11), graphs_per_scale=2,
                                    n_vecs=3, vec_len=(1 << 16) + 3, n_mats=3, mat_n=64)
    return gs, vecs, mats


def _check_request(sv, data, i, kind, a0, a1):
    gs, vecs, mats = data
    out = sv.result(i, kind, a0)
    if kind == 1:
        assert np.array_equal(out, oracle.lonestar_bfs(gs[a0], a1)), ("bfs", i)
    elif kind == 2:
        assert out[0] == vecs[a0].min(), ("reduce", i)
    else:
        ref = mats[a0, 0].astype(np.float64) @ mats[a0, 1].astype(np.float64)
        assert np.max(np.abs(out - ref)) / np.max(np.abs(ref)) <= 1e-5, ("matmul", i)
    return out


def test_requests_only(data):
    gs, vecs, mats = data
    with Runtime(**FAST) as rt, Serve(rt, graphs=gs, vecs=vecs, mats=mats,
                                      arena_bytes=64 << 20) as sv:
        st = sv.run(rate=4000, duration_s=0.1, seed=5, keep_results=True,
                    bfs_groups=3, reduce_groups=2, matmul_groups=4)
        assert st["completed"] == st["arrived"] > 100
        rq = sv.requests()
        assert set(np.unique(rq["kind"])) == {1, 2, 3}
        for i in range(len(rq["kind"])):
            _check_request(sv, data, i, rq["kind"][i], rq["arg0"][i], rq["arg1"][i])
        assert st["lat_p50_us"] > 0 and st["lat_p99_us"] >= st["lat_p50_us"]
        # execution (device) is part of the latency (host); both recorded per request
        assert 0 < st["exec_p50_us"] <= st["lat_p99_us"] and st["wait_p50_us"] >= 0
        done = rq["latency_ns"] >= 0
        assert np.all(rq["exec_ns"][done] > 0) and np.all(rq["exec_ns"][done] <= rq["latency_ns"][done])


def test_same_alone_and_in_the_mix(data):
    """Each request alone (one in flight, no persistent job) and in the mix
    (many in flight, persistent job resizing around them): identical bits."""
    gs, vecs, mats = data
    pg = graphs.rmat(14, 16, seed=11)
    nv = graphs.seeded_node_values(pg.num_nodes, 4)
    src = graphs.max_degree_vertex(pg)
    with Runtime(**FAST) as rt:
        with PersistentApp(rt, "color", pg, node_values=nv) as ca, \
                PersistentApp(rt, "lonestar_bfs", pg, source=src) as ba, \
                Serve(rt, ca, ba, graphs=gs, vecs=vecs, mats=mats, arena_bytes=64 << 20) as sv:
            cfg = dict(rate=3000, duration_s=0.08, seed=9, keep_results=True, bfs_groups=2,
                       reduce_groups=3, matmul_groups=2)
            st = sv.run(max_in_flight=1, **cfg)
            assert st["completed"] == st["arrived"] > 50
            rq = sv.requests()
            alone = [_check_request(sv, data, i, rq["kind"][i], rq["arg0"][i], rq["arg1"][i])
                     for i in range(len(rq["kind"]))]
            st = sv.run(reps=40, reserve=2, max_in_flight=64, **cfg)
            rq2 = sv.requests()
            assert st["persist_reps"] == 40
            n = min(len(rq2["kind"]), len(alone))
            assert n > 10
            for i in range(n):
                assert (rq2["kind"][i], rq2["arg0"][i], rq2["arg1"][i]) == \
                    (rq["kind"][i], rq["arg0"][i], rq["arg1"][i])
                out = sv.result(i, rq2["kind"][i], rq2["arg0"][i])
                assert np.array_equal(out, alone[i]), i
            assert np.array_equal(ca.result(), oracle.color(pg, nv))
            assert np.array_equal(ba.result(), oracle.lonestar_bfs(pg, src))


def test_persistent_job_cedes_and_takes_back_groups(data):
    gs, vecs, mats = data
    pg = graphs.rmat(15, 16, seed=12)
    nv = graphs.seeded_node_values(pg.num_nodes, 6)
    src = graphs.max_degree_vertex(pg)
    with Runtime(**FAST) as rt:
        with PersistentApp(rt, "color", pg, node_values=nv) as ca, \
                PersistentApp(rt, "lonestar_bfs", pg, source=src) as ba, \
                Serve(rt, ca, ba, graphs=gs, vecs=vecs, mats=mats, arena_bytes=64 << 20) as sv:
            alone = sv.run(reps=20)
            assert alone["persist_reps"] == 20 and alone["kills"] == 0
            st = sv.run(rate=5000, duration_s=5.0, reps=20, seed=3, bfs_groups=8,
                        reduce_groups=8, matmul_groups=8)
            assert st["persist_reps"] == 20
            assert st["kills"] > 0 and st["forks"] > 0
            assert st["completed"] == st["arrived"] > 0
            assert np.array_equal(ca.result(), oracle.color(pg, nv))
            assert np.array_equal(ba.result(), oracle.lonestar_bfs(pg, src))
            # the 1 ms groups-over-time trace saw the job shrink and grow back
            t, g = sv.groups_trace()
            assert len(t) == len(g) > 0 and np.all(np.diff(t) > 0)
            assert g.min() == st["persist_groups_min"] and g.min() < g.max()
            assert g.min() <= st["persist_groups_mean"] <= g.max()


def test_persistent_job_capped(data):
    """persist_max_groups: the resident job starts on and forks up to at most
    that many groups (the groups-over-time trace never exceeds it), leaving
    the rest to requests; results stay exact."""
    gs, vecs, mats = data
    pg = graphs.rmat(14, 16, seed=13)
    nv = graphs.seeded_node_values(pg.num_nodes, 7)
    src = graphs.max_degree_vertex(pg)
    with Runtime(**FAST) as rt:
        with PersistentApp(rt, "color", pg, node_values=nv) as ca, \
                PersistentApp(rt, "lonestar_bfs", pg, source=src) as ba, \
                Serve(rt, ca, ba, graphs=gs, vecs=vecs, mats=mats, arena_bytes=64 << 20) as sv:
            cap = max(2, rt.sm_count())
            st = sv.run(rate=5000, duration_s=5.0, reps=20, seed=4, bfs_groups=8,
                        reduce_groups=8, matmul_groups=8, persist_max_groups=cap)
            assert st["persist_reps"] == 20
            assert st["completed"] == st["arrived"] > 0
            t, g = sv.groups_trace()
            assert len(g) > 0 and g.max() <= cap, (g.max(), cap)
            assert np.array_equal(ca.result(), oracle.color(pg, nv))
            assert np.array_equal(ba.result(), oracle.lonestar_bfs(pg, src))
            alone = sv.run(reps=5, persist_max_groups=cap)
            assert alone["persist_reps"] == 5 and alone["kills"] == 0
            t, g = sv.groups_trace()
            assert len(g) == 0 or g.max() <= cap


def test_admission_waits_for_memory(data):
    gs, vecs, mats = data
    with Runtime(**FAST) as rt, Serve(rt, graphs=gs, vecs=vecs, mats=mats,
                                      arena_bytes=160 << 10) as sv:
        st = sv.run(rate=20000, duration_s=0.03, seed=2, keep_results=True, frac_bfs=0.6,
                    frac_reduce=0.2)
        assert st["waited_for_memory"] > 0
        assert st["completed"] == st["arrived"] > 100
        rq = sv.requests()
        for i in range(len(rq["kind"])):
            _check_request(sv, data, i, rq["kind"][i], rq["arg0"][i], rq["arg1"][i])


def test_request_larger_than_arena_is_refused(data):
    gs, vecs, mats = data
    from gpu_workgroup_managment_gb300 import WgmError
    with Runtime(**FAST) as rt, Serve(rt, graphs=gs, vecs=vecs, mats=mats,
                                      arena_bytes=8192) as sv:
        with pytest.raises(WgmError):
            sv.run(rate=1000, duration_s=0.05, seed=1, frac_bfs=1.0, frac_reduce=0.0)


def _djb2_diag(C):
    h = 5381
    for i in range(C.shape[0]):
        h = (h * 33 + int(C[i, i]) % (1 << 32)) % (1 << 32)
    return h


def test_int32_reference_variants(data):
    """reduce.cl (int32 min) and matmult.cl (wrapping int32 product and the
    djb2 hash of its diagonal) as served requests, checked exactly."""
    gs, vecs, mats = data
    rng = np.random.default_rng(8)
    ivecs = rng.integers(1, 2**31 - 1, size=(2, (1 << 15) + 5), dtype=np.int64).astype(np.int32)
    imats = rng.integers(-2**31, 2**31 - 1, size=(2, 2, 64, 64), dtype=np.int64).astype(np.int32)
    with Runtime(**FAST) as rt, Serve(rt, graphs=gs, vecs=vecs, mats=mats,
                                      arena_bytes=64 << 20) as sv:
        sv.set_int_data(ivecs, imats)
        st = sv.run(rate=3000, duration_s=0.05, seed=4, keep_results=True, frac_bfs=0.0,
                    frac_reduce=0.5, frac_int=1.0, reduce_groups=3, matmul_groups=2)
        assert st["completed"] == st["arrived"] > 20
        rq = sv.requests()
        assert set(np.unique(rq["kind"])) == {4, 5}
        for i in range(len(rq["kind"])):
            k, a0 = int(rq["kind"][i]), int(rq["arg0"][i])
            out = sv.result(i, k, a0)
            if k == 4:
                assert out[0] == ivecs[a0].min(), i
            else:
                A = imats[a0, 0].astype(np.int64)
                B = imats[a0, 1].astype(np.int64)
                C = ((A @ B) % (1 << 32)).astype(np.uint32).view(np.int32)
                assert np.array_equal(out[1:].reshape(64, 64), C), i
                assert (int(out[0]) % (1 << 32)) == _djb2_diag(C), i
