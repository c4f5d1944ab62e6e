"""wgm_bfs_noalloc: the BFS entry point for callers that cannot allocate GPU
memory (their own pool allocator owns the device, or cudaMalloc/cudaFree's
implicit synchronisation is not acceptable on their call path).

It runs on caller-owned device buffers with a static scratch array inside the
library.  Checked through the C-ABI against the regular entry point
(wgm_run_persistent, which allocates its own buffers), bit-exact, on two calls
in a row, so the second call also shows that the scratch left behind by the
first call does not leak into the result.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import PersistentApp, Runtime, graphs
from gpu_workgroup_managment_gb300._lib import STATUS_CODE, lib

pytestmark = pytest.mark.gpu

MAX_NODES = 1 << 18  # WGM_NOALLOC_MAX_NODES in include/wgm.h


def _regular_bfs(g, source):
    with Runtime() as rt, PersistentApp(rt, "lonestar_bfs", g, source=source) as app:
        app.run()
        return app.result()


def _noalloc_bfs(torch, g, source):
    dev = torch.device("cuda:0")
    rp = torch.from_numpy(g.row_ptr).to(dev)
    col = torch.from_numpy(g.col if g.num_edges else np.zeros(1, np.int32)).to(dev)
    dist = torch.full((g.num_nodes,), -1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    st = lib.wgm_bfs_noalloc(C.c_void_p(rp.data_ptr()), C.c_void_p(col.data_ptr()),
                             g.num_nodes, g.num_edges, source, C.c_void_p(dist.data_ptr()),
                             None)
    assert st == 0, f"wgm_bfs_noalloc returned {st}"
    return dist.cpu().numpy().view(np.uint32)


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    first = graphs.lonestar_view(graphs.grid(128, 96))
    second = graphs.lonestar_view(graphs.rmat(14, 16, seed=21))
    src2 = graphs.max_degree_vertex(second)
    got1 = _noalloc_bfs(torch, first, 0)
    got2 = _noalloc_bfs(torch, second, src2)
    assert np.array_equal(got1, _regular_bfs(first, 0))
    assert np.array_equal(got2, _regular_bfs(second, src2))


def test_noalloc_rejects_graph_beyond_limit():
    st = lib.wgm_bfs_noalloc(C.c_void_p(16), C.c_void_p(16), MAX_NODES + 1, 10, 0,
                             C.c_void_p(16), None)
    assert st == STATUS_CODE["WGM_ERR_INVALID"]


def test_noalloc_rejects_bad_arguments_then_still_matches():
    """Arguments the entry point refuses before it launches anything: a
    source below 0 or at num_nodes, and no column array for a graph with
    edges.  A valid call afterwards still equals the regular entry point."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    g = graphs.lonestar_view(graphs.rmat(12, 8, seed=5))
    bad = STATUS_CODE["WGM_ERR_INVALID"]
    p = C.c_void_p(16)  # never dereferenced: every case is refused first
    for source, col in ((-1, p), (g.num_nodes, p), (0, None)):
        st = lib.wgm_bfs_noalloc(p, col, g.num_nodes, g.num_edges, source, p, None)
        assert st == bad, (source, col, st)
    src = graphs.max_degree_vertex(g)
    assert np.array_equal(_noalloc_bfs(torch, g, src), _regular_bfs(g, src))


def test_noalloc_refuses_a_capturing_stream():
    """The call waits for its BFS, which a stream under capture cannot do: it
    returns WGM_ERR_STATE and the caller's capture still completes and
    replays."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    g = graphs.lonestar_view(graphs.grid(16, 16))
    dev = torch.device("cuda:0")
    rp = torch.from_numpy(g.row_ptr).to(dev)
    col = torch.from_numpy(g.col).to(dev)
    dist = torch.zeros(g.num_nodes, dtype=torch.int32, device=dev)
    x = torch.zeros(4, device=dev)
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        x.add_(1.0)
        st = lib.wgm_bfs_noalloc(C.c_void_p(rp.data_ptr()), C.c_void_p(col.data_ptr()),
                                 g.num_nodes, g.num_edges, 0, C.c_void_p(dist.data_ptr()),
                                 C.c_void_p(s.cuda_stream))
    assert st == STATUS_CODE["WGM_ERR_STATE"]
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(x.cpu(), torch.full((4,), 1.0))  # captured once, replayed once
    assert np.array_equal(_noalloc_bfs(torch, g, 0), _regular_bfs(g, 0))
