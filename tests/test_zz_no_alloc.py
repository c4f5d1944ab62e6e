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
