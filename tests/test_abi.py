"""C-ABI surface and host logic (no GPU needed).

The library must load on a machine without a GPU, export every function
include/wgm.h declares, and report WGM_ERR_NO_DEVICE instead of crashing.
"""
import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import graphs
from gpu_workgroup_managment_gb300._lib import WgmConfig, header_functions, lib


def test_exports_every_declared_function():
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []


def test_config_default():
    import ctypes as C
    cfg = WgmConfig()
    lib.wgm_config_default(C.byref(cfg))
    assert cfg.threads_per_wg == 256 and cfg.spin_timeout_ns > 0 and cfg.run_timeout_ns > 0
    assert cfg.discovery_extra_rounds == 10  # discovery.cl:43


def test_status_strings():
    for s in range(0, -10, -1):
        assert lib.wgm_status_string(s)


def test_app_names_match_reference_plugins():
    assert lib.wgm_persistent_app_name(1) == b"lonestar_bfs"
    assert lib.wgm_persistent_kernel_name(1) == b"drelax2"
    assert lib.wgm_persistent_app_name(3) == b"color"
    assert lib.wgm_persistent_kernel_name(4) == b"mis_combined"
    assert lib.wgm_persistent_app_name(99) is None


def test_grid_generator_shape():
    g = graphs.grid(256, 256)
    assert g.num_nodes == 65536 and g.num_edges == 261120
    # (up, left, right, down) order
    v = 256 * 5 + 7
    assert list(g.col[g.row_ptr[v]:g.row_ptr[v + 1]]) == [v - 256, v - 1, v + 1, v + 256]


def test_rmat_deterministic_and_symmetric():
    a = graphs.rmat(11, 16, seed=42)
    b = graphs.rmat(11, 16, seed=42)
    assert np.array_equal(a.row_ptr, b.row_ptr) and np.array_equal(a.col, b.col)
    assert np.array_equal(a.weights, b.weights)
    src = np.repeat(np.arange(a.num_nodes), a.degrees())
    fwd = set(zip(src.tolist(), a.col.tolist()))
    assert all((v, u) in fwd for (u, v) in fwd)
    assert all(u != v for (u, v) in fwd)
    assert len(fwd) == a.num_edges  # no duplicates
    assert a.weights.min() >= 1 and a.weights.max() <= 1000
    w = dict(zip(zip(src.tolist(), a.col.tolist()), a.weights.tolist()))
    assert all(w[(u, v)] == w[(v, u)] for (u, v) in list(fwd)[:2000])
    for v in range(0, a.num_nodes, 97):
        row = a.col[a.row_ptr[v]:a.row_ptr[v + 1]]
        assert np.all(np.diff(row) > 0)


def test_rmat_other_seed_differs():
    assert not np.array_equal(graphs.rmat(10, seed=1).col, graphs.rmat(10, seed=2).col)


def test_swap_labels_preserves_structure():
    g = graphs.rmat(9, 8, seed=3)
    s = graphs.max_degree_vertex(g)
    h = graphs.swap_labels(g, s)
    assert h.degrees()[0] == g.degrees()[s]
    assert h.num_edges == g.num_edges
    def edges(x):
        src = np.repeat(np.arange(x.num_nodes), x.degrees())
        return set(zip(src.tolist(), x.col.tolist()))
    m = {0: s, s: 0}
    relabel = {(m.get(u, u), m.get(v, v)) for (u, v) in edges(h)}
    assert relabel == edges(g)


def test_lonestar_view_drops_last_edge():
    g = graphs.grid(4, 4)
    lv = graphs.lonestar_view(g)
    assert lv.row_ptr[-1] == g.num_edges - 1 and lv.num_edges == g.num_edges


def test_gr_roundtrip(tmp_path):
    g = graphs.rmat(8, 8, seed=1)
    p = str(tmp_path / "g.gr")
    graphs.write_gr(p, g)
    h = graphs.read_gr(p)
    assert np.array_equal(g.row_ptr, h.row_ptr) and np.array_equal(g.col, h.col)
    assert np.array_equal(g.weights, h.weights)


def test_node_values_distinct():
    nv = graphs.seeded_node_values(1 << 20, 3)
    assert np.unique(nv).shape[0] == nv.shape[0]
    r = graphs.reference_node_values(1 << 20)
    assert np.all(np.diff(r) > 0)


def test_runtime_without_gpu_reports_no_device():
    import os
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    from gpu_workgroup_managment_gb300 import Runtime, WgmError
    with pytest.raises(WgmError) as e:
        Runtime()
    assert e.value.name == "WGM_ERR_NO_DEVICE"
