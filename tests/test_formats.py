"""On-disk formats: Metis and DIMACS round trips, the reference parsers'
CSR reproduced by ref_compat, solution files in both styles."""
import numpy as np
import pytest

from gpu_workgroup_managment_gb300 import graphs
from gpu_workgroup_managment_gb300 import formats as F


def _same(a, b):
    return np.array_equal(a.row_ptr, b.row_ptr) and np.array_equal(a.col, b.col)


def test_metis_round_trip(tmp_path):
    g = graphs.rmat(9, 8, seed=3)
    g = graphs.Graph(g.row_ptr, g.col)
    deg = np.diff(g.row_ptr)
    p = tmp_path / "g.metis"
    F.write_metis(str(p), g)
    h = F.read_metis(str(p))
    assert _same(g, h)
    if np.all(deg > 0):
        assert _same(g, F.read_metis(str(p), ref_compat=True))


def test_metis_separators_comments_and_isolated(tmp_path):
    p = tmp_path / "s.metis"
    p.write_text("% comment\n4 2\n2,3\n1\n1 0 4\n\n")
    g = F.read_metis(str(p))
    assert list(g.row_ptr) == [0, 2, 3, 4, 4] and list(g.col) == [1, 2, 0, 0]
    with pytest.raises(ValueError):
        F.read_metis(str(p), ref_compat=True)


def test_dimacs_round_trip_and_reference_layout(tmp_path):
    g = graphs.grid(7, 9)
    g.weights = graphs.uniform_weights(g, 5)
    p = tmp_path / "g.gr.dimacs"
    F.write_dimacs(str(p), g)
    h = F.read_dimacs(str(p))
    assert _same(g, h) and np.array_equal(g.weights, h.weights)
    r = F.read_dimacs(str(p), ref_compat=True)
    # the reference stores each arc (u, v) as row v, col u, twice
    assert r.num_edges == g.num_edges
    arcs = [(int(l.split()[1]) - 1, int(l.split()[2]) - 1) for l in p.read_text().splitlines()
            if l.startswith("a")]
    # rows are started only for tails that occur, in tail order (parse.cpp:764-775): the
    # k-th row of the reference's CSR holds the heads of the k-th distinct tail, twice
    tails = sorted({v for _, v in arcs})
    for k, t in enumerate(tails):
        heads = sorted([u for u, v in arcs if v == t] * 2)
        assert sorted(r.col[r.row_ptr[k]:r.row_ptr[k + 1]].tolist()) == heads
    assert np.all(r.row_ptr[len(tails):] == r.num_edges)


def test_dimacs_reference_rows_after_an_empty_vertex(tmp_path):
    p = tmp_path / "e.dimacs"
    p.write_text("c x\np sp 4 2\na 1 3 7\na 2 3 5\n")
    r = F.read_dimacs(str(p), directed=True, ref_compat=True)
    # arcs become rows 2 (tail 3) only: rows start at 0 for the first row seen
    # and every later row entry is the edge count (parse.cpp:764-775)
    assert list(r.row_ptr) == [0, 2, 2, 2, 2] and list(r.col) == [0, 1]


def test_solution_files(tmp_path):
    v = np.array([0, 3, 1000000000, 7])
    for style in ("pannotia", "lonestar"):
        p = tmp_path / f"sol.{style}"
        F.write_solution(str(p), v, style)
        assert np.array_equal(F.read_solution(str(p)), v)
        assert F.diff_solution(v, str(p))
        assert not F.diff_solution(v + 1, str(p))
    assert (tmp_path / "sol.pannotia").read_text().splitlines()[1] == "2: 3"
    assert (tmp_path / "sol.lonestar").read_text().splitlines()[1] == "2:3"
