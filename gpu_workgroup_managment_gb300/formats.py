"""On-disk graph and solution formats of the reference's inputs and checks.

* Galois `.gr` v1 (Lonestar inputs): `graphs.read_gr` / `graphs.write_gr`.
* Metis adjacency (Pannotia colour/MIS inputs; reader at
  pannotia/graph_parser/parse.cpp:58-175): a header line "n m", then line i
  lists the 1-based neighbours of vertex i, separated by any of " ,.-"; a
  token <= 0 ends the line; '%' lines are comments; an undirected file lists
  both directions and states m once (the reader doubles it).
* DIMACS shortest-path (Pannotia SSSP inputs; reader at parse.cpp:692-797):
  "p sp n m", then "a u v w" arcs (1-based), 'c' comments.
* Solution files: Lonestar's check reads "i:value" lines
  (lonestar/graph_apps/bfs/bfs.h:336-365), Pannotia's "i: value" lines, i
  1-based (pannotia/graph_apps/color/color.h:156, sssp.h:134-168).

Readers return the correct CSR.  `ref_compat=True` reproduces what the
reference's own parsers build instead:
* DIMACS: the reader stores every arc as (tail, head) - the transpose - and
  for an undirected file stores that same pair twice rather than the
  reverse (parse.cpp:735-745); rows of vertices without arcs are filled with
  the running index at the end (parse.cpp:773-775), so rows after an empty
  vertex shift.  Reproduced exactly.
* Metis: rows are started only for vertices that have edges and the rest of
  the row array is left unwritten (parse.cpp:150-160), so a file with an
  isolated vertex has no defined reference CSR; ref_compat raises there.
"""
from __future__ import annotations

import re

import numpy as np

from .graphs import Graph

_METIS_SPLIT = re.compile(r"[ ,.\-]+")


def read_metis(path: str, ref_compat: bool = False) -> Graph:
    rows: list[list[int]] = []
    n = m = None
    with open(path) as f:
        for line in f:
            if line.startswith("%"):
                continue
            if n is None:
                parts = line.split()
                n, m = int(parts[0]), int(parts[1])
                continue
            nb = []
            for tok in _METIS_SPLIT.split(line.strip()):
                if not tok:
                    continue
                v = int(tok)
                if v <= 0:
                    break
                nb.append(v - 1)
            rows.append(nb)
    if n is None:
        raise ValueError("no Metis header line")
    rows += [[] for _ in range(n - len(rows))]
    rows = rows[:n]
    if ref_compat and any(len(r) == 0 for r in rows):
        raise ValueError("the reference's Metis reader leaves rows undefined for isolated vertices")
    deg = np.array([len(r) for r in rows], np.int64)
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum(deg)
    col = np.array([c for r in rows for c in r], np.int32)
    if np.any(col >= n):
        raise ValueError("neighbour id beyond the vertex count")
    return Graph(rp, col)


def write_metis(path: str, g: Graph) -> None:
    """Undirected Metis file of a symmetric graph (m = directed edges / 2)."""
    with open(path, "w") as f:
        f.write(f"{g.num_nodes} {g.num_edges // 2}\n")
        for v in range(g.num_nodes):
            nb = g.col[g.row_ptr[v]:g.row_ptr[v + 1]] + 1
            f.write(" ".join(str(int(x)) for x in nb) + "\n")


def read_dimacs(path: str, directed: bool = False, ref_compat: bool = False) -> Graph:
    arcs = []
    n = None
    with open(path) as f:
        for line in f:
            if not line or line[0] == "c":
                continue
            if line[0] == "p":
                parts = line.split()
                n = int(parts[2])
            elif line[0] == "a":
                _, u, v, w = line.split()[:4]
                arcs.append((int(u) - 1, int(v) - 1, int(w)))
    if n is None:
        raise ValueError("no DIMACS problem line")
    a = np.array(arcs, np.int64).reshape(-1, 3)
    if ref_compat:
        # (row, col) = (tail, head): the transpose; undirected: the same pair twice
        src, dst, w = a[:, 1], a[:, 0], a[:, 2]
        if not directed:
            src, dst, w = np.repeat(src, 2), np.repeat(dst, 2), np.repeat(w, 2)
        order = np.argsort(src, kind="stable")
        src, dst, w = src[order], dst[order], w[order]
        rp = np.zeros(n + 1, np.int32)
        starts, idx = [], 0
        prev = -1
        for i, r in enumerate(src):
            if r != prev:
                starts.append(i)
                prev = r
        rc = len(starts)
        rp[:rc] = starts
        rp[rc:] = len(src)
        return Graph(rp, dst.astype(np.int32), w.astype(np.uint32))
    src, dst, w = a[:, 0], a[:, 1], a[:, 2]
    if not directed:
        src, dst, w = np.concatenate([src, dst]), np.concatenate([dst, src]), np.concatenate([w, w])
    order = np.lexsort((dst, src))
    src, dst, w = src[order], dst[order], w[order]
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum(np.bincount(src, minlength=n))
    return Graph(rp, dst.astype(np.int32), w.astype(np.uint32))


def write_dimacs(path: str, g: Graph, directed: bool = False) -> None:
    """Arcs of the graph (each undirected edge once unless `directed`)."""
    w = g.weights if g.weights is not None else np.ones(g.num_edges, np.uint32)
    src = np.repeat(np.arange(g.num_nodes), np.diff(g.row_ptr))
    keep = np.ones(g.num_edges, bool) if directed else src <= g.col
    with open(path, "w") as f:
        f.write(f"p sp {g.num_nodes} {int(keep.sum())}\n")
        for u, v, x in zip(src[keep], g.col[keep], w[keep]):
            f.write(f"a {u + 1} {v + 1} {int(x)}\n")


def write_solution(path: str, values: np.ndarray, style: str = "pannotia") -> None:
    """One line per vertex, 1-based: "i: v" (Pannotia) or "i:v" (Lonestar)."""
    sep = ": " if style == "pannotia" else ":"
    with open(path, "w") as f:
        for i, v in enumerate(np.asarray(values).tolist()):
            f.write(f"{i + 1}{sep}{v}\n")


def read_solution(path: str) -> np.ndarray:
    vals = []
    with open(path) as f:
        for line in f:
            if ":" in line:
                vals.append(int(line.split(":", 1)[1]))
    return np.array(vals, np.int64)


def diff_solution(values: np.ndarray, path: str) -> bool:
    """The reference's diff_solution_file_int: every value equal, in order."""
    want = read_solution(path)
    v = np.asarray(values).astype(np.int64)
    return len(want) >= len(v) and bool(np.array_equal(want[:len(v)], v))
