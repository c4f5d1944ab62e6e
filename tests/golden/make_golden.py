"""Generate the golden fixtures in this directory from the REFERENCE's own
kernels (its OpenCL sources compiled as C++ under the one-work-group shim,
oracle/_ref; build with `python oracle/build_ref.py`).

Each fixture stores the inputs (CSR, weights, priorities) and the outputs the
reference produced, so tests can pin both the CPU oracle and the GPU kernels
to the reference without the reference being present.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gpu_workgroup_managment_gb300 import graphs  # noqa: E402
from oracle import build_ref, oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def cases():
    g = graphs.grid(32, 32)
    g.weights = graphs.uniform_weights(g, seed=11)
    yield "grid32", g, 0
    r = graphs.rmat(10, 16, seed=5)
    s = graphs.max_degree_vertex(r)
    yield "rmat10", graphs.swap_labels(r, s), s
    # ragged: isolated vertices, a chain, a star (hub) and a pair
    rows = [[1, 2, 3, 4, 5, 6, 7, 8], [0], [0], [0], [0], [0], [0], [0], [0, 9], [8, 10],
            [9], [], [13], [12], []]
    rp = np.zeros(len(rows) + 1, np.int32)
    rp[1:] = np.cumsum([len(x) for x in rows])
    col = np.array([y for x in rows for y in x], np.int32)
    h = graphs.Graph(rp, col, None, "ragged")
    h.weights = graphs.uniform_weights(h, seed=3)
    yield "ragged", h, 0


def main() -> int:
    if build_ref.reference_root() is None:
        print("reference checkout not found; nothing generated")
        return 1
    build_ref.build()
    for name, g, orig_source in cases():
        lv = graphs.lonestar_view(g)
        nv_ref = graphs.reference_node_values(g.num_nodes)
        nv_seed = graphs.seeded_node_values(g.num_nodes, 17)
        out = {
            "row_ptr": g.row_ptr, "col": g.col, "weights": g.weights,
            "node_value_ref": nv_ref, "node_value_seed": nv_seed,
            "orig_source": np.int32(orig_source),
            "bfs": oracle.ref_lonestar_bfs(lv),
            "sssp": oracle.ref_lonestar_sssp(lv),
            "color_ref": oracle.ref_color(g, nv_ref),
            "color_seed": oracle.ref_color(g, nv_seed),
            "mis_ref": oracle.ref_mis(g, nv_ref),
            "mis_seed": oracle.ref_mis(g, nv_seed),
            "psssp": oracle.ref_pannotia_sssp(g),
        }
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
        print(name, g.num_nodes, g.num_edges)
    A, B = oracle.matmult_inputs(64, 1234)
    Cm, h = oracle.ref_matmult(A, B)
    rng = np.random.default_rng(9)
    buf = rng.integers(1, 2**31 - 1, size=1 << 13, dtype=np.int32)
    np.savez_compressed(os.path.join(OUT, "tasks.npz"), A=A, B=B, C=Cm, hash=np.int32(h),
                        reduce_in=buf, reduce_min=np.int32(oracle.ref_reduce(buf)))
    print("tasks")
    return 0


if __name__ == "__main__":
    sys.exit(main())
