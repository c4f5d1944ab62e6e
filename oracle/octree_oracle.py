"""CPU restatement of the reference's octree build
(src/test_suite/final_octree/device/octree.cl:215-316, init at :106-147).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker, never on the
product path.

The build is a recursion over tasks: a task (box centre and half-width, a
range [beg, end) of one of two buffers, which buffer) counts its particles
per octant (octree.cl:96-101: bit 0 x >= centre.x, bit 1 y, bit 2 z), moves
them into the other buffer grouped by octant, and for each octant either
recurses (more than maxchilds particles; child centre = centre +- half-width,
half-width halved, buffers swapped, octree.cl:262-272) or closes a leaf whose
particles end up in the first buffer (octree.cl:290-300).

The GPU build runs the tasks in any order and places the particles of an
octant in any order, so what is fixed is the set of leaves - each leaf's
range, its parent box and octant - and the multiset of particles in each
leaf's range.  `build` returns exactly those, with the particles of each
range in one arbitrary order (stable by input position).
"""
from __future__ import annotations

import numpy as np

ROOT = (np.float32(0.0), np.float32(0.0), np.float32(0.0), np.float32(256.0))


def build(particles: np.ndarray, maxchilds: int = 5):
    """-> (particles_out (n, 4) float32, leaves sorted: (beg, end, parent box
    (x, y, z, w) as floats, octant))."""
    p = np.ascontiguousarray(particles, dtype=np.float32)
    n = p.shape[0]
    buf = [p.copy(), np.zeros_like(p)]
    leaves = []
    stack = [(ROOT, 0, n, 0)]
    while stack:
        (mx, my, mz, w), beg, end, flip = stack.pop()
        frm, to = buf[flip], buf[1 - flip]
        pts = frm[beg:end]
        box = ((pts[:, 0] >= mx).astype(np.int64) + 2 * (pts[:, 1] >= my)
               + 4 * (pts[:, 2] >= mz))
        counts = np.bincount(box, minlength=8)
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
        to[beg:end] = pts[np.argsort(box, kind="stable")]
        for o in range(8):
            s0, c = beg + int(starts[o]), int(counts[o])
            if c > maxchilds:
                sx = np.float32(1 if o & 1 else -1)
                sy = np.float32(1 if o & 2 else -1)
                sz = np.float32(1 if o & 4 else -1)
                child = (np.float32(mx + w * sx), np.float32(my + w * sy),
                         np.float32(mz + w * sz), np.float32(w / np.float32(2)))
                stack.append((child, s0, s0 + c, 1 - flip))
            else:
                leaves.append((s0, s0 + c, (float(mx), float(my), float(mz), float(w)), o))
                if flip == 0:
                    buf[0][s0:s0 + c] = to[s0:s0 + c]
    return buf[0], sorted(leaves)


def same_leaf_contents(a: np.ndarray, b: np.ndarray, leaves) -> bool:
    """Every leaf range holds the same particles (bit for bit) in a and b."""
    for beg, end, _, _ in leaves:
        if end - beg < 1:
            continue
        x = a[beg:end].view(np.uint32)
        y = b[beg:end].view(np.uint32)
        kx = np.lexsort(x.T[::-1])
        ky = np.lexsort(y.T[::-1])
        if not np.array_equal(x[kx], y[ky]):
            return False
    return True
