"""Work-stealing octree build as a persistent app: the reference's
offer_kill / offer_fork stress test (src/test_suite/final_octree: device
kernel octree.cl, host plugin octree.h) over libwgm's C-ABI.

An `Octree` is a wgm_app: `run()` is wgm_run_persistent on the standalone
kernel, and a `Communicator` built on it runs the same task loop inside the
megakernel, where groups are killed and forked while it works.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import WgmRunStats, check, lib
from .runtime import RunStats


def clustered_particles(n: int, seed: int, cluster: int = 100) -> np.ndarray:
    """Seeded particles shaped like the reference's generator (octree.h:55-77):
    clusters of `cluster` particles; per cluster y and z centres uniform in
    [-400, 400], each particle +-50 around them; x is the particle's index in
    its cluster +-50 (the reference's inner loop variable shadows the x
    centre).  w = 0.  n is rounded down to whole clusters, as there."""
    rng = np.random.default_rng(seed)
    nc = n // cluster
    out = np.zeros((nc * cluster, 4), np.float32)
    cy = rng.random(nc, dtype=np.float32) * 800.0 - 400.0
    cz = rng.random(nc, dtype=np.float32) * 800.0 - 400.0
    k = np.tile(np.arange(cluster, dtype=np.float32), nc)
    out[:, 0] = k + (rng.random(nc * cluster, dtype=np.float32) * 100.0 - 50.0)
    out[:, 1] = np.repeat(cy, cluster) + (rng.random(nc * cluster, dtype=np.float32) * 100.0 - 50.0)
    out[:, 2] = np.repeat(cz, cluster) + (rng.random(nc * cluster, dtype=np.float32) * 100.0 - 50.0)
    return out


class Octree:
    """octree.h's plugin: maxchilds = FLAGS_maxChildren (5), pool_size =
    FLAGS_pool_size (50000), tree_cap = tree entries (MAXTREESIZE there)."""

    def __init__(self, rt, particles: np.ndarray, maxchilds: int = 5, pool_size: int = 50000,
                 tree_cap: int = 0):
        self.rt = rt
        p = np.ascontiguousarray(particles, dtype=np.float32)
        if p.ndim != 2 or p.shape[1] != 4:
            raise ValueError("particles must be (n, 4) float32")
        self.n = p.shape[0]
        # deep chains of single-child boxes need far more entries than
        # particles when maxchilds is small (MAXTREESIZE is 50M there)
        self.tree_cap = tree_cap or (16 * self.n + (1 << 20))
        h = C.c_void_p()
        check(lib.wgm_octree_create(rt.handle, self.n, p.ctypes.data, maxchilds, pool_size,
                                    self.tree_cap, C.byref(h)), "wgm_octree_create")
        self._h = h

    def run(self, num_wgs: int = 0) -> RunStats:
        st = WgmRunStats()
        check(lib.wgm_run_persistent(self.rt.handle, self._h, num_wgs, C.byref(st)),
              "run_persistent(octree)")
        return RunStats(st.groups, st.rounds, st.device_status, st.device_site,
                        st.kernel_ms, st.host_ms)

    def particles(self) -> np.ndarray:
        out = np.empty((self.n, 4), np.float32)
        check(lib.wgm_app_read_result(self._h, out.ctypes.data, out.nbytes), "read_result")
        return out

    def tree(self) -> tuple[np.ndarray, int, int]:
        """(tree entries [0, tree_size), particles done, tasks run)."""
        size, done, tasks = C.c_uint32(), C.c_uint32(), C.c_int32()
        check(lib.wgm_octree_read(self._h, None, 0, C.byref(size), C.byref(done),
                                  C.byref(tasks)))
        used = min(size.value, self.tree_cap)
        t = np.zeros(max(used, 1), np.uint32)
        check(lib.wgm_octree_read(self._h, t.ctypes.data, t.shape[0], None, None, None))
        return t[:used], done.value, tasks.value

    def check(self) -> bool:
        ok = C.c_int32()
        check(lib.wgm_octree_check(self._h, C.byref(ok)))
        return bool(ok.value)

    def close(self) -> None:
        if self._h:
            lib.wgm_app_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def leaves(tree: np.ndarray, n: int) -> list[tuple[int, int, tuple[float, float, float, float]]]:
    """Walk a built tree from the root block: every leaf as (beg, end, box),
    beg/end its particle range (children lie in octant order, each range
    after its elder siblings'), box its (x, y, z, half-width)."""
    out = []
    size_cache: dict[int, int] = {}

    def subtree(pos: int) -> int:
        if pos in size_cache:
            return size_cache[pos]
        s = 0
        for o in range(8):
            e = int(tree[pos + o])
            s += (e & 0x7FFFFFFF) if e & 0x80000000 else subtree(e)
        size_cache[pos] = s
        return s

    stack = [(0, 0, (0.0, 0.0, 0.0, 256.0))]
    while stack:
        pos, beg, (mx, my, mz, w) = stack.pop()
        for o in range(8):
            e = int(tree[pos + o])
            cx = np.float32(mx) + np.float32(w) * np.float32(1 if o & 1 else -1)
            cy = np.float32(my) + np.float32(w) * np.float32(1 if o & 2 else -1)
            cz = np.float32(mz) + np.float32(w) * np.float32(1 if o & 4 else -1)
            if e & 0x80000000:
                c = e & 0x7FFFFFFF
                out.append((beg, beg + c, (float(mx), float(my), float(mz), float(w)), o))
                beg += c
            else:
                sz = subtree(e)
                stack.append((e, beg, (float(cx), float(cy), float(cz), float(np.float32(w) / 2))))
                beg += sz
    return sorted(out)
