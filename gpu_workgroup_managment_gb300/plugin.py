"""Apps built outside the library (wgm_app_register in include/wgm.h).

An app author writes a phase function against include/wgm_device.cuh,
instantiates wgm_app_kernels<App> for its standalone kernel and megakernel,
and exports a function that fills a wgm_app_vtable.  build_app compiles such
a source into a shared library (nvcc, sm_103a, include/ on the include
path); RegisteredApp registers a filled table with a runtime and runs it
like a built-in app (standalone, or as the communicator's persistent app).
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

from ._lib import WgmAppVtable, check, lib
from .runtime import RunStats, WgmRunStats

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def build_app(source: str, out: str) -> str:
    """Compile an app's .cu into the shared library `out` against include/."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = out + ".tmp"
    subprocess.run([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-shared", "-Xcompiler",
                    "-fPIC", "-I", INCLUDE, source, "-o", tmp], check=True)
    os.replace(tmp, out)
    return out


class RegisteredApp:
    """A registered app (kind WGM_APP_PLUGIN): `vtable` is a filled
    WgmAppVtable; the runtime owns it from here on (wgm_app_destroy calls its
    clean)."""

    def __init__(self, rt, vtable: WgmAppVtable):
        self.rt = rt
        self.vtable = vtable
        h = C.c_void_p()
        check(lib.wgm_app_register(rt.handle, C.byref(vtable), C.byref(h)), "wgm_app_register")
        self._h = h

    @property
    def name(self) -> str:
        return self.vtable.app_name.decode()

    def run(self, num_wgs: int = 0) -> RunStats:
        st = WgmRunStats()
        check(lib.wgm_run_persistent(self.rt.handle, self._h, num_wgs, C.byref(st)),
              f"run_persistent({self.name})")
        return RunStats(st.groups, st.rounds, st.device_status, st.device_site,
                        st.kernel_ms, st.host_ms)

    def read(self, nbytes: int) -> np.ndarray:
        out = np.empty(nbytes, np.uint8)
        check(lib.wgm_app_read_result(self._h, out.ctypes.data, nbytes), "read_result")
        return out

    def check(self) -> bool:
        ok = C.c_int()
        check(lib.wgm_app_check(self._h, C.byref(ok)), "wgm_app_check")
        return bool(ok.value)

    def rounds(self) -> int:
        r = C.c_int()
        check(lib.wgm_app_rounds(self._h, C.byref(r)))
        return r.value

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
