"""Build libwgm.so (the CUDA kernels and the C-ABI) in-tree for sm_103a.

Every translation unit is compiled by nvcc in parallel with
`-gencode arch=compute_103a,code=sm_103a`; the shared library is linked with
the static CUDA runtime so it loads on a machine without a GPU (calls then
return WGM_ERR_NO_DEVICE).  The library is written next to this file; a
SHA-256 of its sources, flags and host architecture (in _build/) decides
whether an existing library is current.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
ROOT = os.path.dirname(PKG)
LIB = os.path.join(PKG, "libwgm.so")
OBJ = os.path.join(PKG, "_build")

SOURCES = ["wgm_kernels.cu", "wgm_runtime.cu", "wgm_apps.cu", "wgm_graphgen.cpp", "wgm_serve.cu",
           "wgm_noalloc.cu", "wgm_mega.cu", "wgm_batch.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwgm")


def _inputs() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    inc = os.path.join(ROOT, "include")
    files += [os.path.join(inc, f) for f in os.listdir(inc)]
    files.append(os.path.abspath(__file__))
    return files


STAMP = os.path.join(OBJ, "libwgm.sha256")


def _digest() -> str:
    """Hash of every input file, the compile flags and this machine's
    architecture: a library built elsewhere (another checkout, another
    host architecture) or from other sources never counts as current."""
    h = hashlib.sha256()
    h.update(" ".join(ARCH + SOURCES).encode())
    h.update(platform.machine().encode())
    for f in sorted(_inputs()):
        h.update(os.path.basename(f).encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


def needs_build() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(STAMP):
        return True
    with open(STAMP) as f:
        return f.read().strip() != _digest()


def _compile(src: str) -> str:
    nvcc = _nvcc()
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp",
           "-I", os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "c++"]
    subprocess.run(cmd, check=True)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    subprocess.run([_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp",
                    "-lgomp"], check=True)
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(_digest())
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
