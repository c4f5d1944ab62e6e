"""Compile the reference's own OpenCL kernels as C++ under the one-work-group
shim (oracle/ref_shim) into oracle/_ref/libref_<app>.so.

TEST INFRASTRUCTURE ONLY.  This reads the reference sources where they lie
(the reference checkout, default /root/reference, or $WGM_REFERENCE_ROOT) and
writes nothing but build outputs under oracle/_ref/.  No reference source is
copied into this repository: the one rewrite the shim needs (a `__local`
array declared inside a kernel body becomes a function-`static`, i.e. storage
shared by all work-items of the group) is applied in memory and the result is
piped straight into the compiler.

Usage:  python oracle/build_ref.py [--reference PATH] [--jobs N]
Returns (exit code 0) silently when the reference checkout is absent.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_shim")

# app name -> (kernel source, restoration_ctx dir, driver macro)
APPS = {
    "lonestar_bfs": ("src/lonestar/graph_apps/bfs/device/standalone.cl",
                     "src/lonestar/graph_apps/bfs", "REF_APP_LONESTAR_BFS"),
    "lonestar_sssp": ("src/lonestar/graph_apps/sssp/device/standalone.cl",
                      "src/lonestar/graph_apps/sssp", "REF_APP_LONESTAR_SSSP"),
    "pannotia_color": ("src/pannotia/graph_apps/color/device/standalone.cl",
                       "src/pannotia/graph_apps/color", "REF_APP_PANNOTIA_COLOR"),
    "pannotia_mis": ("src/pannotia/graph_apps/mis/device/standalone.cl",
                     "src/pannotia/graph_apps/mis", "REF_APP_PANNOTIA_MIS"),
    "pannotia_sssp": ("src/pannotia/graph_apps/sssp/device/standalone.cl",
                      "src/pannotia/graph_apps/sssp", "REF_APP_PANNOTIA_SSSP"),
    "matmult": ("src/non_persistent_kernels/matmult/device/matmult.cl",
                "src/lonestar/graph_apps/bfs", "REF_APP_MATMULT"),
    "reduce": ("src/non_persistent_kernels/reduce/device/reduce.cl",
               "src/lonestar/graph_apps/bfs", "REF_APP_REDUCE"),
}

_LOCAL_DECL = re.compile(r"^(\s*)__local(\s+[^()]*;\s*)$")


def _rewrite_local_decls(text: str) -> str:
    """`__local T x[N];` inside a kernel body -> `static T x[N];`."""
    out = []
    for line in text.splitlines():
        m = _LOCAL_DECL.match(line)
        out.append(m.group(1) + "static" + m.group(2) if m else line)
    return "\n".join(out) + "\n"


def reference_root(explicit: str | None = None) -> str | None:
    root = explicit or os.environ.get("WGM_REFERENCE_ROOT", "/root/reference")
    return root if os.path.isdir(os.path.join(root, "src", "scheduler_rt")) else None


def _build_one(root: str, app: str) -> str:
    src, appdir, macro = APPS[app]
    sched = os.path.join(root, "src", "scheduler_rt")
    common = ["g++", "-std=c++20", "-O2", "-fPIC", "-w", "-pthread"]
    kobj = os.path.join(OUT, f"{app}_kernel.o")
    dobj = os.path.join(OUT, f"{app}_driver.o")
    lib = os.path.join(OUT, f"libref_{app}.so")
    with open(os.path.join(root, src)) as f:
        text = _rewrite_local_decls(f.read())
    subprocess.run(
        common + ["-x", "c++", "-include", os.path.join(SHIM, "cl_shim.h"),
                  "-I", os.path.join(sched, "rt_device"),
                  "-I", os.path.join(root, appdir), "-I", sched,
                  "-c", "-", "-o", kobj],
        input=text.encode(), check=True, cwd=OUT)
    subprocess.run(
        common + ["-I", SHIM, "-I", sched, "-I", os.path.join(root, appdir),
                  f"-D{macro}", "-c", os.path.join(SHIM, "ref_driver.cpp"),
                  "-o", dobj], check=True, cwd=OUT)
    subprocess.run(common + ["-shared", "-o", lib, kobj, dobj], check=True, cwd=OUT)
    return lib


def build(reference: str | None = None, jobs: int = 8) -> list[str]:
    root = reference_root(reference)
    if root is None:
        return []
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        return list(ex.map(lambda a: _build_one(root, a), APPS))


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("--jobs", type=int, default=8)
    args = ap.parse_args()
    libs = build(args.reference, args.jobs)
    for lib in libs:
        print(lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
