"""Builds libibem_gb300.so in-tree with nvcc for sm_103a (no cmake, no torch extension).

The generated sphere/boundary code is refreshed first (codegen.py); every translation
unit is compiled in parallel into _build/ and linked into ibemproject_gb300/libibem_gb300.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libibem_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = [
    "csrc/sphere24.cu", "csrc/sphere60.cu", "csrc/sphere78.cu", "csrc/bem.cu",
    "csrc/solver.cu", "csrc/gemm_tc.cu", "csrc/capi.cu", "csrc/prof.cu", "csrc/mf.cu", "csrc/gnn.cu",
    "csrc/ellipsoid.cu", "csrc/mf60.cu",
    "host/ibem_plugins.cpp", "host/microstructure.cpp", "host/sidecar.cpp",
]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool) -> str:
    path = os.path.join(HERE, src)
    obj = os.path.join(BUILD, os.path.basename(src).replace(".", "_") + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) > max(_deps_mtime(), os.path.getmtime(path)):
        return obj
    cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-c", path, "-o", obj,
           "-I", os.path.join(HERE, "csrc"), "-I", os.path.join(ROOT, "include")]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-4000:]}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


_DEPS = None


def _deps_mtime() -> float:
    global _DEPS
    if _DEPS is None:
        paths = []
        for d in ("csrc", "host"):
            for f in os.listdir(os.path.join(HERE, d)):
                if f.endswith((".h", ".cuh")):
                    paths.append(os.path.join(HERE, d, f))
        paths.append(os.path.join(ROOT, "include", "ibem_gb300.h"))
        _DEPS = max(os.path.getmtime(p) for p in paths)
    return _DEPS


def build(verbose: bool = False, jobs: int | None = None) -> str:
    from . import codegen
    codegen.generate()
    os.makedirs(BUILD, exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
