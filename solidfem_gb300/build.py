"""Build the in-tree CUDA library (solidfem_gb300/lib/libsfem_gb300.so) for sm_103a.

Each translation unit is compiled in parallel with nvcc, then linked into one
shared library with the static CUDA runtime.  No torch, no cmake.

    python -m solidfem_gb300.build
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "lib")
OBJ_DIR = os.path.join(PKG, "lib", "obj")
LIB = os.path.join(OUT_DIR, "libsfem_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["sfem_kernels.cu", "sfem_host.cpp", "sfem_gnn.cu", "sfem_noalloc.cu", "sfem_coarse.cpp", "sfem_patch_nh32.cu",
           "sfem_coarse_kernels.cu"]


def nvcc() -> str:
    for c in [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
                   "-I", CSRC, *extra]


def _compile(src: str) -> str:
    obj = os.path.join(OBJ_DIR, os.path.splitext(os.path.basename(src))[0] + ".o")
    cmd = [nvcc(), *_flags(), "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"] if os.environ.get("SFEM_PTXAS_V") else []
    subprocess.check_call(cmd)
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "sfem.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = True) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"[solidfem_gb300] built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
