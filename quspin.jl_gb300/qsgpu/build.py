"""Builds libqsgpu.so in-tree for sm_103a with nvcc (no GPU needed).

Each translation unit is compiled in parallel, then linked with the static CUDA
runtime, so the library loads with nothing but the NVIDIA kernel driver.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(HERE, "libqsgpu.so")

SOURCES = [
    "qs_basis.cu",
    "qs_matvec.cu",
    "qs_blas.cu",
    "qs_krylov.cu",
    "qs_assembled.cu",
    "qs_noalloc.cu",
    "qs_engine.cu",
    "qs_tools.cu",
    "qs_projector.cu",
    "qs_dense.cpp",
    "qs_op.cpp",
    "qs_capi.cpp",
    "qs_server.cpp",
    "qs_pool.cpp",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
          "-Xcompiler", "-Wall,-Wno-unused-function"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libqsgpu")
    return path


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(PKG), "include", "qsgpu.h"))
    cc = nvcc()
    cmds = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if not _stale(o, [s, __file__] + headers):
            continue
        cmd = [cc, *COMMON, *ARCH, "-c", s, "-o", o]
        if src.endswith(".cu"):
            cmd[1:1] = ["-Xptxas", "-O3"]
        cmds.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, cmds))
    if cmds or not os.path.exists(LIB) or _stale(LIB, objs):
        link = [cc, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs, "-lpthread"]
        run(link)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
