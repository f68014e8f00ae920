"""Build libsysucfd.so in-tree: nvcc for the CUDA translation units (sm_103a only),
g++ for the host C++, compiled in parallel, linked with the static CUDA runtime.

    python -m sysu_cfd_heat_gb300.build
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsysucfd.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SRCS = ["krylov.cu", "cg.cu", "gmres.cu", "fv.cu", "noalloc.cu", "gnn.cu", "amg.cu", "bicg3.cu", "graph_loop.cu"]
CPP_SRCS = ["case.cpp", "solver.cpp", "capi.cpp", "csr_api.cpp", "laspack_gpu.cpp", "output.cpp",
            "gnn_api.cpp", "batch.cpp", "amg_setup.cpp"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".hpp", ".h", ".cuh"))]
    hs.append(os.path.join(os.path.dirname(PKG), "include", "sysu_cfd.h"))
    return hs


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _headers() + [os.path.abspath(__file__)])


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I" + CSRC, "-I" + os.path.join(os.path.dirname(PKG), "include"), "-I" + os.path.join(cuda, "include")]
    jobs = []
    objs = []
    for s in CU_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append([nvcc] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                                         "-Xptxas", "-v" if verbose else "-O3"] + inc + ["-c", src, "-o", obj])
    for s in CPP_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _stale(obj, src):
            # no FMA contraction on the host: geometry rounds like the reference
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
                        + inc + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static", "-Xcompiler", "-fPIC",
                                                             "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
