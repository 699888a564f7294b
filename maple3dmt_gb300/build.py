"""Builds the in-tree native library maple3dmt_gb300/_lib/libm3d_gb300.so.

Host C++ (mesh builder, layout producer) is compiled with g++, the CUDA
translation units with nvcc for sm_103a only, in parallel; nvcc links the
shared library with the static CUDA runtime.  Host code is built with
-ffp-contract=off so the layout arithmetic matches on x86 and Arm.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_lib", "obj")
LIB = os.path.join(LIB_DIR, "libm3d_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SRCS = ["host/octree_build.cpp", "host/mesh_capi.cpp", "host/layout.cpp", "host/layout_capi.cpp", "host/amg.cpp",
             "host/regularization.cpp"]
CUDA_SRCS = ["cuda/krylov.cu", "cuda/physics.cu", "cuda/gradcorr.cu", "cuda/regularization.cu", "cuda/dot.cu",
             "cuda/learned.cu", "solver.cu", "learned_solver.cu", "capi.cu", "noalloc.cu", "learned_capi.cu"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _compile(cmd: list[str]) -> tuple[list[str], int, str]:
    r = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, r.returncode, (r.stdout + r.stderr)


def _stale(obj: str, src: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def build_library(force: bool = False, verbose: bool = False, extra_nvcc: list[str] | None = None) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = []
    for d, _, fs in os.walk(CSRC):
        headers += [os.path.join(d, f) for f in fs if f.endswith((".hpp", ".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    nvcc = _nvcc()
    jobs, objs = [], []
    for s in HOST_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, s.replace("/", "_") + ".o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])
    for s in CUDA_SRCS:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, s.replace("/", "_") + ".o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            jobs.append([nvcc, "-std=c++17", "-O3", *ARCH, "-lineinfo", "--expt-relaxed-constexpr",
                         "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
                         *(extra_nvcc or []), "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for cmd, rc, out in ex.map(_compile, jobs):
                if verbose or rc != 0:
                    sys.stderr.write(" ".join(cmd) + "\n" + out)
                if rc != 0:
                    raise RuntimeError(f"compile failed: {cmd[-3]}")
    if jobs or force or not os.path.exists(LIB):
        tmp = LIB + f".{os.getpid()}.tmp"
        cmd = [nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-lpthread"]
        _, rc, out = _compile(cmd)
        if rc != 0:
            sys.stderr.write(out)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose="-v" in sys.argv))
