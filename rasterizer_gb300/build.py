"""Builds librasterizer_gb300.so in-tree (nvcc for sm_103a + g++ for host code).

Compiler flags that matter for exactness: --fmad=false (no contraction of a
multiply and an add into one rounding), -ftz=false and IEEE division/sqrt on
the device; -ffp-contract=off for host code.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib", "librasterizer_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "--fmad=false", "-ftz=false", "-prec-div=true", "-prec-sqrt=true", "-lineinfo",
                     "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I" + CSRC, "-I" + INCLUDE]
CXX_FLAGS = ["-O2", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-I" + CSRC,
             "-I" + INCLUDE]

CU_SOURCES = ["kernels.cu", "learned.cu", "capi.cu", "bake_gpu.cu", "sah_gpu.cu"]
CXX_SOURCES = ["bake.cpp", "files.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".cpp"))]
    return files + [os.path.join(INCLUDE, "rasterizer_gb300.h"), __file__]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    nvcc = _nvcc()
    procs, objs = [], []
    for src in CU_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        cmd = [nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    for src in CXX_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        cmd = ["g++"] + CXX_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for cmd, p in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            failed.append(" ".join(cmd) + "\n" + out)
        elif verbose and out.strip():
            print(out)
    if failed:
        raise RuntimeError("build failed:\n" + "\n".join(failed))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
