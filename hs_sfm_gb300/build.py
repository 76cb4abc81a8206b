"""Build recipe of libgba.so (sm_103a only).

Compiles the CUDA translation units of hs_sfm_gb300/csrc in parallel with
nvcc (-gencode arch=compute_103a,code=sm_103a) and links them into
hs_sfm_gb300/_build/libgba.so.  No cmake; a couple of minutes at most.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgba.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = ["gba_kernels.cu", "gba_plan.cu", "gba_noalloc.cu", "gba_server.cu", "gba_triangulate.cu",
         "gba_calibrate.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "gba.h"))
    return files


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps())


def _compile(unit: str) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT_DIR, unit + ".o")
    cmd = [nvcc()] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                             "-Xcompiler", "-fvisibility=hidden", "-I", INCLUDE, "-c", src,
                             "-o", obj]
    subprocess.run(cmd, check=True)
    return obj


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(_compile, UNITS))
    tmp = LIB + ".tmp"
    subprocess.run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
