"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/gba_oracle.cpp into oracle/_build/libgba_oracle.so with the
host compiler.  The product library never links it.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgba_oracle.so")
SOURCES = [os.path.join(HERE, "gba_oracle.cpp"), os.path.join(HERE, "gba_oracle_triangulate.cpp")]
HEADERS = [os.path.join(HERE, "gba_oracle.h"),
           os.path.join(os.path.dirname(HERE), "include", "gba.h")]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in SOURCES + HEADERS)


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O3", "-std=c++17", "-shared", "-fPIC", "-fno-fast-math",
           "-ffp-contract=off", "-o", LIB + ".tmp"] + SOURCES
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
