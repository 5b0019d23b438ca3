"""Build recipe of the CPU oracle (test infrastructure only): oracle/_build/liboracle.so.

Compiled with the host C++ compiler and OpenMP; no CUDA.  Used by tests/, by
__graft_entry__.smoke() as the checker and by bench.py's CPU-baseline leg.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(ORACLE_DIR, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
SOURCES = [os.path.join(ORACLE_DIR, "mpm_oracle.cpp")]


def is_stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(f) > t for f in SOURCES + [os.path.abspath(__file__)])


def build(force: bool = False) -> str:
    if not force and not is_stale():
        return LIB_PATH
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", *SOURCES, "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
