"""Build the CPU oracle (test infrastructure only) into oracle/_build/.

g++ with OpenMP and -ffp-contract=off, so every Float64 operation rounds as the
reference's Julia code does (no fused multiply-add).

Usage: python oracle/build.py [--force]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "vf_oracle.cpp"
HDR = HERE / "vf_oracle.h"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libvforacle.so"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and all(p.stat().st_mtime <= LIB.stat().st_mtime for p in (SRC, HDR, Path(__file__))):
        return LIB
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler for the oracle")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
