"""Build libvfsm103.so, the sm_103a shallow-water step library, in-tree.

Eight translation units compile in parallel with nvcc and link into one shared
library with the CUDA runtime linked statically:

  vf_f64.cu  Float64 kernels, -fmad=false (each operation rounds as in Julia),
             quotients through correctly rounded reciprocals (VF_FP64_MARKSTEIN:
             the IEEE quotient's bits); tile kernels held to 80 registers
             (three resident blocks per SM)
  vf_f64f.cu Float64 per-step kernels with faithful quotients, -fmad=true
             (VF_ARITH_FAITHFUL; held to a tolerance, not to the bits)
  vf_f32.cu  Float32 kernels, contraction and fast division allowed
  vf_abi.cu  the extern "C" boundary of include/volumefluxes_sm103.h
  vf_noalloc.cu  the allocation-free water-volume entry point
  vf_batch.cu  the batched-ensemble entry points
  vf_server.cu  the serving engine
  vf_adjoint_host.cu  the reverse sweep (checkpointing, recomputation)

Usage: python volumefluxes.jl_gb300/build_native.py [--force]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
LIB_DIR = HERE / "volumefluxes_sm103" / "lib"
LIB = LIB_DIR / "libvfsm103.so"
BUILD_DIR = HERE / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing",
          f"-I{INCLUDE}", f"-I{CSRC}"]
UNITS = {
    "vf_f64.cu": ["-fmad=false", "-DVF_TILE_MIN_BLOCKS=3", "-DVF_FP64_MARKSTEIN=1"],
    "vf_f64f.cu": ["-fmad=true", "-DVF_TILE_MIN_BLOCKS=3"],
    "vf_f32.cu": ["-fmad=true", "-ftz=true", "-prec-sqrt=false"],
    "vf_abi.cu": [],
    "vf_noalloc.cu": [],
    "vf_batch.cu": [],
    "vf_server.cu": [],
    "vf_adjoint_host.cu": [],
}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the sm_103a library cannot be built")
    return cand


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(s.stat().st_mtime <= t for s in sources()) and Path(__file__).stat().st_mtime <= t


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    exe = nvcc()
    procs = []
    objs = []
    for unit, flags in UNITS.items():
        obj = BUILD_DIR / (unit + ".o")
        objs.append(obj)
        cmd = [exe, *ARCH, *COMMON, *flags, "-c", str(CSRC / unit), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((unit, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for unit, cmd, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            sys.stdout.write(out)
        if p.returncode != 0:
            failed.append(f"{unit}: {' '.join(cmd)}\n{out}")
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    tmp = LIB.with_suffix(".so.tmp")
    link = [exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(link) + "\n" + r.stdout)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
