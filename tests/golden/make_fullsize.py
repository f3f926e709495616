"""Regenerate the full-size golden record of the wet/dry hills workload from the oracle.

Workload: 4096 x 4096 cells over [0,4096]^2 m, 64 seeded Gaussian hills
(seed 20240901) + 1e-3 slope, w = max(1.5, B_cell), Manning n = 0.03
(friction_bsa2012), rain 1e-5 m/s, infiltration 2e-6 m/s, wall BCs, RK2,
CFL 0.25, 1000 perform_step(Inf) calls (src/simulator.jl:145-212).

The fields are too large to store (403 MB per state), so the record holds:
  - the SHA-256 of the terrain and of the initial state, so a machine that
    regenerates them can check it built the same inputs;
  - the whole dt sequence;
  - at steps 1, 2, 10, 100, 300 and 1000: the SHA-256 of each interior field
    (little-endian Float64, C order of the (nx, ny) array), its sum and its
    max-norm;
  - at step 1000: two full rows and two full columns of each field, for a
    tolerance comparison when the hashes differ.

The oracle runs on all host cores; on an 8-core x86 host this takes about
20 minutes.

Usage: python tests/golden/make_fullsize.py [--steps N] [--out PATH]
"""
from __future__ import annotations

import argparse
import hashlib
import math
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "volumefluxes.jl_gb300"))
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE.parent))

N = 4096
STEPS = 1000
CHECKPOINTS = (1, 2, 10, 100, 300, 1000)
ROWS = (1000, 3000)   # interior j indices of the stored rows (h[:, j])
COLS = (1500, 3500)   # interior i indices of the stored columns (h[i, :])
FIELDS = ("w", "hu", "hv")
OUT = HERE / "hills_wet_dry_4096_rk2_1000.npz"


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def summary(fields) -> dict:
    out = {}
    for name, a in zip(FIELDS, fields):
        out[f"{name}_sha"] = sha(a)
        out[f"{name}_sum"] = float(np.sum(a, dtype=np.float64))
        out[f"{name}_max"] = float(np.abs(a).max())
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=STEPS)
    ap.add_argument("--out", default=str(OUT))
    args = ap.parse_args()

    from volumefluxes_sm103 import scenarios as S
    from oracle import vf_oracle as O
    from vfhelpers import oracle_from

    O.set_threads(os.cpu_count() or 1)
    sc = S.hills_wet_dry(N)
    o = oracle_from(sc)
    rec = {"B_sha": sha(sc.B), "w0_sha": sha(sc.w0), "n": N, "steps": args.steps}
    cps = [c for c in CHECKPOINTS if c <= args.steps]
    dts = []
    table = {}
    t0 = time.time()
    for k in range(1, args.steps + 1):
        dts.append(o.perform_step(math.inf))
        if k in cps:
            f = o.interior()
            for key, v in summary(f).items():
                table.setdefault(key, []).append(v)
            print(f"step {k}: t = {math.fsum(dts):.6f} s, {time.time() - t0:.0f} s elapsed", flush=True)
    w, hu, hv = o.interior()
    arrays = {}
    for name, a in zip(FIELDS, (w, hu, hv)):
        arrays[f"{name}_rows"] = np.stack([a[:, j] for j in ROWS])
        arrays[f"{name}_cols"] = np.stack([a[i, :] for i in COLS])
    np.savez_compressed(
        args.out,
        dts=np.asarray(dts),
        checkpoints=np.asarray(cps),
        rows=np.asarray(ROWS), cols=np.asarray(COLS),
        B_sha=rec["B_sha"], w0_sha=rec["w0_sha"],
        **{k: np.asarray(v) for k, v in table.items()},
        **arrays,
    )
    print("wrote", args.out, f"({time.time() - t0:.0f} s of oracle time on {O.get_threads()} threads)")


if __name__ == "__main__":
    main()
