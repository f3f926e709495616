"""Regenerate the golden fixtures of this directory from the oracle.

The reference (Julia) cannot run here and publishes no golden fields; the
oracle is pinned by the reference's own known-answer tests
(tests/test_oracle_kats.py). These fixtures freeze the inputs and the oracle's
outputs of two small cases, so that the oracle and the CUDA library are both
checked against fixed bits (tests/test_golden.py, tests/test_gpu_golden.py):

  dam_break_64_rk2_10.npz   circular dam break, 64x64 over [0,1]^2, RK2, CFL 0.2,
                            10 perform_step(Inf) calls
  hills_48x40_rk2_20.npz    wet/dry hills with bottom source, rain, infiltration
                            and Manning friction, RK2, CFL 0.25, 20 steps

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "volumefluxes.jl_gb300"))
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE.parent))

CASES = {
    "dam_break_64_rk2_10": 10,
    "hills_48x40_rk2_20": 20,
}


def generated_scenario(name):
    from volumefluxes_sm103 import scenarios as S
    from vfhelpers import hills_rect
    if name.startswith("dam_break"):
        return S.circular_dam_break(64)
    return hills_rect(48, 40)


def scenario(name):
    """The case with its inputs (terrain, initial state) read from the fixture:
    numpy's exp may differ in the last bit between machines, so the terrain is
    stored rather than regenerated."""
    from dataclasses import replace
    ref = np.load(HERE / f"{name}.npz")
    sc = generated_scenario(name)
    return replace(sc, B=ref["B"] if ref["B"].size else None, w0=ref["w0"], hu0=ref["hu0"], hv0=ref["hv0"])


def run_oracle(name):
    from vfhelpers import oracle_from
    o = oracle_from(scenario(name))
    dts = [o.perform_step(math.inf) for _ in range(CASES[name])]
    w, hu, hv = o.interior()
    return np.asarray(dts), w, hu, hv


def main():
    from vfhelpers import oracle_from
    for name in CASES:
        sc = generated_scenario(name)
        o = oracle_from(sc)
        dts = np.asarray([o.perform_step(math.inf) for _ in range(CASES[name])])
        w, hu, hv = o.interior()
        B = np.zeros(0) if sc.B is None else sc.B
        np.savez_compressed(HERE / f"{name}.npz", B=B, w0=sc.w0, hu0=sc.hu0, hv0=sc.hv0, dts=dts, w=w, hu=hu, hv=hv)
        print("wrote", name)


if __name__ == "__main__":
    main()
