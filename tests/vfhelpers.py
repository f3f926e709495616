"""Helpers shared by the tests: building the same scenario in the oracle and in the library."""
from __future__ import annotations

import numpy as np

from oracle import vf_oracle as O
from volumefluxes_sm103 import scenarios as S

LAWS = {"bsa2012": O.FRICTION_BSA2012, "fcg2016": O.FRICTION_FCG2016, "bh2021": O.FRICTION_BH2021}


def oracle_from(sc: S.Scenario, real_bytes: int = 8, sources=None) -> O.OracleSim:
    """An oracle simulation with the scenario's grid, terrain, sources, friction and stepper."""
    if sources is None:
        src = []
        if sc.bottom_source:
            src.append((O.SRC_BOTTOM, 0.0))
        if sc.rain_m_per_h is not None:
            src.append((O.SRC_CONST_RAIN, sc.rain_m_per_h))
        if sc.infiltration_m_per_s is not None:
            src.append((O.SRC_CONST_INFIL, sc.infiltration_m_per_s))
    else:
        src = sources
    fr = LAWS[sc.friction_law] if sc.manning_n is not None else O.FRICTION_NONE
    o = O.OracleSim(nx=sc.nx, ny=sc.ny, extent=sc.extent, real_bytes=real_bytes, theta=sc.theta, sources=src,
                    friction=fr, friction_Cz=(sc.manning_n ** 2 if sc.manning_n else 0.0),
                    stepper=O.STEPPER_RK2 if sc.stepper == "rk2" else O.STEPPER_FE, cfl=sc.cfl, B=sc.B,
                    **sc.eq)
    o.set_interior(sc.w0, sc.hu0, sc.hv0)
    return o


def hills_rect(nx: int, ny: int, n_hills: int = 6, seed: int = 7, **kw) -> S.Scenario:
    """Wet/dry hill terrain on a non-square grid with Δ = 1 m and every source term."""
    extent = ((0.0, float(nx)), (0.0, float(ny)))
    B = S.hill_bottom(nx, ny, extent, n_hills, seed, width=(0.05 * max(nx, ny), 0.25 * max(nx, ny)))
    Bc = 0.25 * (B[:-1, :-1] + B[1:, :-1] + B[:-1, 1:] + B[1:, 1:])[2:-2, 2:-2]
    w0 = np.maximum(1.5, Bc)
    z = np.zeros_like(w0)
    args = dict(name=f"hills_{nx}x{ny}", nx=nx, ny=ny, extent=extent, B=B, w0=w0, hu0=z, hv0=z.copy(), cfl=0.25,
                rain_m_per_h=0.036, infiltration_m_per_s=2e-6, manning_n=0.03, bottom_source=True)
    args.update(kw)
    return S.Scenario(**args)


def max_rel(a, b) -> float:
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)
