"""Helpers shared by the tests: building the same scenario in the oracle and in the library."""
from __future__ import annotations

import numpy as np

from oracle import vf_oracle as O
import volumefluxes_sm103 as vf
from volumefluxes_sm103 import scenarios as S

LAWS = {"bsa2012": O.FRICTION_BSA2012, "fcg2016": O.FRICTION_FCG2016, "bh2021": O.FRICTION_BH2021}


def oracle_sources(source_terms):
    """Oracle source list and the tables/fields to upload, from API source-term objects."""
    src, tables, fields, functional = [], {}, {}, {}
    for i, st in enumerate(source_terms):
        if type(st) is vf.SourceTermBottom:
            src.append((O.SRC_BOTTOM, 0.0))
        elif isinstance(st, vf.ConstantRain):
            src.append((O.SRC_CONST_RAIN, st.rain_rate))
        elif isinstance(st, vf.ConstantInfiltration):
            src.append((O.SRC_CONST_INFIL, st.infiltration_rate))
        elif isinstance(st, vf.TimeDependentRain):
            src.append((O.SRC_TIME_RAIN, 0.0))
            tables[i] = (st.time, st.rain_rates)
        elif isinstance(st, vf.HortonInfiltration):
            src.append((O.SRC_HORTON, st.fc, st.f0, st.k))
            fields[i] = st.factor
        elif isinstance(st, vf.FunctionalRain):
            src.append((O.SRC_RAIN_FIELD, 0.0))
            functional[i] = st
        else:
            raise TypeError(type(st))
    return src, tables, fields, functional


class OracleRun:
    """The oracle driven like the API Simulator (re-evaluating FunctionalRain each step)."""

    def __init__(self, sc: S.Scenario, real_bytes: int = 8):
        src, tables, fields, self.functional = oracle_sources(sc.source_terms())
        fr = LAWS[sc.friction_law] if sc.manning_n is not None else O.FRICTION_NONE
        self.o = O.OracleSim(nx=sc.nx, ny=sc.ny, extent=sc.extent, real_bytes=real_bytes, theta=sc.theta,
                             sources=src, friction=fr, friction_Cz=(sc.manning_n ** 2 if sc.manning_n else 0.0),
                             stepper=O.STEPPER_RK2 if sc.stepper == "rk2" else O.STEPPER_FE, cfl=sc.cfl, B=sc.B,
                             bc={"periodic": O.BC_PERIODIC, "neumann": O.BC_NEUMANN}.get(sc.bc, O.BC_WALL),
                             reconstruction=O.REC_NONE if sc.reconstruction == "none" else O.REC_LINEAR, **sc.eq)
        for i, (t, r) in tables.items():
            self.o.set_source_table(i, t, r)
        for i, f in fields.items():
            self.o.set_source_field(i, f)
        self.o.t = sc.t0
        self.o.set_interior(sc.w0, sc.hu0, sc.hv0)

    def perform_step(self, max_dt):
        for i, st in self.functional.items():
            self.o.set_source_field(i, st.field(self.o.t))
        return self.o.perform_step(max_dt)

    def simulate_to_time(self, endtime, **kw):
        if not self.functional:
            return self.o.simulate_to_time(endtime, **kw)
        n = 0
        while self.o.t < endtime:
            dt = self.perform_step(endtime - self.o.t)
            self.o.t = self.o.t + dt
            n += 1
        return n

    def __getattr__(self, name):
        return getattr(self.o, name)


def oracle_from(sc: S.Scenario, real_bytes: int = 8):
    """An oracle simulation with the scenario's grid, terrain, sources, friction, BC and stepper."""
    return OracleRun(sc, real_bytes)


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
