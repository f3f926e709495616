"""Seeded scenario builders for the measured and parity-tested workloads.

  circular_dam_break   2D circular dam break on [0,1]^2, flat bottom, RK2, CFL 0.2
                       (w = 2 inside radius 0.15 around (0.5, 0.5), else 1).
  hills_wet_dry        square domain with Δ = 1 m, bottom = sum of seeded Gaussian
                       hills (amplitude U[0.5,4] m, width U[50,400] m) + 1e-3 * x,
                       w = max(1.5, B_cell) (dry islands), Manning-type friction
                       n = 0.03 (friction_bsa2012, Cz = n^2), rain 1e-5 m/s,
                       infiltration 2e-6 m/s, wall BCs, RK2, CFL 0.25.
  differentiation_case the gradient workload: n x n cells, Δ = 1 m, 16 seeded hills
                       (amplitude U[0.2,1] m, width U[50,200] m) + 1e-3 slope,
                       uniform initial depth 1 m, Manning n = 0.03 (bsa2012),
                       rain 2e-5 m/s, wall BCs, RK2, CFL 0.25; 32 seeded gauge
                       cells; the target comes from the same steps on the
                       terrain plus a seeded perturbation (8 hills of U[-0.1,0.1] m).
  ensemble_member      one flood scenario of the batched ensemble: square side
                       log-uniform in [64, 1024] cells with Δ = 1 m, 8-32 seeded
                       hills (amplitude U[0.5,4] m, width U[50,400] m, centres in
                       the domain) + 1e-3 * x, uniform initial depth U[0,2] m over
                       the terrain (w = B_cell + h0), rain U[0,5e-5] m/s,
                       Manning n U[0.01,0.08] (friction_bsa2012, Cz = n^2), wall
                       BCs, RK2, CFL 0.25, end time U[10,600] s (rounded to a
                       Float32 value, so Float32 time reaches it exactly), and
                       depth_cutoff = 8e-2 as the reference's terrain example
                       uses (examples/terrain.jl:92): with the default 1e-5, thin
                       draining layers on the hill flanks drive the CFL step
                       down to ~1e-5 s and a member needs millions of steps.

Random numbers come from splitmix64 so any language can regenerate them.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import api as vf

MASK64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea & Flood 2014): the state advances by the golden-ratio
    increment and each output is the state passed through a 64-bit finaliser."""

    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))


@dataclass
class Scenario:
    """Everything needed to build the same run in the library and in the oracle."""
    name: str
    nx: int
    ny: int
    extent: tuple
    B: np.ndarray | None            # corners (nx+5, ny+5), None for a flat zero bottom
    w0: np.ndarray                  # interior (nx, ny)
    hu0: np.ndarray
    hv0: np.ndarray
    cfl: float
    stepper: str = "rk2"            # "rk2" or "fe"
    rain_m_per_h: float | None = None
    infiltration_m_per_s: float | None = None
    manning_n: float | None = None
    theta: float = 1.2
    bottom_source: bool = False
    friction_law: str = "bsa2012"   # friction_bsa2012 / friction_fcg2016 / friction_bh2021
    eq: dict = field(default_factory=dict)  # ShallowWaterEquations keywords (rho, g, depth_cutoff, ...)
    bc: str = "wall"                # "wall", "periodic" or "neumann"
    reconstruction: str = "linear"  # "linear" or "none"
    sources: list | None = None     # explicit source-term objects (overrides the flags above)
    t0: float = 0.0
    meta: dict = field(default_factory=dict)

    def grid(self) -> vf.CartesianGrid:
        return vf.CartesianGrid(self.nx, self.ny, gc=2,
                                boundary={"periodic": vf.PeriodicBC(), "neumann": vf.NeumannBC()}.get(self.bc,
                                                                                                      vf.WallBC()),
                                extent=[list(self.extent[0]), list(self.extent[1])])

    def source_terms(self) -> list:
        if self.sources is not None:
            return list(self.sources)
        st = []
        if self.bottom_source:
            st.append(vf.SourceTermBottom())
        if self.rain_m_per_h is not None:
            st.append(vf.ConstantRain(self.rain_m_per_h))
        if self.infiltration_m_per_s is not None:
            st.append(vf.ConstantInfiltration(self.infiltration_m_per_s))
        return st

    def system(self, backend: vf.SM103Backend):
        """(ConservedSystem, time stepper, grid) of the scenario script."""
        grid = self.grid()
        bottom = vf.ConstantBottomTopography() if self.B is None else vf.BottomTopography2D(self.B, backend, grid)
        eq = vf.ShallowWaterEquations(bottom, **self.eq)
        friction = None
        if self.manning_n is not None:
            law = {"bsa2012": vf.friction_bsa2012, "fcg2016": vf.friction_fcg2016,
                   "bh2021": vf.friction_bh2021}[self.friction_law]
            friction = vf.ImplicitFriction(Cz=self.manning_n ** 2, friction_function=law)
        rec = vf.NoReconstruction() if self.reconstruction == "none" else vf.LinearReconstruction(self.theta)
        system = vf.ConservedSystem(backend, rec, vf.CentralUpwind(eq), eq, grid, self.source_terms(), friction)
        stepper = vf.RungeKutta2() if self.stepper == "rk2" else vf.ForwardEulerStepper()
        return system, stepper, grid

    def config(self, backend: vf.SM103Backend):
        """The C-ABI configuration of the scenario (no device work)."""
        system, stepper, grid = self.system(backend)
        return vf.system_config(backend, system, stepper, grid, self.cfl)

    def build(self, backend: vf.SM103Backend) -> vf.Simulator:
        """The scenario script, written against the reference's API."""
        system, stepper, grid = self.system(backend)
        sim = vf.Simulator(backend, system, stepper, grid, cfl=self.cfl, t0=self.t0)
        vf.set_current_state(sim, (self.w0, self.hu0, self.hv0))
        return sim


def circular_dam_break(n: int = 256, radius: float = 0.15, cfl: float = 0.2) -> Scenario:
    grid = vf.CartesianGrid(n, n, gc=2, boundary=vf.WallBC())
    c = vf.cell_centers(grid)
    r = np.sqrt((c[:, :, 0] - 0.5) ** 2 + (c[:, :, 1] - 0.5) ** 2)
    w0 = np.where(r < radius, 2.0, 1.0)
    z = np.zeros_like(w0)
    return Scenario(name=f"circular_dam_break_{n}", nx=n, ny=n, extent=((0.0, 1.0), (0.0, 1.0)), B=None, w0=w0,
                    hu0=z, hv0=z.copy(), cfl=cfl)


_LN2_HI = float.fromhex("0x1.62e42fee00000p-1")  # ln 2 to 32 bits: kd * _LN2_HI is exact for |kd| < 2^20
_LN2_LO = float.fromhex("0x1.a39ef35793c76p-33")  # ln 2 - _LN2_HI
_INV_FACT = [1.0]
for _n in range(1, 15):
    _INV_FACT.append(_INV_FACT[-1] / _n)


def det_exp(x: np.ndarray) -> np.ndarray:
    """exp(x) for x <= 0 from IEEE +, -, *, / and exact scaling only, so the same
    bits come out on every machine (numpy's exp is not correctly rounded and its
    SIMD variants differ between x86 and Arm in the last bit). Cody-Waite
    reduction x = k ln 2 + r with |r| <= ln 2 / 2 and a two-part ln 2, then the
    Taylor series of exp(r) to degree 14 in Horner form, then ldexp by k; within
    a few ulp of exp."""
    x = np.asarray(x, dtype=np.float64)
    kd = np.rint(x * 1.4426950408889634)  # nearest double to 1/ln 2
    kd = np.maximum(kd, -1100.0)
    r = (x - kd * _LN2_HI) - kd * _LN2_LO
    q = np.full_like(r, _INV_FACT[14])
    for n in range(13, -1, -1):
        q = q * r + _INV_FACT[n]
    out = np.ldexp(q, kd.astype(np.int64))
    return np.where(x < -745.0, 0.0, out)


def hill_bottom(nx: int, ny: int, extent, n_hills: int, seed: int, slope: float = 1e-3,
                amp=(0.5, 4.0), width=(50.0, 400.0)) -> np.ndarray:
    """Corner bottom (nx+5, ny+5): slope * x plus n_hills Gaussian hills
    a * exp(-(x-cx)^2 / (2 s^2)) * exp(-(y-cy)^2 / (2 s^2)), centres uniform in the
    domain, a ~ U[amp], s ~ U[width], drawn from splitmix64(seed). Each hill is
    the outer product of two 1D Gaussians evaluated with det_exp, so the terrain
    is bit-for-bit the same on every machine."""
    grid = vf.CartesianGrid(nx, ny, gc=2, boundary=vf.WallBC(), extent=[list(extent[0]), list(extent[1])])
    xv = vf.cell_faces(grid, 1, interior=False)
    yv = vf.cell_faces(grid, 2, interior=False)
    rng = SplitMix64(seed)
    (x0, x1), (y0, y1) = extent
    B = slope * np.broadcast_to(xv[:, None], (xv.size, yv.size))
    for _ in range(n_hills):
        cx = rng.uniform(x0, x1)
        cy = rng.uniform(y0, y1)
        a = rng.uniform(*amp)
        s = rng.uniform(*width)
        two_s2 = 2.0 * s * s
        ex = det_exp(-((xv - cx) * (xv - cx)) / two_s2)
        ey = det_exp(-((yv - cy) * (yv - cy)) / two_s2)
        B = B + (a * ex)[:, None] * ey[None, :]
    return B


def hills_wet_dry(n: int = 4096, seed: int = 20240901, n_hills: int = 64, w_init: float = 1.5,
                  cfl: float = 0.25, length: float | None = None) -> Scenario:
    L = float(n) if length is None else float(length)
    extent = ((0.0, L), (0.0, L))
    scale = L / 4096.0
    B = hill_bottom(n, n, extent, n_hills, seed, amp=(0.5, 4.0), width=(50.0 * scale, 400.0 * scale))
    Bc = 0.25 * (B[:-1, :-1] + B[1:, :-1] + B[:-1, 1:] + B[1:, 1:])[2:-2, 2:-2]
    w0 = np.maximum(w_init, Bc)
    z = np.zeros_like(w0)
    return Scenario(name=f"hills_wet_dry_{n}", nx=n, ny=n, extent=extent, B=B, w0=w0, hu0=z, hv0=z.copy(), cfl=cfl,
                    rain_m_per_h=1e-5 * 3600, infiltration_m_per_s=2e-6, manning_n=0.03, bottom_source=True,
                    meta={"seed": seed, "n_hills": n_hills})


ENSEMBLE_DEPTH_CUTOFF = 8e-2  # examples/terrain.jl:92


@dataclass
class EnsembleSpec:
    """Draws of one ensemble member (everything but the arrays)."""
    index: int
    seed: int
    side: int
    n_hills: int
    rain_m_per_s: float
    manning_n: float
    h0: float
    endtime: float


def ensemble_specs(count: int = 256, seed: int = 20241203, side_range=(64, 1024)) -> list[EnsembleSpec]:
    """The seeded draws of `count` ensemble members (one splitmix64 stream)."""
    rng = SplitMix64(seed)
    lo, hi = np.log(side_range[0]), np.log(side_range[1])
    out = []
    for i in range(count):
        side = int(round(float(np.exp(rng.uniform(lo, hi)))))
        side = min(max(side, side_range[0]), side_range[1])
        n_hills = 8 + min(24, int(rng.uniform(0.0, 25.0)))
        rain = rng.uniform(0.0, 5e-5)
        n = rng.uniform(0.01, 0.08)
        h0 = rng.uniform(0.0, 2.0)
        endtime = float(np.float32(rng.uniform(10.0, 600.0)))
        out.append(EnsembleSpec(i, rng.next_u64(), side, n_hills, rain, n, h0, endtime))
    return out


def ensemble_member(spec: EnsembleSpec) -> Scenario:
    n = spec.side
    L = float(n)
    extent = ((0.0, L), (0.0, L))
    B = hill_bottom(n, n, extent, spec.n_hills, spec.seed, amp=(0.5, 4.0), width=(50.0, 400.0))
    Bc = 0.25 * (B[:-1, :-1] + B[1:, :-1] + B[:-1, 1:] + B[1:, 1:])[2:-2, 2:-2]
    w0 = Bc + spec.h0
    z = np.zeros_like(w0)
    return Scenario(name=f"ensemble_{spec.index}_{n}", nx=n, ny=n, extent=extent, B=B, w0=w0, hu0=z, hv0=z.copy(),
                    cfl=0.25, rain_m_per_h=spec.rain_m_per_s * 3600, manning_n=spec.manning_n, bottom_source=True,
                    eq={"depth_cutoff": ENSEMBLE_DEPTH_CUTOFF},
                    meta={"seed": spec.seed, "n_hills": spec.n_hills, "endtime": spec.endtime, "h0": spec.h0})


@dataclass
class ServingSpec:
    spec: EnsembleSpec
    real: str  # "f32" or "f64"


def serving_specs(count: int = 48, seed: int = 20241204, side_range=(128, 2048),
                  endtime_range=(2.0, 20.0)) -> list[ServingSpec]:
    """Requests of the serving workload: ensemble members with sides
    log-uniform in side_range, Float32 or Float64 with probability 1/2 each, end
    times uniform in endtime_range (rounded to Float32 values)."""
    rng = SplitMix64(seed ^ 0x5EC0)
    base = ensemble_specs(count, seed=seed, side_range=side_range)
    out = []
    for sp in base:
        sp.endtime = float(np.float32(rng.uniform(*endtime_range)))
        out.append(ServingSpec(sp, "f32" if rng.uniform() < 0.5 else "f64"))
    return out


@dataclass
class DiffCase:
    scenario: Scenario
    gauges: np.ndarray        # (32, 2) interior cell indices [i, j]
    B_target: np.ndarray      # perturbed corners, the target run's terrain


def differentiation_case(n: int = 512, seed: int = 20241205, n_gauges: int = 32, depth: float = 1.0) -> DiffCase:
    L = float(n)
    extent = ((0.0, L), (0.0, L))
    B = hill_bottom(n, n, extent, 16, seed, amp=(0.2, 1.0), width=(50.0, 200.0))
    pert = hill_bottom(n, n, extent, 8, seed + 1, slope=0.0, amp=(-0.1, 0.1), width=(30.0, 120.0))
    Bc = 0.25 * (B[:-1, :-1] + B[1:, :-1] + B[:-1, 1:] + B[1:, 1:])[2:-2, 2:-2]
    w0 = Bc + depth
    z = np.zeros_like(w0)
    rng = SplitMix64(seed + 2)
    gauges = np.array([[int(rng.uniform(0, n)), int(rng.uniform(0, n))] for _ in range(n_gauges)], dtype=np.int32)
    sc = Scenario(name=f"diff_{n}", nx=n, ny=n, extent=extent, B=B, w0=w0, hu0=z, hv0=z.copy(), cfl=0.25,
                  rain_m_per_h=2e-5 * 3600, manning_n=0.03, bottom_source=True, meta={"seed": seed})
    return DiffCase(sc, np.minimum(gauges, n - 1), B + pert)
