"""Host-side mirror of VolumeFluxes.jl's scenario API for the sm_103a backend.

Object names, constructor keywords, defaults and error behaviour follow the
reference (paths below are within the VolumeFluxes.jl project); Julia's
mutating `f!` functions are spelled `f` here. A scenario script written
against the reference -- CartesianGrid, ShallowWaterEquations,
BottomTopography2D, LinearReconstruction, CentralUpwind, source terms,
ImplicitFriction, ConservedSystem, RungeKutta2, Simulator, simulate_to_time,
callbacks -- runs unchanged except that it passes `SM103Backend()` where it
passed `make_cpu_backend()` / `make_cuda_backend()`.

Every step runs in libvfsm103.so on the GPU. Configurations the CUDA path does
not implement raise `ArgumentError` when the Simulator is built; nothing falls
back to a CPU implementation.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Any, Callable, Iterable, Sequence

import numpy as np

from . import _native as N


class ArgumentError(ValueError):
    """Julia's ArgumentError: a configuration this backend cannot run."""


class DomainError(ValueError):
    """Julia's DomainError: an array of the wrong shape (src/bottom_topography.jl:78-82)."""


XDIR = 1
YDIR = 2


# --------------------------------------------------------------------------- grid
class BoundaryCondition:
    pass


class PeriodicBC(BoundaryCondition):
    """src/grid.jl:21-22 (periodic ghost update src/bc.jl:29-40; not on the sm_103a path)."""


class WallBC(BoundaryCondition):
    """src/grid.jl:24-25; reflective wall, src/bc.jl:81-110."""


class NeumannBC(BoundaryCondition):
    """src/grid.jl:27-28 (src/bc.jl:49-60; not on the sm_103a path)."""


class CartesianGrid:
    """CartesianGrid(nx, ny; gc=1, boundary=PeriodicBC(), extent=[0 1; 0 1]), src/grid.jl:82-90.

    The defaults are the reference's; the sm_103a Simulator needs gc=2 and WallBC().
    """

    def __init__(self, nx: int, ny: int | None = None, *, gc: int = 1, boundary: BoundaryCondition | None = None,
                 extent=None):
        if ny is None:
            raise ArgumentError("only 2D CartesianGrid(nx, ny) is supported by the sm_103a backend")
        self.nx, self.ny = int(nx), int(ny)
        self.gc = int(gc)
        self.boundary = PeriodicBC() if boundary is None else boundary
        ext = np.array([[0.0, 1.0], [0.0, 1.0]] if extent is None else extent, dtype=np.float64)
        if ext.shape != (2, 2):
            raise ArgumentError("extent must be [[x0, x1], [y0, y1]]")
        self.extent = ext
        self.ghostcells = (self.gc, self.gc)
        self.totalcells = (self.nx + 2 * self.gc, self.ny + 2 * self.gc)
        self.delta = ((ext[0, 1] - ext[0, 0]) / self.nx, (ext[1, 1] - ext[1, 0]) / self.ny)

    def size(self) -> tuple[int, int]:
        return self.totalcells

    def interior_size(self) -> tuple[int, int]:
        return (self.nx, self.ny)

    def __repr__(self):
        return (f"CartesianGrid({self.nx}, {self.ny}; gc={self.gc}, boundary={type(self.boundary).__name__}(), "
                f"extent={self.extent.tolist()})")


def compute_dx(grid: CartesianGrid, direction: int = XDIR) -> float:
    """src/grid.jl:163-164."""
    return grid.delta[direction - 1]


def compute_dy(grid: CartesianGrid) -> float:
    return grid.delta[1]


def _linrange(a: float, b: float, n: int) -> np.ndarray:
    # Julia's LinRange element k (0-based) is (1 - t)*a + t*b with t = k/(n-1).
    k = np.arange(n, dtype=np.float64)
    t = k / (n - 1)
    return (1 - t) * a + t * b


def cell_faces(grid: CartesianGrid, direction: int | None = None, interior: bool = True) -> np.ndarray:
    """Face coordinates, src/grid.jl:103-135.

    With a direction: the 1D face coordinates along it. Without: an array of
    shape (Nx+1, Ny+1, 2) of (x, y) face intersections.
    """
    def faces(d):
        x0, x1 = grid.extent[d - 1]
        if interior:
            n = (grid.nx, grid.ny)[d - 1]
            return _linrange(x0, x1, n + 1)
        dx = compute_dx(grid, d)
        gcd = grid.ghostcells[d - 1]
        return _linrange(x0 - gcd * dx, x1 + gcd * dx, grid.totalcells[d - 1] + 1)

    if direction is not None:
        return faces(direction)
    xf, yf = faces(XDIR), faces(YDIR)
    out = np.empty((xf.size, yf.size, 2))
    out[:, :, 0] = xf[:, None]
    out[:, :, 1] = yf[None, :]
    return out


def cell_centers(grid: CartesianGrid, direction: int | None = None, interior: bool = True) -> np.ndarray:
    """Cell centres, src/grid.jl:151-161: face intersection + (dx, dy)/2, shape
    (nx, ny, 2). With a direction (src/grid.jl:145-149): the 1D centres along
    it, faces[:-1] + (faces[1] - faces[0])/2."""
    if direction is not None:
        f1 = cell_faces(grid, direction, interior=interior)
        return f1[:-1] + (f1[1] - f1[0]) / 2.0
    f = cell_faces(grid, interior=interior)
    c = f[:-1, :-1, :].copy()
    c[:, :, 0] += compute_dx(grid) / 2
    c[:, :, 1] += compute_dy(grid) / 2
    return c


def cell_center(grid: CartesianGrid, I: tuple[int, int]) -> tuple[float, float]:
    """src/grid.jl:117-121 (1-based total-grid index)."""
    x = grid.extent[0, 0] + compute_dx(grid) * (I[0] - 0.5 - grid.ghostcells[0])
    y = grid.extent[1, 0] + compute_dy(grid) * (I[1] - 0.5 - grid.ghostcells[1])
    return (x, y)


# --------------------------------------------------------------------------- bottom
class ConstantBottomTopography:
    """ConstantBottomTopography(B=0.0), src/bottom_topography.jl:24-27."""

    def __init__(self, B: float = 0.0):
        self.B = float(B)


class BottomTopography2D:
    """BottomTopography2D(B, backend, grid), src/bottom_topography.jl:51-57.

    B holds bottom elevations at cell corners, shape size(grid) .+ 1, indexed B[i, j].
    """

    def __init__(self, B, backend=None, grid: CartesianGrid | None = None):
        B = np.asarray(B, dtype=np.float64)
        if grid is not None:
            expected = (grid.totalcells[0] + 1, grid.totalcells[1] + 1)
            if B.shape != expected:
                raise DomainError(f"Bottom topography should be of size {expected} but got {B.shape}")
        self.B = B


def is_zero(bottom) -> bool:
    """src/bottom_topography.jl:84."""
    return bool(np.all(np.asarray(bottom.B) == 0.0))


def B_cell(bottom, i: int, j: int) -> float:
    """Host lookup, src/bottom_topography.jl:87,97 (1-based total-grid indices)."""
    if isinstance(bottom, ConstantBottomTopography):
        return bottom.B
    B = bottom.B
    return 0.25 * (B[i - 1, j - 1] + B[i, j - 1] + B[i - 1, j] + B[i, j])


def B_face_left(bottom, i: int, j: int, direction: int) -> float:
    """src/bottom_topography.jl:88,98,100."""
    if isinstance(bottom, ConstantBottomTopography):
        return bottom.B
    B = bottom.B
    if direction == XDIR:
        return 0.5 * (B[i - 1, j - 1] + B[i - 1, j])
    return 0.5 * (B[i - 1, j - 1] + B[i, j - 1])


def B_face_right(bottom, i: int, j: int, direction: int) -> float:
    """src/bottom_topography.jl:89,99,101."""
    if isinstance(bottom, ConstantBottomTopography):
        return bottom.B
    B = bottom.B
    if direction == XDIR:
        return 0.5 * (B[i, j - 1] + B[i, j])
    return 0.5 * (B[i - 1, j] + B[i, j])


def collect_topography_cells(bottom, grid: CartesianGrid, interior: bool = True) -> np.ndarray:
    """Cell-averaged bottom, src/bottom_topography.jl:111-146."""
    if isinstance(bottom, ConstantBottomTopography):
        dims = grid.interior_size() if interior else grid.size()
        return np.ones(dims) * bottom.B
    B = bottom.B
    by = 0.5 * (B[:-1, :] + B[1:, :])
    cells = 0.5 * (by[:, :-1] + by[:, 1:])
    if interior:
        g = grid.gc
        return cells[g:-g, g:-g]
    return cells


# --------------------------------------------------------------------------- equations
class ShallowWaterEquations:
    """ShallowWaterEquations(B; ρ=1, g=9.81, depth_cutoff=1e-5, desingularizing_kappa=1e-5),
    src/equations/swe_2D.jl:22-29. Conserved variables (:h, :hu, :hv), where :h holds w."""

    def __init__(self, B=None, *, rho: float = 1.0, g: float = 9.81, depth_cutoff: float = 1e-5,
                 desingularizing_kappa: float = 1e-5, **kw):
        rho = kw.pop("ρ", rho)
        if kw:
            raise TypeError(f"unexpected keywords {sorted(kw)}")
        self.B = ConstantBottomTopography() if B is None else B
        self.rho, self.g = float(rho), float(g)
        self.depth_cutoff = float(depth_cutoff)
        self.desingularizing_kappa = float(desingularizing_kappa)


conserved_variable_names = ("h", "hu", "hv")


def desingularize(eq: ShallowWaterEquations, h: float) -> float:
    """Host restatement of src/equations/equation.jl:40-62 for scalar checks."""
    k = eq.desingularizing_kappa
    return math.copysign(1.0, h) * max(abs(h), min(h * h / (2 * k) + k / 2.0, k))


class Reconstruction:
    pass


class LinearReconstruction(Reconstruction):
    """LinearReconstruction(theta=1.2), src/reconstruction/linearreconstruction.jl:22-25."""

    def __init__(self, theta: float = 1.2):
        self.theta = float(theta)


class NoReconstruction(Reconstruction):
    """src/reconstruction/noreconstruction.jl:21 (not on the sm_103a path)."""


def minmod(a, b, c):
    """src/reconstruction/linearreconstruction.jl:28-35 (host, elementwise on arrays)."""
    a, b, c = np.broadcast_arrays(np.asarray(a), np.asarray(b), np.asarray(c))
    pos = (a > 0) & (b > 0) & (c > 0)
    neg = (a < 0) & (b < 0) & (c < 0)
    out = np.where(pos, np.minimum(np.minimum(a, b), c), 0)
    out = np.where(neg, np.maximum(np.maximum(a, b), c), out)
    return out if out.ndim else out.item()


class NumericalFlux:
    pass


class CentralUpwind(NumericalFlux):
    """CentralUpwind(eq), src/numericalflux/swe/centralupwind.jl:21-23."""

    def __init__(self, eq):
        self.eq = eq


# --------------------------------------------------------------------------- sources
class SourceTerm:
    pass


class SourceTermBottom(SourceTerm):
    """src/abstract_types.jl:36; evaluation src/sourceterms/source_term_bottom.jl:24-41."""


class SourceTermRain(SourceTerm):
    pass


class SourceTermInfiltration(SourceTerm):
    pass


class ConstantRain(SourceTermRain):
    """ConstantRain(rain_rate) with the rate in m/h, src/sourceterms/source_term_rain.jl:24-30."""

    def __init__(self, rain_rate: float):
        self.rain_rate = float(rain_rate)


class ConstantInfiltration(SourceTermInfiltration):
    """ConstantInfiltration(infiltration_rate) in m/s, src/sourceterms/source_term_infiltration.jl:73-81."""

    def __init__(self, infiltration_rate: float):
        self.infiltration_rate = float(infiltration_rate)


class TimeDependentRain(SourceTermRain):
    """TimeDependentRain(rain_rates, time=[0.0]) with rates in m/h, src/sourceterms/source_term_rain.jl:32-41."""

    def __init__(self, rain_rates, time=(0.0,)):
        rates = np.asarray(rain_rates, dtype=np.float64).reshape(-1)
        times = np.asarray(time, dtype=np.float64).reshape(-1)
        if rates.shape != times.shape:
            raise DomainError("Dimensions of input parameters rain_rates and time does not match")
        self.rain_rates, self.time = rates, times


class FunctionalRain(SourceTermRain):
    """FunctionalRain(rain_function, grid): rain_function(t, x, y) in m/s at cell centres,
    src/sourceterms/source_term_rain.jl:57-68. The host evaluates it over the grid at the
    step's start time and uploads the field (the closure cannot cross the C ABI)."""

    def __init__(self, rain_function: Callable, grid: CartesianGrid):
        self.rain_function = rain_function
        self.grid = grid

    def field(self, t: float) -> np.ndarray:
        g = self.grid
        I = np.arange(1, g.totalcells[0] + 1, dtype=np.float64)
        J = np.arange(1, g.totalcells[1] + 1, dtype=np.float64)
        x = g.extent[0, 0] + compute_dx(g) * (I - 0.5 - g.ghostcells[0])
        y = g.extent[1, 0] + compute_dy(g) * (J - 0.5 - g.ghostcells[1])
        X, Y = np.meshgrid(x, y, indexing="ij")
        try:
            f = np.asarray(self.rain_function(t, X, Y), dtype=np.float64)
            if f.shape != X.shape:
                f = np.broadcast_to(f, X.shape)
        except Exception:
            f = np.vectorize(lambda a, b: float(self.rain_function(t, a, b)))(X, Y)
        return np.ascontiguousarray(f, dtype=np.float64)


class HortonInfiltration(SourceTermInfiltration):
    """HortonInfiltration(grid, backend; factor=1.0, fc=3.272e-5, f0=1.977e-4, k=2.43e-3),
    src/sourceterms/source_term_infiltration.jl:21-47: f(t) = factor*(fc + (f0 - fc)*exp(-k*t))."""

    def __init__(self, grid: CartesianGrid, backend=None, *, factor=1.0, fc: float = 3.272e-5, f0: float = 1.977e-4,
                 k: float = 2.43e-3):
        fa = np.asarray(factor, dtype=np.float64)
        if fa.ndim == 0:
            fa = np.full(grid.size(), float(fa))
        elif fa.shape != grid.size():
            raise DomainError(f"Infiltration factor should be of size {grid.size()} but got {fa.shape}")
        self.factor, self.fc, self.f0, self.k = fa, float(fc), float(f0), float(k)


def compute_rain(rain, t=None, index=None):
    """src/sourceterms/source_term_rain.jl:30,45-54,65-68 (host evaluation)."""
    if isinstance(rain, TimeDependentRain):
        idx = 0
        while idx + 1 < rain.time.size and not (t < rain.time[idx + 1]):
            idx += 1
        return rain.rain_rates[idx] / 3600
    if isinstance(rain, FunctionalRain):
        x, y = cell_center(rain.grid, index)
        return rain.rain_function(t, x, y)
    return rain.rain_rate / 3600


def compute_infiltration(infiltration, t=None, index=None):
    """src/sourceterms/source_term_infiltration.jl:68-81 (host evaluation; index is 1-based)."""
    if isinstance(infiltration, HortonInfiltration):
        f = infiltration
        return f.factor[index[0] - 1, index[1] - 1] * (f.fc + (f.f0 - f.fc) * math.exp(-f.k * t))
    return infiltration.infiltration_rate


# --------------------------------------------------------------------------- friction
def friction_bsa2012(c, h, speed):
    """src/friction.jl:30-33 (Manning form: -c*|u| / (h^(1/3)*h))."""
    return -c * speed / (np.cbrt(h) * h)


def friction_fcg2016(c, h, speed):
    """src/friction.jl:35-38."""
    return -c * speed / (np.cbrt(h) * h * h)


def friction_bh2021(c, h, speed):
    """src/friction.jl:40-43."""
    return -c * speed / (h * h)


_FRICTION_CODES = {
    friction_bsa2012: N.VF_FRICTION_BSA2012,
    friction_fcg2016: N.VF_FRICTION_FCG2016,
    friction_bh2021: N.VF_FRICTION_BH2021,
}


class ImplicitFriction:
    """ImplicitFriction(; Cz=0.03^2, friction_function=friction_bh2021), src/friction.jl:23-27."""

    def __init__(self, *, Cz: float = 0.03 ** 2, friction_function: Callable = friction_bh2021):
        self.Cz = float(Cz)
        self.friction_function = friction_function


# --------------------------------------------------------------------------- steppers
class TimeStepper:
    pass


class RungeKutta2(TimeStepper):
    """src/timestepper/rungekutta.jl:21-24."""


class ForwardEulerStepper(TimeStepper):
    """src/timestepper/forwardeuler.jl:23-26."""


def number_of_substeps(stepper: TimeStepper) -> int:
    return 2 if isinstance(stepper, RungeKutta2) else 1


# --------------------------------------------------------------------------- backend
class SM103Backend:
    """The GB300 backend: every step runs in libvfsm103.so (hand-written sm_103a kernels).

    Stands beside KernelAbstractionBackend (src/backends/kernel_abstractions.jl:29-40);
    `realtype` is np.float64 or np.float32, `device` a CUDA ordinal.
    `arithmetic` (Float64 only): "reference" rounds every operation as the
    reference does (results equal its CPU path bit for bit); "faithful" uses
    faithful quotients and fused multiply-adds in the per-step kernels, held
    to 1e-12 relative max-norm against the reference path instead of to its
    bits.
    """

    def __init__(self, realtype=np.float64, device: int = 0, arithmetic: str = "reference"):
        rt = np.dtype(realtype)
        if rt not in (np.dtype(np.float64), np.dtype(np.float32)):
            raise ArgumentError("realtype must be float64 or float32")
        if arithmetic not in ("reference", "faithful"):
            raise ArgumentError("arithmetic must be 'reference' or 'faithful'")
        if arithmetic == "faithful" and rt != np.dtype(np.float64):
            raise ArgumentError("faithful arithmetic is a Float64 mode")
        self.realtype = rt.type
        self.device = int(device)
        self.arithmetic = arithmetic


def name(backend) -> str:
    return "SM103" if isinstance(backend, SM103Backend) else type(backend).__name__


def get_available_backends() -> list:
    """The sm_103a backend only: there is no CPU backend in this package."""
    return [SM103Backend()]


def convert_to_backend(backend, array):
    """src/backends/buffer.jl:23-25: arrays stay host arrays until a Simulator uploads them."""
    return np.asarray(array)


# --------------------------------------------------------------------------- system
class System:
    pass


class ConservedSystem(System):
    """ConservedSystem(backend, reconstruction, numericalflux, equation, grid, source_terms, implicit_source_term),
    src/system.jl:24-58. Validates like the reference (is_compatible, src/system.jl:81-83 and
    src/equations/equation.jl:74-84)."""

    def __init__(self, backend, reconstruction, numericalflux, equation, grid, source_terms=None,
                 implicit_source_term=None):
        if source_terms is None:
            source_terms = []
        elif isinstance(source_terms, SourceTerm):
            source_terms = [source_terms]
        self.backend = backend
        self.reconstruction = reconstruction
        self.numericalflux = numericalflux
        self.equation = equation
        self.grid = grid
        self.source_terms = list(source_terms)
        self.implicit_source_term = implicit_source_term
        if isinstance(equation.B, BottomTopography2D):
            expected = (grid.totalcells[0] + 1, grid.totalcells[1] + 1)
            if equation.B.B.shape != expected:
                raise DomainError(f"Bottom topography should be of size {expected} but got {equation.B.B.shape}")
        if not is_zero(equation.B) and not any(type(s) is SourceTermBottom for s in self.source_terms):
            raise ArgumentError("Found non-zero bottom topography in equation, but no corresponding source term. "
                                "Did you forget to add a source term to your system?")


# --------------------------------------------------------------------------- state views
@dataclass
class StateView:
    """Planes of one state as (nx, ny) numpy arrays indexed [i, j] (x first)."""
    h: np.ndarray
    hu: np.ndarray
    hv: np.ndarray

    def __getitem__(self, k):
        return (self.h, self.hu, self.hv)[k]

    def stack(self) -> np.ndarray:
        return np.stack([self.h, self.hu, self.hv], axis=-1)


def _to_planes(new_state, nx: int, ny: int, dtype) -> list[np.ndarray]:
    if isinstance(new_state, StateView):
        planes = [new_state.h, new_state.hu, new_state.hv]
    elif isinstance(new_state, dict):
        planes = [new_state["h"], new_state["hu"], new_state["hv"]]
    elif isinstance(new_state, (list, tuple)) and len(new_state) == 3:
        planes = list(new_state)
    else:
        a = np.asarray(new_state)
        if a.shape != (nx, ny, 3):
            raise DomainError(f"state must have shape ({nx}, {ny}, 3) or be three ({nx}, {ny}) planes; got {a.shape}")
        planes = [a[:, :, 0], a[:, :, 1], a[:, :, 2]]
    out = []
    for p in planes:
        p = np.asarray(p, dtype=dtype)
        if p.shape != (nx, ny):
            raise DomainError(f"state planes must have shape ({nx}, {ny}); got {p.shape}")
        out.append(np.ascontiguousarray(p.T))  # x fastest, as the reference's column-major arrays
    return out


# --------------------------------------------------------------------------- simulator
def system_config(backend, system: "ConservedSystem", timestepper, grid: CartesianGrid, cfl: float) -> N.VfConfig:
    """The C-ABI configuration of a ConservedSystem + Simulator (no device work)."""
    s, g = system, grid
    eq = s.equation
    if not isinstance(eq, ShallowWaterEquations):
        raise ArgumentError("the sm_103a backend runs ShallowWaterEquations (2D practical SWE) only")
    if not isinstance(s.reconstruction, (LinearReconstruction, NoReconstruction)):
        raise ArgumentError(f"{type(s.reconstruction).__name__} is not implemented on the sm_103a backend")
    if not isinstance(s.numericalflux, CentralUpwind):
        raise ArgumentError(f"{type(s.numericalflux).__name__} is not implemented on the sm_103a backend")
    if not isinstance(g.boundary, (WallBC, PeriodicBC, NeumannBC)):
        raise ArgumentError(f"{type(g.boundary).__name__} is not implemented on the sm_103a backend")
    if g.gc != 2:
        raise ArgumentError("the sm_103a backend needs CartesianGrid(...; gc=2)")
    if isinstance(timestepper, RungeKutta2):
        stepper = N.VF_STEPPER_RK2
    elif isinstance(timestepper, ForwardEulerStepper):
        stepper = N.VF_STEPPER_FE
    else:
        raise ArgumentError(f"{type(timestepper).__name__} is not implemented on the sm_103a backend")
    cfg = N.VfConfig()
    cfg.abi_version = N.VF_ABI_VERSION
    cfg.nx, cfg.ny, cfg.gc = g.nx, g.ny, g.gc
    for i, v in enumerate(g.extent.reshape(-1)):
        cfg.extent[i] = float(v)
    cfg.real_bytes = np.dtype(backend.realtype).itemsize
    cfg.g, cfg.rho = eq.g, eq.rho
    cfg.depth_cutoff, cfg.desingularizing_kappa = eq.depth_cutoff, eq.desingularizing_kappa
    if isinstance(s.reconstruction, NoReconstruction):
        cfg.reconstruction, cfg.theta = N.VF_REC_NONE, 0.0
    else:
        cfg.reconstruction, cfg.theta = N.VF_REC_LINEAR, s.reconstruction.theta
    if len(s.source_terms) > N.VF_MAX_SOURCES:
        raise ArgumentError("too many source terms")
    for i, st in enumerate(s.source_terms):
        if type(st) is SourceTermBottom:
            cfg.source_kind[i], cfg.source_rate[i] = N.VF_SRC_BOTTOM, 0.0
        elif isinstance(st, ConstantRain):
            cfg.source_kind[i], cfg.source_rate[i] = N.VF_SRC_CONST_RAIN, st.rain_rate
        elif isinstance(st, ConstantInfiltration):
            cfg.source_kind[i], cfg.source_rate[i] = N.VF_SRC_CONST_INFIL, st.infiltration_rate
        elif isinstance(st, TimeDependentRain):
            cfg.source_kind[i] = N.VF_SRC_TIME_RAIN
        elif isinstance(st, HortonInfiltration):
            cfg.source_kind[i], cfg.source_rate[i] = N.VF_SRC_HORTON, st.fc
            cfg.source_aux[i][0], cfg.source_aux[i][1] = st.f0, st.k
        elif isinstance(st, FunctionalRain):
            cfg.source_kind[i] = N.VF_SRC_RAIN_FIELD
        else:
            raise ArgumentError(f"{type(st).__name__} is not implemented on the sm_103a backend")
    cfg.n_sources = len(s.source_terms)
    fr = s.implicit_source_term
    if fr is None:
        cfg.friction, cfg.friction_Cz = N.VF_FRICTION_NONE, 0.0
    elif isinstance(fr, ImplicitFriction):
        if fr.friction_function not in _FRICTION_CODES:
            raise ArgumentError("ImplicitFriction needs friction_bsa2012, friction_fcg2016 or friction_bh2021")
        cfg.friction, cfg.friction_Cz = _FRICTION_CODES[fr.friction_function], fr.Cz
    else:
        raise ArgumentError(f"{type(fr).__name__} is not implemented on the sm_103a backend")
    cfg.stepper = stepper
    cfg.bc = (N.VF_BC_PERIODIC if isinstance(g.boundary, PeriodicBC)
              else N.VF_BC_NEUMANN if isinstance(g.boundary, NeumannBC) else N.VF_BC_WALL)
    cfg.cfl = float(np.dtype(backend.realtype).type(cfl))
    if isinstance(eq.B, ConstantBottomTopography):
        cfg.bottom_is_constant, cfg.bottom_constant = 1, eq.B.B
    elif isinstance(eq.B, BottomTopography2D):
        cfg.bottom_is_constant, cfg.bottom_constant = 0, 0.0
    else:
        raise ArgumentError(f"{type(eq.B).__name__} is not supported")
    cfg.device = backend.device
    return cfg


class Simulator:
    """Simulator(backend, system, timestepper, grid; cfl=0.25, t0=0.0), src/simulator.jl:60-91.

    Creates the device-resident simulation in libvfsm103.so. Raises
    ArgumentError for any configuration outside the sm_103a path.
    """

    def __init__(self, backend, system: ConservedSystem, timestepper, grid: CartesianGrid, *, cfl: float = 0.25,
                 t0: float = 0.0):
        if not isinstance(backend, SM103Backend):
            raise ArgumentError("this package runs only SM103Backend simulations")
        self.backend = backend
        self.system = system
        self.timestepper = timestepper
        self.grid = grid
        self.dtype = np.dtype(backend.realtype)
        self.cfl = float(self.dtype.type(cfl))
        self.t = float(self.dtype.type(t0))
        self.current_timestep = 0.0
        self._h = None
        self._lib = N.load()
        cfg = self._config()
        h = C.c_void_p()
        N.check(self._lib, None, self._lib.vf_create(C.byref(cfg), C.byref(h)))
        self._h = h
        if getattr(backend, "arithmetic", "reference") == "faithful":
            N.check(self._lib, self._h, self._lib.vf_set_arithmetic(self._h, N.VF_ARITH_FAITHFUL))
        eqB = system.equation.B
        if isinstance(eqB, BottomTopography2D):
            B = np.ascontiguousarray(np.asarray(eqB.B, dtype=self.dtype).T)
            N.check(self._lib, self._h, self._lib.vf_upload_bottom(self._h, N.ptr(B)))
        self._functional = []
        for i, st in enumerate(system.source_terms):
            if isinstance(st, TimeDependentRain):
                t_, r_ = np.ascontiguousarray(st.time), np.ascontiguousarray(st.rain_rates)
                N.check(self._lib, self._h, self._lib.vf_set_source_table(self._h, i, N.ptr(t_), N.ptr(r_), t_.size))
            elif isinstance(st, HortonInfiltration):
                self._upload_field(i, st.factor)
            elif isinstance(st, FunctionalRain):
                self._functional.append((i, st))

    def _upload_field(self, index: int, field: np.ndarray):
        f = np.ascontiguousarray(np.asarray(field, dtype=self.dtype).T)  # x fastest
        N.check(self._lib, self._h, self._lib.vf_set_source_field(self._h, index, N.ptr(f)))

    def _refresh_functional(self):
        """Re-evaluate FunctionalRain at the step's start time (src/sourceterms/source_term_rain.jl:65-76)."""
        for i, st in self._functional:
            self._upload_field(i, st.field(self.t))

    def _config(self) -> N.VfConfig:
        return system_config(self.backend, self.system, self.timestepper, self.grid, self.cfl)

    # -- lifecycle
    def close(self):
        if self._h is not None and self._h.value:
            self._lib.vf_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise RuntimeError("simulator is closed")
        return self._h

    def launch_count(self) -> int:
        return int(self._lib.vf_launch_count(self.handle))


def set_current_state(simulator: Simulator, new_state) -> None:
    """set_current_state!(simulator, new_state), src/simulator.jl:119-139: interior upload + wall ghosts."""
    g = simulator.grid
    w, hu, hv = _to_planes(new_state, g.nx, g.ny, simulator.dtype)
    lib = simulator._lib
    N.check(lib, simulator.handle, lib.vf_set_interior_state(simulator.handle, N.ptr(w), N.ptr(hu), N.ptr(hv)))


def current_interior_state(simulator: Simulator, out: StateView | None = None) -> StateView:
    """collect(current_interior_state(simulator).h/.hu/.hv), src/simulator.jl:114-115.

    With `out`, the planes are written into its (nx, ny) arrays, which must be
    x-fastest (the transpose of a C-contiguous (ny, nx) array) of the backend's
    real type -- e.g. views of pinned host buffers."""
    g = simulator.grid
    if out is None:
        planes = [np.empty((g.ny, g.nx), dtype=simulator.dtype) for _ in range(3)]
        result = StateView(*(p.T for p in planes))
    else:
        planes = [a.T for a in (out.h, out.hu, out.hv)]
        for p in planes:
            if p.shape != (g.ny, g.nx) or p.dtype != simulator.dtype or not p.flags.c_contiguous:
                raise ArgumentError("out planes must be x-fastest (nx, ny) arrays of the backend's real type")
        result = out
    lib = simulator._lib
    N.check(lib, simulator.handle, lib.vf_get_interior_state(simulator.handle, *(N.ptr(p) for p in planes)))
    return result


def current_state(simulator: Simulator) -> StateView:
    """collect(current_state(simulator)) with ghost cells, planes of size(grid).

    Corner ghost cells are never written by the wall update or read by the
    scheme; they hold zeros here."""
    N1, N2 = simulator.grid.size()
    buf = np.empty(3 * N1 * N2, dtype=simulator.dtype)
    lib = simulator._lib
    N.check(lib, simulator.handle, lib.vf_download_state(simulator.handle, N.ptr(buf)))
    p = buf.reshape(3, N2, N1)
    return StateView(p[0].T, p[1].T, p[2].T)


def current_time(simulator: Simulator) -> float:
    return simulator.t


def current_timestep(simulator: Simulator) -> float:
    return simulator.current_timestep


def perform_step(simulator: Simulator, max_dt: float) -> None:
    """perform_step!(simulator, max_dt), src/simulator.jl:145-177 (does not advance t)."""
    dt = C.c_double()
    lib = simulator._lib
    if simulator._functional:
        simulator._refresh_functional()
    N.check(lib, simulator.handle, lib.vf_step(simulator.handle, float(max_dt), float(simulator.t), C.byref(dt)))
    simulator.current_timestep = dt.value


def water_volume(simulator: Simulator) -> float:
    """Float64 sum over interior cells of (w - B_cell) * dx * dy, computed on the device."""
    out = C.c_double()
    lib = simulator._lib
    N.check(lib, simulator.handle, lib.vf_water_volume(simulator.handle, C.byref(out)))
    return out.value


# --------------------------------------------------------------------------- callbacks
def sample_cells(simulator: Simulator, cells) -> StateView:
    """(w, hu, hv) at the given interior cells ((n, 2) array of 0-based [i, j])
    read on the device: a gauge read without collecting the whole interior."""
    g = np.ascontiguousarray(np.asarray(cells, dtype=np.int32).reshape(-1, 2))
    gi, gj = np.ascontiguousarray(g[:, 0]), np.ascontiguousarray(g[:, 1])
    out = [np.empty(len(g), dtype=simulator.dtype) for _ in range(3)]
    lib = simulator._lib
    N.check(lib, simulator.handle, lib.vf_sample_cells(simulator.handle, N.ptr(gi), N.ptr(gj), len(g), N.ptr(out[0]),
                                                       N.ptr(out[1]), N.ptr(out[2])))
    return StateView(*out)


class GaugeRecorder:
    """Callback recording (t, w at the gauges) with device-side reads; wrap it in
    an IntervalWriter to record at fixed intervals (src/callbacks.jl:40-55)."""

    def __init__(self, cells):
        self.cells = np.asarray(cells, dtype=np.int32).reshape(-1, 2)
        self.times: list[float] = []
        self.values: list[np.ndarray] = []

    def __call__(self, t, simulator):
        self.times.append(float(t))
        self.values.append(sample_cells(simulator, self.cells).h.copy())


class IntervalWriter:
    """IntervalWriter(step, writer), src/callbacks.jl:40-55: calls writer(t, simulator) when t + dt >= current_t."""

    def __init__(self, step: float = 1.0, writer: Callable | None = None, current_t: float = 0.0):
        if callable(step) and writer is None:
            step, writer = 1.0, step
        self.current_t = float(current_t)
        self.step = float(step)
        self.writer = writer

    def __call__(self, t, simulator):
        dt = current_timestep(simulator)
        if t + dt >= self.current_t:
            self.writer(t, simulator)
            self.current_t += self.step


class MultipleCallbacks:
    """src/callbacks.jl:74-82."""

    def __init__(self, callbacks: Iterable):
        self.callbacks = list(callbacks)

    def __call__(self, t, simulator):
        for c in self.callbacks:
            c(t, simulator)


def _interval_writers(callback) -> list[IntervalWriter] | None:
    if isinstance(callback, IntervalWriter):
        return [callback]
    if isinstance(callback, MultipleCallbacks) and all(isinstance(c, IntervalWriter) for c in callback.callbacks):
        return list(callback.callbacks)
    return None


def simulate_to_time(simulator: Simulator, endtime: float, *, match_endtime: bool = True, callback=None,
                     show_progress: bool = False, maximum_timestep: float | None = None) -> None:
    """simulate_to_time(simulator, endtime; match_endtime, callback, maximum_timestep), src/simulator.jl:179-212.

    Without a callback, or with IntervalWriter callbacks only, the time loop runs
    on the device and returns to the host only when a writer is due. Any other
    callback is called after every step, as in the reference.
    """
    if callback is not None and not callable(callback) and isinstance(callback, Iterable):
        callback = MultipleCallbacks(callback)
    lib = simulator._lib
    h = simulator.handle
    max_ts = -1.0 if maximum_timestep is None else float(maximum_timestep)
    writers = None if callback is None else _interval_writers(callback)
    if (callback is None or writers is not None) and not simulator._functional:
        while simulator.t < endtime:
            stop = min((w.current_t for w in writers), default=math.inf) if writers else math.inf
            t_out, steps, last_dt = C.c_double(), C.c_int64(), C.c_double()
            N.check(lib, h, lib.vf_simulate(h, simulator.t, float(endtime), int(match_endtime), max_ts, stop, 0,
                                            C.byref(t_out), C.byref(steps), C.byref(last_dt)))
            if steps.value == 0:
                break
            simulator.t = t_out.value
            simulator.current_timestep = last_dt.value
            if callback is not None:
                callback(simulator.t, simulator)
        return
    f32 = simulator.dtype == np.float32
    while simulator.t < endtime:
        max_dt = endtime - simulator.t if match_endtime else math.inf
        if maximum_timestep is not None:
            max_dt = min(max_dt, maximum_timestep)
        perform_step(simulator, max_dt)
        if f32:
            simulator.t = float(np.float32(simulator.t) + np.float32(simulator.current_timestep))
        else:
            simulator.t += simulator.current_timestep
        if callback is not None:
            callback(simulator.t, simulator)
