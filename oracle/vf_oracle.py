"""ctypes wrapper of the CPU oracle (oracle/vf_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libvforacle.so"

SRC_BOTTOM, SRC_CONST_RAIN, SRC_CONST_INFIL, SRC_TIME_RAIN, SRC_HORTON, SRC_RAIN_FIELD = 1, 2, 3, 4, 5, 6
BC_WALL, BC_PERIODIC, BC_NEUMANN = 1, 2, 3
REC_LINEAR, REC_NONE = 1, 2
FRICTION_NONE, FRICTION_BSA2012, FRICTION_FCG2016, FRICTION_BH2021 = 0, 1, 2, 3
STEPPER_FE, STEPPER_RK2 = 1, 2


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("gc", C.c_int),
        ("extent", C.c_double * 4),
        ("real_bytes", C.c_int),
        ("g", C.c_double), ("rho", C.c_double), ("depth_cutoff", C.c_double), ("desingularizing_kappa", C.c_double),
        ("reconstruction", C.c_int), ("theta", C.c_double),
        ("n_sources", C.c_int), ("source_kind", C.c_int * 8), ("source_rate", C.c_double * 8),
        ("source_aux", (C.c_double * 2) * 8),
        ("friction", C.c_int), ("friction_Cz", C.c_double),
        ("stepper", C.c_int), ("bc", C.c_int), ("cfl", C.c_double),
        ("bottom_is_constant", C.c_int), ("bottom_constant", C.c_double),
    ]


_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        import importlib.util
        spec = importlib.util.spec_from_file_location("_vf_oracle_build", HERE / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = C.CDLL(os.fspath(LIB_PATH))
    P = C.c_void_p
    D = C.c_double
    sig = {
        "vfo_create": (C.c_int, [C.POINTER(Params), P, C.POINTER(C.c_void_p)]),
        "vfo_destroy": (None, [P]),
        "vfo_set_interior": (C.c_int, [P, P, P, P]),
        "vfo_get_state": (C.c_int, [P, P]),
        "vfo_get_interior": (C.c_int, [P, P, P, P]),
        "vfo_perform_step": (C.c_int, [P, D, C.POINTER(D)]),
        "vfo_simulate_to_time": (C.c_int, [P, D, C.c_int, D, C.c_longlong, C.POINTER(C.c_longlong)]),
        "vfo_time": (D, [P]),
        "vfo_set_time": (None, [P, D]),
        "vfo_current_timestep": (D, [P]),
        "vfo_set_threads": (C.c_int, [C.c_int]),
        "vfo_get_threads": (C.c_int, []),
        "vfo_minmod": (D, [D, D, D]),
        "vfo_minmod_slope": (D, [D, D, D, D]),
        "vfo_bottom_lookup": (D, [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
        "vfo_update_bc_wall": (C.c_int, [P, C.c_int, C.c_int, C.c_int]),
        "vfo_cbrt": (D, [D]),
        "vfo_exp": (D, [D]),
        "vfo_set_source_table": (C.c_int, [P, C.c_int, P, P, C.c_int]),
        "vfo_set_source_field": (C.c_int, [P, C.c_int, P]),
        "vfo_update_bc_periodic": (C.c_int, [P, C.c_int, C.c_int, C.c_int]),
        "vfo_update_bc_neumann": (C.c_int, [P, C.c_int, C.c_int, C.c_int]),
        "vfo_desingularize": (D, [D, D]),
        "vfo_dual_gauge_loss": (C.c_int, [C.POINTER(Params), P, P, D, P, P, P, P, C.c_int, P, P, P, C.c_int,
                                          C.POINTER(D), C.POINTER(D), P]),
        "vfo_frozen_gauge_loss": (C.c_int, [C.POINTER(Params), P, P, P, P, P, C.c_int, P, P, P, C.c_int,
                                            C.POINTER(D), P]),
        "vfo_ext_gauge_loss": (C.c_int, [C.POINTER(Params), P, P, D, D, D, P, P, P, P, C.c_int, P, P, P, C.c_int,
                                         C.POINTER(D), C.POINTER(D), P]),
        "vfo_branch_counting": (None, [C.c_int]),
        "vfo_branch_counts": (C.c_int, [C.POINTER(C.c_ulonglong), C.c_int]),
    }
    for n, (r, a) in sig.items():
        f = getattr(lib, n)
        f.restype = r
        f.argtypes = a
    _lib = lib
    return lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


class OracleSim:
    """One oracle simulation; arrays use the reference's (nx, ny) [i, j] indexing."""

    def __init__(self, *, nx, ny, extent=((0.0, 1.0), (0.0, 1.0)), real_bytes=8, g=9.81, rho=1.0,
                 depth_cutoff=1e-5, desingularizing_kappa=1e-5, theta=1.2, sources=(), friction=FRICTION_NONE,
                 friction_Cz=0.0, stepper=STEPPER_RK2, cfl=0.25, B=None, bottom_constant=0.0, gc=2, bc=BC_WALL,
                 reconstruction=REC_LINEAR):
        """sources: list of (kind, rate) or (kind, rate, aux0, aux1)."""
        self.lib = load()
        p = Params()
        p.nx, p.ny, p.gc = nx, ny, gc
        e = np.asarray(extent, dtype=np.float64).reshape(-1)
        for i in range(4):
            p.extent[i] = e[i]
        p.real_bytes = real_bytes
        p.g, p.rho, p.depth_cutoff, p.desingularizing_kappa = g, rho, depth_cutoff, desingularizing_kappa
        p.reconstruction, p.theta = reconstruction, theta
        p.n_sources = len(sources)
        for i, src in enumerate(sources):
            p.source_kind[i], p.source_rate[i] = src[0], src[1]
            if len(src) > 2:
                p.source_aux[i][0], p.source_aux[i][1] = src[2], src[3]
        p.friction, p.friction_Cz = friction, friction_Cz
        p.stepper, p.bc, p.cfl = stepper, bc, cfl
        self.nx, self.ny, self.gc = nx, ny, gc
        self.N1, self.N2 = nx + 2 * gc, ny + 2 * gc
        if B is None:
            p.bottom_is_constant, p.bottom_constant = 1, bottom_constant
            bptr = None
        else:
            B = np.asarray(B, dtype=np.float64)
            assert B.shape == (self.N1 + 1, self.N2 + 1)
            self._B = np.ascontiguousarray(B.T)
            p.bottom_is_constant = 0
            bptr = _p(self._B)
        self.p = p
        h = C.c_void_p()
        rc = self.lib.vfo_create(C.byref(p), bptr, C.byref(h))
        if rc != 0:
            raise ValueError(f"oracle rejected the configuration ({rc})")
        self.h = h

    def __del__(self):
        try:
            if self.h:
                self.lib.vfo_destroy(self.h)
        except Exception:
            pass

    def set_source_table(self, index, times, rates):
        t = np.ascontiguousarray(times, dtype=np.float64)
        r = np.ascontiguousarray(rates, dtype=np.float64)
        assert self.lib.vfo_set_source_table(self.h, index, _p(t), _p(r), len(t)) == 0

    def set_source_field(self, index, field):
        """field: (N1, N2) array over the total grid, indexed [i, j]."""
        f = np.ascontiguousarray(np.asarray(field, dtype=np.float64).T)
        assert f.shape == (self.N2, self.N1)
        assert self.lib.vfo_set_source_field(self.h, index, _p(f)) == 0

    def set_interior(self, w, hu, hv):
        planes = [np.ascontiguousarray(np.asarray(a, dtype=np.float64).T) for a in (w, hu, hv)]
        assert all(pl.shape == (self.ny, self.nx) for pl in planes)
        assert self.lib.vfo_set_interior(self.h, *(_p(pl) for pl in planes)) == 0

    def interior(self):
        planes = [np.empty((self.ny, self.nx)) for _ in range(3)]
        assert self.lib.vfo_get_interior(self.h, *(_p(pl) for pl in planes)) == 0
        return tuple(pl.T for pl in planes)

    def state(self):
        buf = np.empty(3 * self.N1 * self.N2)
        assert self.lib.vfo_get_state(self.h, _p(buf)) == 0
        p = buf.reshape(3, self.N2, self.N1)
        return tuple(x.T for x in p)

    def perform_step(self, max_dt):
        dt = C.c_double()
        assert self.lib.vfo_perform_step(self.h, float(max_dt), C.byref(dt)) == 0
        return dt.value

    def simulate_to_time(self, endtime, match_endtime=True, maximum_timestep=None, max_steps=0):
        n = C.c_longlong()
        mts = -1.0 if maximum_timestep is None else float(maximum_timestep)
        assert self.lib.vfo_simulate_to_time(self.h, float(endtime), int(match_endtime), mts, int(max_steps),
                                             C.byref(n)) == 0
        return n.value

    @property
    def t(self):
        return self.lib.vfo_time(self.h)

    @t.setter
    def t(self, v):
        self.lib.vfo_set_time(self.h, float(v))

    @property
    def current_timestep(self):
        return self.lib.vfo_current_timestep(self.h)


def set_threads(n: int) -> int:
    return load().vfo_set_threads(int(n))


def dual_gauge_loss(sim: OracleSim, w, hu, hv, dts, gauges, target, *, B=None, Bdot=None, Cz=None, Cz_dot=0.0):
    """Loss sum_g (w[g] - target[g])^2 after len(dts) steps with the frozen dt
    sequence, from the interior state (w, hu, hv) ((nx, ny) arrays), in Float64
    dual numbers through the oracle with sim's configuration: returns (loss,
    d loss along (Bdot, Cz_dot)). B / Cz override sim's bottom corners
    ((N1+1, N2+1), [i, j]) and friction coefficient; gauges: (n, 2) interior
    indices [i, j]."""
    lib = sim.lib
    p = Params()
    C.pointer(p)[0] = sim.p
    if Cz is not None:
        p.friction_Cz = float(Cz)
    Bt = sim._B if B is None else np.ascontiguousarray(np.asarray(B, dtype=np.float64).T)
    Bd = None if Bdot is None else np.ascontiguousarray(np.asarray(Bdot, dtype=np.float64).T)
    arrs = [np.ascontiguousarray(np.asarray(a, dtype=np.float64).T) for a in (w, hu, hv)]
    d = np.ascontiguousarray(dts, dtype=np.float64)
    g = np.asarray(gauges, dtype=np.int32)
    gi, gj = np.ascontiguousarray(g[:, 0]), np.ascontiguousarray(g[:, 1])
    tg = np.ascontiguousarray(target, dtype=np.float64)
    loss, dloss = C.c_double(), C.c_double()
    rc = lib.vfo_dual_gauge_loss(C.byref(p), _p(Bt), None if Bd is None else _p(Bd), float(Cz_dot), _p(arrs[0]),
                                 _p(arrs[1]), _p(arrs[2]), _p(d), len(d), _p(gi), _p(gj), _p(tg), len(tg),
                                 C.byref(loss), C.byref(dloss), sim.h)
    if rc != 0:
        raise ValueError(f"oracle dual run failed ({rc})")
    return loss.value, dloss.value


def get_threads() -> int:
    return load().vfo_get_threads()


def _gauge_args(sim, w, hu, hv, dts, gauges, target, B, Cz):
    p = Params()
    C.pointer(p)[0] = sim.p
    if Cz is not None:
        p.friction_Cz = float(Cz)
    Bt = sim._B if B is None else np.ascontiguousarray(np.asarray(B, dtype=np.float64).T)
    arrs = [np.ascontiguousarray(np.asarray(a, dtype=np.float64).T) for a in (w, hu, hv)]
    d = np.ascontiguousarray(dts, dtype=np.float64)
    g = np.asarray(gauges, dtype=np.int32)
    gi, gj = np.ascontiguousarray(g[:, 0]), np.ascontiguousarray(g[:, 1])
    tg = np.ascontiguousarray(target, dtype=np.float64)
    return p, Bt, arrs, d, gi, gj, tg


def frozen_gauge_loss(sim: OracleSim, w, hu, hv, dts, gauges, target, *, B=None, Cz=None) -> float:
    """The loss of dual_gauge_loss in plain Float64: from the interior state,
    len(dts) steps with the frozen dt sequence, B / Cz overriding sim's."""
    p, Bt, arrs, d, gi, gj, tg = _gauge_args(sim, w, hu, hv, dts, gauges, target, B, Cz)
    loss = C.c_double()
    rc = sim.lib.vfo_frozen_gauge_loss(C.byref(p), _p(Bt), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(d), len(d),
                                       _p(gi), _p(gj), _p(tg), len(tg), C.byref(loss), sim.h)
    if rc != 0:
        raise ValueError(f"oracle frozen run failed ({rc})")
    return loss.value


def branch_signature(run) -> tuple:
    """Branch-outcome counts of the oracle while `run()` executes (see
    vfo_branch_counting): runs with equal signatures took the same branches."""
    lib = load()
    lib.vfo_branch_counting(1)
    try:
        run()
        out = (C.c_ulonglong * 32)()
        n = lib.vfo_branch_counts(out, 32)
        return tuple(int(out[i]) for i in range(n))
    finally:
        lib.vfo_branch_counting(0)


def ext_gauge_loss(sim: OracleSim, w, hu, hv, dts, gauges, target, *, Bdir=None, Cz_dir1=0.0, Cz_dir2=0.0,
                   eps=0.0):
    """The frozen-dt loss in extended precision (long double) at B + eps*Bdir and
    Cz + eps*Cz_dir1 + eps^2*Cz_dir2 (perturbations formed in that precision),
    as (hi, lo) doubles whose sum is the loss."""
    p, Bt, arrs, d, gi, gj, tg = _gauge_args(sim, w, hu, hv, dts, gauges, target, None, None)
    Bd = None if Bdir is None else np.ascontiguousarray(np.asarray(Bdir, dtype=np.float64).T)
    hi, lo = C.c_double(), C.c_double()
    rc = sim.lib.vfo_ext_gauge_loss(C.byref(p), _p(Bt), None if Bd is None else _p(Bd), float(Cz_dir1),
                                    float(Cz_dir2), float(eps), _p(arrs[0]), _p(arrs[1]), _p(arrs[2]), _p(d), len(d),
                                    _p(gi), _p(gj), _p(tg), len(tg), C.byref(hi), C.byref(lo), sim.h)
    if rc != 0:
        raise ValueError(f"oracle extended-precision run failed ({rc})")
    return hi.value, lo.value


def ext_central_difference(sim: OracleSim, w, hu, hv, dts, gauges, target, Bdir, Cz_dir1, Cz_dir2, eps):
    """Central difference of the loss along (Bdir, Cz) in extended precision,
    with the branch-outcome signatures of the +eps and -eps runs:
    (fd, sig_plus, sig_minus)."""
    runs = {}
    sigs = {}
    for sign in (1, -1):
        def run(sign=sign):
            runs[sign] = ext_gauge_loss(sim, w, hu, hv, dts, gauges, target, Bdir=Bdir, Cz_dir1=Cz_dir1,
                                        Cz_dir2=Cz_dir2, eps=sign * eps)
        sigs[sign] = branch_signature(run)
    (ph, pl), (mh, ml) = runs[1], runs[-1]
    return ((ph - mh) + (pl - ml)) / (2 * eps), sigs[1], sigs[-1]
