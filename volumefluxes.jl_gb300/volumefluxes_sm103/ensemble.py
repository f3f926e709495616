"""Many simulations at once: the batched-ensemble entry points of libvfsm103.so.

The reference advances one Simulator per simulate_to_time call
(src/simulator.jl:179-212). `simulate_batch` runs that loop for a list of
simulators at once, each to its own end time with its own CFL dt; on the
device every simulation is one thread-block cluster that keeps stepping until
its end time, and the GPU's block scheduler starts the next pending simulation
whenever a cluster finishes. `BatchRun` is the non-blocking form used by the
serving loop: launch, poll which simulations have finished, collect them one
by one while the rest keep running.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _native as N
from .api import ArgumentError, Simulator


@dataclass
class BatchOptions:
    """Work granularity of the batch: a simulation with k 32x16 tiles gets the
    smallest power-of-two cluster c <= max_cluster with c * tiles_per_cta >= k;
    Float32 column-marching members split their strips into segments of
    seg_rows rows; members of at least wide_cells cells run the whole-grid
    kernels instead of a cluster. None keeps the library default. time_limit_s
    bounds the batch's device time from its start (watchdog)."""
    tiles_per_cta: int | None = None
    max_cluster: int | None = None
    time_limit_s: float | None = None
    seg_rows: int | None = None
    wide_cells: int | None = None  # members this large run the whole-grid kernels; -1: never

    def native(self) -> N.VfBatchOptions:
        o = N.VfBatchOptions()
        o.tiles_per_cta = int(self.tiles_per_cta or 0)
        o.max_cluster = int(self.max_cluster or 0)
        o.time_limit_s = float(self.time_limit_s or 0.0)
        o.seg_rows = int(self.seg_rows or 0)
        o.wide_cells = int(self.wide_cells or 0)
        return o


@dataclass
class BatchResult:
    t: float
    steps: int
    last_dt: float
    status: int  # N.VF_BATCH_*


STATUS_NAMES = {N.VF_BATCH_OK: "ok", N.VF_BATCH_TIMEOUT: "timeout", N.VF_BATCH_STALLED: "stalled",
                N.VF_BATCH_MAX_STEPS: "max_steps"}


def _handles(sims: Sequence[Simulator]):
    for s in sims:
        if s._functional:
            raise ArgumentError("FunctionalRain is evaluated on the host every step; it cannot run in a batch")
    arr = (C.c_void_p * len(sims))(*[s.handle.value for s in sims])
    return arr


def _opts(options: BatchOptions | None):
    return C.byref(options.native()) if options is not None else None


class BatchRun:
    """A launched batch (vf_batch_launch). Simulators in it must not be used
    until `collect(i)` (or `finish()`) has handed them back."""

    def __init__(self, sims: Sequence[Simulator], endtimes, *, match_endtime: bool = True,
                 maximum_timestep: float | None = None, max_steps: int = 0, options: BatchOptions | None = None):
        if not sims:
            raise ArgumentError("empty batch")
        self.sims = list(sims)
        self._lib = N.load()
        n = len(self.sims)
        ends = np.ascontiguousarray(np.broadcast_to(np.asarray(endtimes, dtype=np.float64), (n,)))
        t0 = np.ascontiguousarray([s.t for s in self.sims], dtype=np.float64)
        self._keep = (_handles(self.sims), ends, t0)
        b = C.c_void_p()
        max_ts = -1.0 if maximum_timestep is None else float(maximum_timestep)
        N.check_batch(self._lib, None, self._lib.vf_batch_launch(self._keep[0], n, N.ptr(t0), N.ptr(ends),
                                                                 int(match_endtime), max_ts, int(max_steps),
                                                                 _opts(options), C.byref(b)))
        self._b = b
        self._results: list[BatchResult | None] = [None] * n

    def __len__(self):
        return len(self.sims)

    def n_done(self) -> int:
        c = C.c_int32()
        N.check_batch(self._lib, self._b, self._lib.vf_batch_poll(self._b, C.byref(c)))
        return c.value

    def is_done(self, i: int) -> bool:
        rc = self._lib.vf_batch_is_done(self._b, int(i))
        if rc < 0:
            N.check_batch(self._lib, self._b, rc)
        return rc == 1

    def collect(self, i: int) -> BatchResult:
        if self._results[i] is not None:
            return self._results[i]
        t, st, ldt, s = C.c_double(), C.c_int64(), C.c_double(), C.c_int32()
        N.check_batch(self._lib, self._b, self._lib.vf_batch_collect(self._b, int(i), C.byref(t), C.byref(st),
                                                                     C.byref(ldt), C.byref(s)))
        r = BatchResult(t.value, st.value, ldt.value, s.value)
        sim = self.sims[i]
        sim.t = r.t
        if r.steps:
            sim.current_timestep = r.last_dt
        self._results[i] = r
        return r

    def wait(self) -> None:
        N.check_batch(self._lib, self._b, self._lib.vf_batch_wait(self._b))

    def finish(self) -> list[BatchResult]:
        """Wait for every simulation, collect them all, free the batch."""
        if self._b is None:
            return list(self._results)
        self.wait()
        out = [self.collect(i) for i in range(len(self.sims))]
        self.free()
        return out

    def free(self) -> None:
        if self._b is not None:
            b, self._b = self._b, None
            N.check_batch(self._lib, None, self._lib.vf_batch_free(b))

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def simulate_batch(sims: Sequence[Simulator], endtimes, *, match_endtime: bool = True,
                   maximum_timestep: float | None = None, max_steps: int = 0,
                   options: BatchOptions | None = None) -> list[BatchResult]:
    """simulate_to_time(sim, endtime) for every simulator at once, on the device.

    Equivalent to `for s, T in zip(sims, endtimes): simulate_to_time(s, T)` with
    callback = nothing: each simulator's t and current_timestep are updated and
    its state is the state at its end time (bitwise the same in Float64).
    """
    return BatchRun(sims, endtimes, match_endtime=match_endtime, maximum_timestep=maximum_timestep,
                    max_steps=max_steps, options=options).finish()


def cluster_size(sim: Simulator, options: BatchOptions | None = None) -> int:
    lib = N.load()
    c = C.c_int32()
    N.check_batch(lib, None, lib.vf_batch_cluster_size(sim.handle, _opts(options), C.byref(c)))
    return c.value


DEFAULT_CANDIDATES = tuple(BatchOptions(tiles_per_cta=tp, seg_rows=sr)
                           for tp in (4, 8, 16, 32, 64) for sr in (None, 16, 32))


def autotune(sims: Sequence[Simulator], *, steps: int = 100, candidates: Sequence[BatchOptions] | None = None,
             repeats: int = 1) -> tuple[BatchOptions, list[tuple[BatchOptions, float]]]:
    """Choose the batch's work granularity by measurement.

    Runs the given simulators as one batch of `steps` steps each (no end time)
    under every candidate option set and returns the one with the most
    cell-updates per second, with the whole table. The simulators advance by
    repeats * steps per candidate; use throwaway copies of the real members.
    """
    import time

    cands = list(candidates or DEFAULT_CANDIDATES)
    cells = sum(s.grid.nx * s.grid.ny for s in sims)
    simulate_batch(sims, 1e30, max_steps=2, match_endtime=False)  # first-use costs outside the timing
    table = []
    for c in cands:
        best = math.inf
        for _ in range(repeats):
            t0 = time.perf_counter()
            res = simulate_batch(sims, 1e30, max_steps=steps, match_endtime=False, options=c)
            el = time.perf_counter() - t0
            done = sum(s.grid.nx * s.grid.ny * r.steps for s, r in zip(sims, res))
            best = min(best, el * (cells * steps) / max(done, 1))
        table.append((c, cells * steps / best))
    table.sort(key=lambda e: -e[1])
    return table[0][0], table
