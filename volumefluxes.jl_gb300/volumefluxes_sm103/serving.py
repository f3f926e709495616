"""Serving: flood simulations submitted as requests, run with continuous batching.

`Server` wraps the library's serving engine (vf_server_* in
include/volumefluxes_sm103.h). A request carries a scenario (grid, terrain,
rain, friction), the real type and an end time; the engine admits requests
oldest-first while their device memory fits the HBM budget, launches each
poll's admissions as one batch beside the batches still running, and hands the
final interior state back when the request's cluster finishes. Requests run to
their end time exactly as `simulate_to_time` would run them alone.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .api import ArgumentError, SM103Backend, StateView
from .ensemble import BatchOptions


@dataclass
class ServeResult:
    t: float
    steps: int
    last_dt: float
    status: int
    state: StateView  # final interior (h, hu, hv), each (nx, ny)
    submit_s: float = 0.0  # engine clock: seconds since the server was created
    admit_s: float = 0.0
    done_s: float = 0.0

    @property
    def latency_s(self) -> float:
        return self.done_s - self.submit_s


class Request:
    """A request's configuration and arrays in the library's layout, prepared
    ahead of submission so that submitting costs no host copies."""

    def __init__(self, scenario, realtype, endtime: float, device: int = 0):
        be = SM103Backend(realtype, device=device)
        self.cfg = scenario.config(be)
        dt = np.dtype(realtype)
        self.B = None if scenario.B is None else np.ascontiguousarray(np.asarray(scenario.B, dtype=dt).T)
        self.w, self.hu, self.hv = (np.ascontiguousarray(np.asarray(a, dtype=dt).T)
                                    for a in (scenario.w0, scenario.hu0, scenario.hv0))
        self.out = [np.empty((scenario.ny, scenario.nx), dtype=dt) for _ in range(3)]
        self.t0 = float(scenario.t0)
        self.endtime = float(endtime)


class Server:
    def __init__(self, hbm_budget_bytes: int, *, options: BatchOptions | None = None, max_steps: int = 0,
                 device: int = 0):
        self._lib = N.load()
        s = C.c_void_p()
        opt = C.byref(options.native()) if options is not None else None
        N.check_server(self._lib, None, self._lib.vf_server_create(int(device), int(hbm_budget_bytes), opt,
                                                                   int(max_steps), C.byref(s)))
        self._s = s
        self.device = device
        self._live = {}  # ticket -> arrays the engine reads or writes

    def submit(self, scenario, realtype=None, endtime: float | None = None) -> int:
        """Queue one request (a Request, or a scenario with its real type and end
        time); returns its ticket."""
        req = scenario if isinstance(scenario, Request) else Request(scenario, realtype, endtime, self.device)
        tk = C.c_int64()
        N.check_server(self._lib, self._s, self._lib.vf_server_submit(
            self._s, C.byref(req.cfg), None if req.B is None else N.ptr(req.B), N.ptr(req.w), N.ptr(req.hu),
            N.ptr(req.hv), req.t0, req.endtime, N.ptr(req.out[0]), N.ptr(req.out[1]), N.ptr(req.out[2]), C.byref(tk)))
        self._live[tk.value] = req
        return tk.value

    def poll(self, capacity: int = 4096) -> list[int]:
        """Tickets that finished since the last poll (non-blocking)."""
        buf = (C.c_int64 * capacity)()
        n = C.c_int32()
        N.check_server(self._lib, self._s, self._lib.vf_server_poll(self._s, buf, capacity, C.byref(n)))
        return list(buf[:min(n.value, capacity)])

    def result(self, ticket: int, release: bool = True) -> ServeResult:
        t, st, ldt, s = C.c_double(), C.c_int64(), C.c_double(), C.c_int32()
        N.check_server(self._lib, self._s, self._lib.vf_server_result(self._s, int(ticket), C.byref(t), C.byref(st),
                                                                      C.byref(ldt), C.byref(s)))
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        N.check_server(self._lib, self._s, self._lib.vf_server_timing(self._s, int(ticket), C.byref(a), C.byref(b),
                                                                      C.byref(c)))
        out = self._live[ticket].out
        res = ServeResult(t.value, st.value, ldt.value, s.value, StateView(*(o.T for o in out)), a.value, b.value,
                          c.value)
        if release:
            N.check_server(self._lib, self._s, self._lib.vf_server_release(self._s, int(ticket)))
            del self._live[ticket]
        return res

    def stats(self) -> dict:
        used, q, r, l = C.c_int64(), C.c_int32(), C.c_int32(), C.c_int64()
        N.check_server(self._lib, self._s, self._lib.vf_server_stats(self._s, C.byref(used), C.byref(q), C.byref(r),
                                                                     C.byref(l)))
        return {"used_bytes": used.value, "queued": q.value, "running": r.value, "launches": l.value}

    def close(self):
        if self._s is not None:
            self._lib.vf_server_destroy(self._s)
            self._s = None
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
