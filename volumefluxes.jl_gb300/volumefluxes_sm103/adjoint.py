"""Gradients of a gauge loss through the device time loop (vf_adjoint_* of
include/volumefluxes_sm103.h).

The reference differentiates through its CPU path with ForwardDiff dual
numbers (test/test_swe_ad.jl, examples/optimization.jl): one derivative
direction per pass. Here one reverse sweep on the GPU gives the gradient of

    loss = sum_g (w_final[g] - target[g])^2

with respect to every bottom corner B and the friction coefficient Cz (and so
Manning's n, Cz = n^2) at once, with the dt sequence frozen from the forward
pass and sqrt(N)-step checkpointing. `GaugeLoss` is the torch.autograd.Function
twin of the ChainRulesCore rrule the Julia glue defines.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import replace

import numpy as np

from . import _native as N
from .api import ArgumentError, SM103Backend


class GaugeAdjoint:
    """Forward run with checkpoints and the reverse sweep, for one simulator
    whose current state is the initial state U^0."""

    def __init__(self, sim, n_steps: int, checkpoint_every: int = 0):
        self.sim = sim
        self.n_steps = int(n_steps)
        self._lib = N.load()
        a = C.c_void_p()
        N.check_adjoint(self._lib, None, self._lib.vf_adjoint_create(sim.handle, self.n_steps, int(checkpoint_every),
                                                                     C.byref(a)))
        self._a = a
        self.dts = None

    def forward(self, frozen_dts=None) -> np.ndarray:
        """Run the n_steps from U^0 (with the given dt sequence, else the CFL
        dt of each step); returns the dt sequence."""
        out = np.empty(self.n_steps, dtype=np.float64)
        fz = None if frozen_dts is None else np.ascontiguousarray(frozen_dts, dtype=np.float64)
        if fz is not None and fz.size != self.n_steps:
            raise ArgumentError("frozen_dts needs one dt per step")
        N.check_adjoint(self._lib, self._a, self._lib.vf_adjoint_forward(self._a, None if fz is None else N.ptr(fz),
                                                                         N.ptr(out)))
        self.dts = out
        self.sim.t = float(np.sum(out))
        return out

    def backward(self, gauges, target):
        """(loss, dLoss/dB with the corner array's [i, j] shape, dLoss/dCz)."""
        g = np.asarray(gauges, dtype=np.int32).reshape(-1, 2)
        gi, gj = np.ascontiguousarray(g[:, 0]), np.ascontiguousarray(g[:, 1])
        tg = np.ascontiguousarray(target, dtype=np.float64)
        grid = self.sim.grid
        W, H = grid.nx + 2 * grid.gc + 1, grid.ny + 2 * grid.gc + 1
        gB = np.empty((H, W), dtype=np.float64)
        loss, gcz = C.c_double(), C.c_double()
        N.check_adjoint(self._lib, self._a, self._lib.vf_adjoint_backward(
            self._a, N.ptr(gi), N.ptr(gj), N.ptr(tg), len(tg), C.byref(loss), N.ptr(gB), C.byref(gcz)))
        return loss.value, gB.T.copy(), gcz.value

    def close(self):
        if self._a is not None:
            self._lib.vf_adjoint_destroy(self._a)
            self._a = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gauge_loss(scenario, realtype, gauges, target, dts, *, B=None, manning_n=None) -> float:
    """Loss of the forward run with a frozen dt sequence (no gradient): for
    finite differences and targets."""
    sc = replace(scenario, B=scenario.B if B is None else np.asarray(B),
                 manning_n=scenario.manning_n if manning_n is None else float(manning_n))
    sim = sc.build(SM103Backend(realtype))
    lib = sim._lib
    t = float(sc.t0)
    for dt in dts:
        N.check(lib, sim.handle, lib.vf_step_fixed(sim.handle, float(dt), t))
        t += float(dt)
    w = __import__("volumefluxes_sm103").current_interior_state(sim).h
    g = np.asarray(gauges).reshape(-1, 2)
    d = w[g[:, 0], g[:, 1]].astype(np.float64) - np.asarray(target, dtype=np.float64)
    sim.close()
    loss = 0.0
    for x in d:  # gauge order, as the device sums
        loss += float(x) * float(x)
    return loss


def gauge_values(scenario, realtype, gauges, dts, *, B=None) -> np.ndarray:
    """w at the gauges after the frozen-dt run (targets from a perturbed terrain)."""
    sc = replace(scenario, B=scenario.B if B is None else np.asarray(B))
    sim = sc.build(SM103Backend(realtype))
    lib = sim._lib
    t = float(sc.t0)
    for dt in dts:
        N.check(lib, sim.handle, lib.vf_step_fixed(sim.handle, float(dt), t))
        t += float(dt)
    w = __import__("volumefluxes_sm103").current_interior_state(sim).h
    g = np.asarray(gauges).reshape(-1, 2)
    out = w[g[:, 0], g[:, 1]].astype(np.float64)
    sim.close()
    return out


try:
    import torch

    class GaugeLoss(torch.autograd.Function):
        """loss(B, n) = sum_g (w_final[g] - target[g])^2 after the scenario's
        frozen-dt run with bottom corners B and Manning n (Cz = n^2).

        forward runs the device loop with checkpoints; backward runs the
        reverse sweep and returns dLoss/dB and dLoss/dn = 2 n dLoss/dCz.
        """

        @staticmethod
        def forward(ctx, B, n, scenario, realtype, gauges, target, dts, checkpoint_every=0):
            sc = replace(scenario, B=B.detach().cpu().numpy().astype(np.float64),
                         manning_n=float(n.detach().cpu().item()))
            sim = sc.build(SM103Backend(realtype))
            adj = GaugeAdjoint(sim, len(dts), checkpoint_every)
            adj.forward(dts)
            loss, gB, gCz = adj.backward(gauges, target)
            adj.close()
            sim.close()
            ctx.save_for_backward(torch.from_numpy(gB), torch.tensor(gCz * 2.0 * float(n.item()), dtype=torch.float64))
            return torch.tensor(loss, dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            gB, gn = ctx.saved_tensors
            return grad_out * gB, grad_out * gn, None, None, None, None, None, None
except ImportError:  # torch is optional for the library itself
    GaugeLoss = None


def central_difference(sc, real, gauges, target, dts, Bdir, n_dir: float, eps: float) -> float:
    """(loss(B + eps*Bdir, n + eps*n_dir) - loss(B - eps*Bdir, n - eps*n_dir)) / (2 eps),
    each loss a forward run on the device with the frozen dt sequence."""
    n0 = sc.manning_n
    lp = gauge_loss(sc, real, gauges, target, dts, B=sc.B + eps * Bdir, manning_n=n0 + eps * n_dir)
    lm = gauge_loss(sc, real, gauges, target, dts, B=sc.B - eps * Bdir, manning_n=n0 - eps * n_dir)
    return (lp - lm) / (2 * eps)

