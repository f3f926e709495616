"""Reverse-mode gradients on the GPU (vf_adjoint_*): dLoss/dB for every bottom
corner and dLoss/dCz of the gauge loss sum_g (w_g - target_g)^2, with the dt
sequence frozen from the forward pass, checked against the oracle run on
dual numbers (the stand-in for ForwardDiff through the reference CPU path)
and against central finite differences."""
import math

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import adjoint as AD
from volumefluxes_sm103 import scenarios as S
from oracle import vf_oracle as O
from vfhelpers import oracle_from

pytestmark = pytest.mark.gpu


def small_case(n=40, steps=25):
    case = S.differentiation_case(n, n_gauges=8)
    extra = np.array([[0, 5], [n - 1, 20], [7, 0], [n - 2, n - 1], [1, 1]], dtype=np.int32)  # next to the walls
    gauges = np.concatenate([case.gauges, extra])
    return case, gauges, steps


def run_adjoint(case, gauges, steps, real=np.float64, checkpoint_every=4, dts=None):
    sc = case.scenario
    sim = sc.build(vf.SM103Backend(real))
    adj = AD.GaugeAdjoint(sim, steps, checkpoint_every)
    dts = adj.forward(dts)
    target = AD.gauge_values(sc, np.float64, gauges, dts, B=case.B_target)
    loss, gB, gCz = adj.backward(gauges, target)
    adj.close()
    return dts, target, loss, gB, gCz


def test_adjoint_equals_the_dual_number_oracle():
    case, gauges, steps = small_case()
    dts, target, loss, gB, gCz = run_adjoint(case, gauges, steps)
    sc = case.scenario
    o = oracle_from(sc)
    ref_dts = [o.perform_step(math.inf) for _ in range(steps)]
    assert list(dts) == ref_dts  # the forward pass is the oracle's, bit for bit
    rng = np.random.default_rng(11)
    for k in range(4):
        v = rng.standard_normal(sc.B.shape)
        cz = float(rng.standard_normal()) * 1e-3
        lo, dlo = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, Bdot=v, Cz_dot=cz)
        assert lo == loss
        got = float(np.sum(gB * v)) + gCz * cz
        assert abs(got - dlo) <= 1e-9 * abs(dlo), (k, got, dlo)


def test_checkpoint_interval_does_not_change_the_gradient():
    case, gauges, steps = small_case(n=32, steps=17)
    a = run_adjoint(case, gauges, steps, checkpoint_every=1)
    b = run_adjoint(case, gauges, steps, checkpoint_every=5)
    c = run_adjoint(case, gauges, steps, checkpoint_every=17)
    assert a[2] == b[2] == c[2]
    assert np.array_equal(a[3], b[3]) and np.array_equal(a[3], c[3])
    assert a[4] == b[4] == c[4]


FD_TOL = 1e-6   # relative agreement of the gradient with central differences
FD_EPS = 1e-9   # central-difference step of the extended-precision reference


def smooth_fd(case, gauges, target, dts, v, vn, eps=FD_EPS):
    """Central difference of the loss along (B, n) -> (B + eps v, n + eps vn),
    taken on the oracle in extended precision (long double) so that a step
    small enough to stay on one branch is not swamped by Float64 rounding, and
    whether both perturbed runs took the branches of the unperturbed Float64
    run everywhere (the oracle's branch-outcome counters). Returns (fd, stable)."""
    sc = case.scenario
    o = oracle_from(sc).o
    n0 = sc.manning_n
    base = O.branch_signature(lambda: O.frozen_gauge_loss(o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target))
    fd, sp, sm = O.ext_central_difference(o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, v, 2 * n0 * vn, vn * vn, eps)
    return fd, (sp == base and sm == base)


def test_cz_gradient_matches_central_differences():
    case, gauges, steps = small_case()
    dts, target, loss, gB, gCz = run_adjoint(case, gauges, steps)
    n = case.scenario.manning_n
    fd, stable = smooth_fd(case, gauges, target, dts, np.zeros_like(case.scenario.B), 1.0)
    assert stable
    got = gCz * 2 * n  # d loss / d n = 2n dLoss/dCz
    assert abs(fd - got) <= FD_TOL * abs(got), (fd, got)


def test_smooth_bottom_direction_matches_central_differences():
    case, gauges, steps = small_case()
    dts, target, loss, gB, gCz = run_adjoint(case, gauges, steps)
    sc = case.scenario
    f = vf.cell_faces(sc.grid(), interior=False)
    v = np.exp(-((f[:, :, 0] - 17.0) ** 2 + (f[:, :, 1] - 23.0) ** 2) / (2 * 8.0 ** 2))  # a smooth bump
    fd, stable = smooth_fd(case, gauges, target, dts, v, 0.0)
    assert stable
    got = float(np.sum(gB * v))
    assert abs(fd - got) <= FD_TOL * abs(got), (fd, got)


@pytest.mark.parametrize("n,steps,ndirs", [(40, 25, 12), (64, 60, 6)])
def test_random_directions_match_central_differences_where_differentiable(n, steps, ndirs):
    """Random directions (Gaussian bumps on B plus an n component): where the
    perturbed runs take the unperturbed run's branches (no minmod, wet/dry,
    wave-speed or dry-clamp switch inside the step) the gradient matches the
    central difference to 1e-6; directions that cross a switch are counted and
    must stay a minority."""
    case, gauges, steps = small_case(n=n, steps=steps)
    dts, target, loss, gB, gCz = run_adjoint(case, gauges, steps)
    sc = case.scenario
    f = vf.cell_faces(sc.grid(), interior=False)
    rng = np.random.default_rng(7)
    stable = 0
    for k in range(ndirs):
        v = np.zeros_like(sc.B)
        for _ in range(3):
            cx, cy, s = rng.uniform(0, sc.nx), rng.uniform(0, sc.ny), rng.uniform(0.08 * n, 0.4 * n)
            v += rng.standard_normal() * np.exp(-((f[:, :, 0] - cx) ** 2 + (f[:, :, 1] - cy) ** 2) / (2 * s * s))
        vn = float(rng.standard_normal()) * 1e-3
        fd, ok = smooth_fd(case, gauges, target, dts, v, vn)
        if not ok:
            continue
        stable += 1
        got = float(np.sum(gB * v)) + gCz * 2 * sc.manning_n * vn
        assert abs(fd - got) <= FD_TOL * abs(got), (k, fd, got)
    assert stable >= (3 * ndirs) // 4, stable


def test_float32_gradient_tracks_float64():
    case, gauges, steps = small_case()
    d64 = run_adjoint(case, gauges, steps)
    d32 = run_adjoint(case, gauges, steps, real=np.float32, dts=d64[0])
    rel = np.linalg.norm(d32[3] - d64[3]) / np.linalg.norm(d64[3])
    assert rel < 0.05, rel
    assert abs(d32[4] - d64[4]) <= 0.05 * abs(d64[4])


def test_autograd_function_gives_the_adjoint_gradient():
    torch = pytest.importorskip("torch")
    case, gauges, steps = small_case(n=24, steps=10)
    dts, target, loss, gB, gCz = run_adjoint(case, gauges, steps)
    B = torch.tensor(case.scenario.B, dtype=torch.float64, requires_grad=True)
    n = torch.tensor(case.scenario.manning_n, dtype=torch.float64, requires_grad=True)
    L = AD.GaugeLoss.apply(B, n, case.scenario, np.float64, gauges, target, dts)
    L.backward()
    assert float(L.detach()) == loss
    assert np.array_equal(B.grad.numpy(), gB)
    assert float(n.grad) == gCz * 2 * case.scenario.manning_n


def _variant(kind):
    """The small differentiation case under forward Euler, PeriodicBC,
    NoReconstruction, or with TimeDependentRain and HortonInfiltration (a
    seeded per-cell factor)."""
    from dataclasses import replace
    case, gauges, steps = small_case(n=40, steps=20)
    sc = case.scenario
    if kind == "fe":
        sc = replace(sc, stepper="fe")
    elif kind == "periodic":
        sc = replace(sc, bc="periodic")
    elif kind == "fe_periodic":
        sc = replace(sc, stepper="fe", bc="periodic")
    elif kind == "no_reconstruction":
        sc = replace(sc, reconstruction="none")
    elif kind == "no_reconstruction_fe_periodic":
        sc = replace(sc, reconstruction="none", stepper="fe", bc="periodic")
    elif kind == "dynamic_sources":
        grid = sc.grid()
        rng = np.random.default_rng(3)
        factor = rng.uniform(0.5, 1.5, (sc.nx + 4, sc.ny + 4))
        sc = replace(sc, sources=[vf.SourceTermBottom(),
                                  vf.TimeDependentRain(np.array([200.0, 20.0, 300.0]), np.array([0.0, 2.0, 4.0])),
                                  vf.HortonInfiltration(grid, vf.SM103Backend(), factor=factor, f0=4e-3, fc=1e-4,
                                                        k=0.5)])
    return replace(case, scenario=sc), gauges, steps


@pytest.mark.parametrize("kind", ["fe", "periodic", "fe_periodic", "dynamic_sources", "no_reconstruction",
                                  "no_reconstruction_fe_periodic"])
def test_adjoint_beyond_the_differentiation_workload(kind):
    """Forward Euler, PeriodicBC, NoReconstruction and the time-dependent sources against the
    dual-number oracle (the ForwardDiff stand-in): the forward pass is the
    oracle's bit for bit and the gradient agrees to 1e-9."""
    case, gauges, steps = _variant(kind)
    sc = case.scenario
    dts, target, loss, gB, gCz = run_adjoint(case, gauges, steps)
    o = oracle_from(sc)
    ref = []
    for _ in range(steps):
        dt = o.perform_step(math.inf)
        o.o.t = o.o.t + dt  # the adjoint's forward pass runs from t = 0 with t += dt
        ref.append(dt)
    assert list(dts) == ref
    o = oracle_from(sc)
    rng = np.random.default_rng(13)
    for k in range(3):
        v = rng.standard_normal(sc.B.shape)
        cz = float(rng.standard_normal()) * 1e-3
        lo, dlo = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, Bdot=v, Cz_dot=cz)
        assert lo == loss
        got = float(np.sum(gB * v)) + gCz * cz
        assert abs(got - dlo) <= 1e-9 * abs(dlo), (k, got, dlo)


def test_adjoint_rejects_what_it_does_not_cover():
    from dataclasses import replace
    case, gauges, steps = small_case(n=24, steps=4)
    for sc in (replace(case.scenario, bc="neumann"),):
        sim = sc.build(vf.SM103Backend(np.float64))
        with pytest.raises(vf.ArgumentError):
            AD.GaugeAdjoint(sim, steps)
        sim.close()
