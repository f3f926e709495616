"""The oracle on dual numbers (the stand-in for ForwardDiff through the
reference CPU path, test/test_swe_ad.jl:36, examples/optimization.jl:116):
its value equals the plain oracle's bit for bit, and its directional
derivative matches central differences of the same frozen-dt run. CPU only."""
import math

import numpy as np

from oracle import vf_oracle as O
from vfhelpers import oracle_from
from volumefluxes_sm103 import scenarios as S


def _case(n=24, steps=12):
    case = S.differentiation_case(n, n_gauges=6)
    sc = case.scenario
    o = oracle_from(sc)
    dts = [o.perform_step(math.inf) for _ in range(steps)]
    w = o.interior()[0]
    gauges = case.gauges
    target = w[gauges[:, 0], gauges[:, 1]] + 0.01
    return sc, o, dts, gauges, target, w


def test_dual_value_is_the_plain_oracle_loss():
    sc, o, dts, gauges, target, w = _case()
    lo, _ = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target)
    d = w[gauges[:, 0], gauges[:, 1]] - target
    want = 0.0
    for x in d:  # gauge order
        want += float(x) * float(x)
    assert lo == want


def test_dual_derivative_matches_central_differences():
    sc, o, dts, gauges, target, _ = _case()
    rng = np.random.default_rng(5)
    x = np.arange(sc.B.shape[0])[:, None]
    y = np.arange(sc.B.shape[1])[None, :]
    rel = []
    for k in range(5):
        # a smooth bump direction on B. The loss is only piecewise smooth (minmod
        # branches, max/min of wave speeds), so a central difference can straddle
        # a switch: the bound is on the median, with a looser one on each.
        cx, cy, s = rng.uniform(4, 20), rng.uniform(4, 20), rng.uniform(3, 8)
        v = np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s))
        _, dlo = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, Bdot=v)
        eps = 1e-6
        lp, _ = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, B=sc.B + eps * v)
        lm, _ = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, B=sc.B - eps * v)
        fd = (lp - lm) / (2 * eps)
        rel.append(abs(fd - dlo) / max(abs(dlo), 1e-12))
    assert max(rel) <= 1e-3 and float(np.median(rel)) <= 1e-4, rel
    # the friction coefficient
    cz = o.p.friction_Cz
    _, dcz = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, Cz_dot=1.0)
    eps = 1e-7
    lp, _ = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, Cz=cz + eps)
    lm, _ = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, Cz=cz - eps)
    fd = (lp - lm) / (2 * eps)
    assert abs(fd - dcz) <= 1e-3 * max(abs(dcz), 1e-12), (fd, dcz)


def test_frozen_run_and_branch_signature():
    """The plain frozen-dt run gives the dual run's value bit for bit; its
    branch-outcome signature is reproducible, and a large perturbation of the
    bottom changes it (a branch switch is detected)."""
    sc, o, dts, gauges, target, _ = _case()
    lo, _ = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target)
    assert O.frozen_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target) == lo

    def run(B=None):
        return lambda: O.frozen_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, B=B)

    a, b = O.branch_signature(run()), O.branch_signature(run())
    assert a == b and sum(a) > 0
    rng = np.random.default_rng(3)
    assert O.branch_signature(run(sc.B + 0.05 * rng.standard_normal(sc.B.shape))) != a


def test_extended_precision_differences_match_the_dual_derivative():
    """Central differences in extended precision with a step small enough to
    stay on one branch (checked with the branch signatures) agree with the
    dual-number derivative to 1e-6: the derivative the oracle and the device
    adjoint follow is the derivative of the loss where the loss is smooth."""
    sc, o, dts, gauges, target, _ = _case()
    hi, lo = O.ext_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target)
    plain = O.frozen_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target)
    assert abs((hi + lo) - plain) <= 1e-10 * abs(plain)
    base = O.branch_signature(lambda: O.frozen_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target))
    rng = np.random.default_rng(5)
    x = np.arange(sc.B.shape[0])[:, None]
    y = np.arange(sc.B.shape[1])[None, :]
    n0 = math.sqrt(o.p.friction_Cz)
    stable = 0
    for k in range(6):
        cx, cy, s = rng.uniform(4, 20), rng.uniform(4, 20), rng.uniform(3, 8)
        v = np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * s * s))
        vn = float(rng.standard_normal()) * 1e-3
        fd, sp, sm = O.ext_central_difference(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, v, 2 * n0 * vn,
                                              vn * vn, 1e-9)
        _, d = O.dual_gauge_loss(o.o, sc.w0, sc.hu0, sc.hv0, dts, gauges, target, Bdot=v, Cz_dot=2 * n0 * vn)
        if sp == base and sm == base:
            stable += 1
            assert abs(fd - d) <= 1e-6 * abs(d), (k, fd, d)
    assert stable >= 5
