"""Float64 faithful arithmetic (VF_ARITH_FAITHFUL): the per-step kernels with
faithful quotients and fused multiply-adds, held to a tolerance instead of to
the reference's bits.

Measured at 4096^2 wet/dry over 1000 RK2 steps the mode is 1.5x faster than the
reference-rounded kernels and differs from them by 2.7e-13 in w relative to
max|w|, but by 2.7e-9 / 4.1e-9 in hu / hv relative to max|hu| / max|hv|: the
momenta of this nearly quiescent lake are ~1e-3, three orders below the depths,
so one rounding difference in a momentum flux already exceeds the per-field
1e-12 bound. The bounds asserted here are therefore w within 1e-12 of max|w|
and hu, hv within 1e-12 of max|w| (the state's max-norm), plus the reference's
lake-at-rest property, on the measured workload's cell size (1 m) and two
small cases. Where thin films decide the CFL step (e.g. the same hills on 4 m
cells) rounding picks which film cell is fastest, the dt sequences part, and
the two modes then agree only to the scheme's accuracy: the mode is a
tolerance mode, not a bitwise one.
"""
import math

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import scenarios as S
from vfhelpers import hills_rect
from test_oracle_kats import LAKES

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-12  # relative to the state's max-norm (max |w|)


def _run(sc, mode, steps):
    sim = sc.build(vf.SM103Backend(np.float64, arithmetic=mode))
    dts = []
    for _ in range(steps):
        vf.perform_step(sim, math.inf)
        dts.append(vf.current_timestep(sim))
    return sim, np.asarray(dts), vf.current_interior_state(sim)


@pytest.mark.parametrize("make,steps", [
    (lambda: S.hills_wet_dry(256), 300),
    (lambda: hills_rect(97, 45), 80),
    (lambda: S.circular_dam_break(128), 100),
])
def test_faithful_within_tolerance_of_reference(make, steps):
    sc = make()
    _, dt_ref, ref = _run(sc, "reference", steps)
    _, dt_fast, fast = _run(sc, "faithful", steps)
    scale = np.abs(ref.h).max()
    assert np.abs(dt_fast - dt_ref).max() <= STATE_TOL * dt_ref.max()
    for name, a, b in zip(("h", "hu", "hv"), (fast.h, fast.hu, fast.hv), (ref.h, ref.hu, ref.hv)):
        assert np.abs(a - b).max() <= STATE_TOL * scale, name
    # the faithful kernels are not the reference-rounded ones
    assert not (np.array_equal(fast.hu, ref.hu) and np.array_equal(fast.hv, ref.hv))


@pytest.mark.parametrize("lake", ["step", "bumpy"])
def test_faithful_lake_at_rest(lake):
    """test/test_lake_at_rest_2d.jl:97-119 in faithful arithmetic: max |hu|, |hv| <= 1e-14, w unchanged to 1e-14."""
    sc, T = LAKES[lake]()
    sim = sc.build(vf.SM103Backend(np.float64, arithmetic="faithful"))
    vf.simulate_to_time(sim, T)
    g = vf.current_interior_state(sim)
    assert np.abs(g.hu).max() <= 1e-14 and np.abs(g.hv).max() <= 1e-14
    assert np.abs(g.h - 0.7).max() <= 1e-14


def test_set_arithmetic_rejects_float32_and_unknown_modes():
    sc = S.circular_dam_break(32)
    with pytest.raises(vf.ArgumentError):
        vf.SM103Backend(np.float32, arithmetic="faithful")
    sim = sc.build(vf.SM103Backend(np.float32))
    lib = sim._lib
    assert lib.vf_set_arithmetic(sim.handle, 1) != 0
    assert lib.vf_set_arithmetic(sim.handle, 0) == 0
    sim64 = sc.build(vf.SM103Backend(np.float64))
    assert sim64._lib.vf_set_arithmetic(sim64.handle, 7) != 0
    assert sim64._lib.vf_set_arithmetic(sim64.handle, 1) == 0
