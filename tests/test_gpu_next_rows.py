"""PeriodicBC, NoReconstruction, TimeDependentRain, HortonInfiltration and FunctionalRain on
the GPU: bitwise Float64 parity with the oracle and the reference's known answers."""
import math

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import scenarios as S
from vfhelpers import oracle_from, hills_rect
from test_gpu_parity import assert_bitwise
from test_oracle_kats import check_symmetry
from test_oracle_next_rows import (TIME_RAIN, dry_circle_periodic, flat_lake, functional, horton_case,
                                   no_reconstruction_case, spatial_rain_fn, timedependent_rain_fn)

pytestmark = pytest.mark.gpu


def run_pair(sc, steps, real=np.float64):
    sim = sc.build(vf.SM103Backend(real))
    ora = oracle_from(sc)
    for k in range(steps):
        vf.perform_step(sim, math.inf)
        dt = ora.perform_step(math.inf)
        sim.t += sim.current_timestep
        ora.o.t = ora.o.t + dt
        if real == np.float64:
            assert sim.current_timestep == dt, f"dt differs at step {k}"
    return sim, ora


def terrain_sources(nx, ny, **kw):
    """Wet/dry terrain with friction and the time- and cell-dependent sources."""
    sc = hills_rect(nx, ny, **kw)
    grid = sc.grid()
    f = vf.cell_centers(grid, interior=False)
    factor = 0.5 + 0.5 * (np.sin(f[:, :, 0] / 7.0) ** 2)
    sc.sources = [vf.SourceTermBottom(),
                  vf.TimeDependentRain(np.array([40.0, 5.0, 60.0]), np.array([0.0, 0.5, 1.0])),
                  vf.HortonInfiltration(grid, vf.SM103Backend(), factor=factor, f0=2e-3, fc=1e-4, k=0.8)]
    return sc


CASES = {
    "dry_circle_periodic_rk2": (lambda: dry_circle_periodic(64), 80),
    "hills_periodic_rk2": (lambda: hills_rect(70, 45, bc="periodic"), 60),
    "hills_periodic_partial_tiles_fe": (lambda: hills_rect(37, 19, bc="periodic", stepper="fe"), 60),
    "no_reconstruction_bottom_fe": (lambda: no_reconstruction_case(bottom=True), 60),
    "no_reconstruction_terrain_rk2": (lambda: hills_rect(50, 41, reconstruction="none"), 60),
    "time_rain_and_horton_rk2": (lambda: terrain_sources(64, 48), 80),
    "time_rain_and_horton_periodic_fe": (lambda: terrain_sources(45, 33, bc="periodic", stepper="fe"), 80),
    "functional_rain_spatial_fe": (lambda: functional(spatial_rain_fn), 0),
    "hills_neumann_rk2": (lambda: hills_rect(70, 45, bc="neumann"), 60),
    "hills_neumann_partial_tiles_fe": (lambda: hills_rect(37, 19, bc="neumann", stepper="fe"), 60),
    "time_rain_and_horton_neumann_rk2": (lambda: terrain_sources(45, 33, bc="neumann"), 80),
    "dam_break_neumann_rk2": (lambda: S.Scenario(**{**S.circular_dam_break(64).__dict__, "bc": "neumann"}), 60),
    "no_reconstruction_neumann_fe": (lambda: hills_rect(41, 29, bc="neumann", reconstruction="none", stepper="fe"), 60),
    "hills_periodic_bh2021_nonpow2": (lambda: hills_rect(45, 35, bc="periodic", friction_law="bh2021",
                                                         extent=((0.0, 30.0), (0.0, 21.0))), 60),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_next_rows_bitwise(case):
    make, steps = CASES[case]
    sc = make()
    if steps == 0:  # FunctionalRain: step through the host loop to 3 h
        sim = sc.build(vf.SM103Backend())
        vf.simulate_to_time(sim, 3 * 3600.0)
        ora = oracle_from(sc)
        ora.simulate_to_time(3 * 3600.0)
        assert sim.t == ora.o.t
    else:
        sim, ora = run_pair(sc, steps)
    assert_bitwise(vf.current_interior_state(sim), ora.interior())


def test_dry_state_symmetry_periodic_gpu():
    # test/test_shallow_water_dry_states_2d.jl with its default PeriodicBC
    sim = dry_circle_periodic().build(vf.SM103Backend())
    vf.simulate_to_time(sim, 0.05)
    assert vf.current_time(sim) == 0.05
    g = vf.current_interior_state(sim)
    check_symmetry(g.h, g.hu, g.hv, 1e-12)


def test_horton_drawdown_gpu():
    # test/test_infiltration.jl:74-76 (the CUDA case)
    sc, inf = horton_case()
    sim = sc.build(vf.SM103Backend())
    vf.simulate_to_time(sim, 1e6 + 1000)
    g = vf.current_interior_state(sim)
    assert np.all(g.hu == 0.0) and np.all(g.hv == 0.0)
    assert abs(g.h.max() - (1.0 - inf.fc * 1000)) <= 1e-10 and abs(g.h.min() - (1.0 - inf.fc * 1000)) <= 1e-10


@pytest.mark.parametrize("hours,expected,tol", [(1, 1.015, 1e-12), (3, 1.0353, 1e-4)])
def test_time_dependent_rain_gpu(hours, expected, tol):
    # test/test_rain.jl:79-96 on the device time loop (100x100 as the CUDA cases)
    rain = vf.TimeDependentRain(TIME_RAIN["rates"], TIME_RAIN["times"])
    sim = flat_lake(100, ((0.0, 1000.0), (0.0, 1000.0)), [rain]).build(vf.SM103Backend())
    vf.simulate_to_time(sim, hours * 3600.0)
    g = vf.current_interior_state(sim)
    assert np.all(g.hu == 0.0) and np.all(g.hv == 0.0)
    assert abs(g.h.max() - expected) <= tol and abs(g.h.min() - expected) <= tol


def test_functional_rain_time_dependent_gpu():
    # test/test_rain.jl:123-131
    sim = functional(timedependent_rain_fn).build(vf.SM103Backend())
    vf.simulate_to_time(sim, 3 * 3600.0)
    h = vf.current_interior_state(sim).h
    assert abs(h.max() - 1.0353) <= 1e-4 and abs(h.min() - 1.0353) <= 1e-4


def test_float32_runs_the_new_rows():
    """Float32 at the same simulated time is as close to the Float64 oracle as the
    oracle's own plain Float32 restatement is (wet/dry fronts on steep terrain make
    both lose ~0.5%)."""
    sc = hills_rect(64, 48, bc="periodic")
    grid = sc.grid()
    f = vf.cell_centers(grid, interior=False)
    factor = 0.5 + 0.5 * (np.sin(f[:, :, 0] / 7.0) ** 2)
    sc.sources = [vf.SourceTermBottom(), vf.TimeDependentRain(np.array([0.2, 0.05, 0.3]), np.array([0.0, 0.5, 1.0])),
                  vf.HortonInfiltration(grid, vf.SM103Backend(), factor=factor)]
    T = 1.0
    s32 = sc.build(vf.SM103Backend(np.float32))
    vf.simulate_to_time(s32, T)
    o64, o32 = oracle_from(sc, 8), oracle_from(sc, 4)
    o64.simulate_to_time(T)
    o32.simulate_to_time(T)
    w64 = o64.interior()[0]
    err_ref = np.abs(o32.interior()[0] - w64).max()
    err = np.abs(vf.current_interior_state(s32).h - w64).max()
    assert err <= 2 * err_ref + 1e-5, (err, err_ref)
