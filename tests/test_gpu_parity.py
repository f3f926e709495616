"""Float64 parity of the sm_103a step with the oracle, bit for bit, through the C ABI.

Every case runs the same scenario in the library (via the reference-mirroring
API) and in the oracle, one perform_step at a time, and requires identical dt
sequences and identical interior fields. The stated tolerance for Float64 is
1e-12 relative (max-norm); the kernels reach 0. Float32 runs state their error
against the Float64 oracle.
"""
import math

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import scenarios as S
from vfhelpers import oracle_from, hills_rect, max_rel
from test_oracle_kats import LAKES, dry_circle, check_symmetry, swashes_dam, _flat

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12  # relative max-norm, per field


def run_pair(sc, steps, real=np.float64):
    sim = sc.build(vf.SM103Backend(real))
    ora = oracle_from(sc)
    for k in range(steps):
        vf.perform_step(sim, math.inf)
        dt = ora.perform_step(math.inf)
        if real == np.float64:
            assert vf.current_timestep(sim) == dt, f"dt differs at step {k}"
    got = vf.current_interior_state(sim)
    want = ora.interior()
    return sim, ora, got, want


def assert_bitwise(got, want):
    for name, a, b in zip(("h", "hu", "hv"), (got.h, got.hu, got.hv), want):
        assert max_rel(a, b) <= F64_TOL, name
        assert np.array_equal(a, b), f"{name}: {int((a != b).sum())} cells differ, max |d| {np.abs(a - b).max()}"


def nonsquare_step(nx=13, ny=7):
    w = np.where(np.arange(nx)[:, None] < nx // 3, 2.0, 1.0) * np.ones((nx, ny))
    w[:, ny // 2:] += 0.25
    z = np.zeros_like(w)
    return S.Scenario(name="step", nx=nx, ny=ny, extent=((0.0, 1.0), (0.0, 0.7)), B=None, w0=w, hu0=z, hv0=z.copy(),
                      cfl=0.2)


CASES = {
    # name: (scenario factory, steps)
    "dam_break_256_rk2": (lambda: S.circular_dam_break(256), 200),          # the small configuration, 200 steps
    "partial_tiles_13x7": (lambda: nonsquare_step(13, 7), 60),
    "partial_tiles_33x17": (lambda: nonsquare_step(33, 17), 60),
    "min_grid_2x2": (lambda: nonsquare_step(2, 2), 20),
    "strip_1x_200x2": (lambda: nonsquare_step(200, 2), 40),
    "hills_97x45_all_sources": (lambda: hills_rect(97, 45), 80),
    "hills_96x96_forward_euler": (lambda: hills_rect(96, 96, stepper="fe"), 60),
    "hills_64x48_fcg2016": (lambda: hills_rect(64, 48, friction_law="fcg2016"), 60),
    "hills_64x48_bh2021": (lambda: hills_rect(64, 48, friction_law="bh2021"), 60),
    "hills_65x33_rain_then_infiltration": (lambda: hills_rect(65, 33, rain_m_per_h=3.6, infiltration_m_per_s=1e-3), 60),
    "hills_130x70_no_friction": (lambda: hills_rect(130, 70, manning_n=None), 60),
    "dry_circle_64_rk2": (lambda: dry_circle(64), 80),
    "eq_params_rho_g_cutoff": (lambda: hills_rect(40, 40, eq={"rho": 1.5, "g": 3.7, "depth_cutoff": 1e-4,
                                                            "desingularizing_kappa": 1e-6}, theta=1.7), 60),
    # cell sizes that are not powers of two: 1/Δ * (F_r - F_l) rounds and ΔB/Δ is a division
    "hills_50x30_nonpow2_cells": (lambda: hills_rect(50, 30, extent=((0.0, 37.0), (0.0, 23.0))), 60),
}


@pytest.mark.parametrize("variant", ["march", "tile"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_parity_bitwise(case, variant, monkeypatch):
    """Both kernel designs: column-marching (default) and shared-memory tiles (VF_KERNELS=tile)."""
    monkeypatch.setenv("VF_KERNELS", variant)
    make, steps = CASES[case]
    _, _, got, want = run_pair(make(), steps)
    assert_bitwise(got, want)


@pytest.mark.parametrize("case", sorted(LAKES))
def test_lake_at_rest_gpu(case):
    # test/test_lake_at_rest_2d.jl:97-98, plus bitwise agreement with the oracle
    sc, T = LAKES[case]()
    sim = sc.build(vf.SM103Backend())
    vf.simulate_to_time(sim, T)
    got = vf.current_interior_state(sim)
    assert np.abs(got.hu).max() <= 1e-14 and np.abs(got.hv).max() <= 1e-14
    assert np.abs(got.h - 0.7).max() <= 1e-14
    ora = oracle_from(sc)
    ora.simulate_to_time(T)
    assert sim.t == ora.t
    assert_bitwise(got, ora.interior())


def test_rain_accumulation_gpu():
    # test/test_rain.jl:68-78 (the CUDA case uses the 100x100 grid)
    sc = _flat(100, ((0.0, 1000.0), (0.0, 1000.0)), rain_m_per_h=0.01)
    sim = sc.build(vf.SM103Backend())
    vf.simulate_to_time(sim, 3 * 3600)
    assert abs(vf.current_time(sim) - 3 * 3600) <= 1e-10
    got = vf.current_interior_state(sim)
    assert np.all(got.hu == 0.0) and np.all(got.hv == 0.0)
    assert abs(got.h.max() - 1.03) <= 1e-12 and abs(got.h.min() - 1.03) <= 1e-12


def test_infiltration_drawdown_gpu():
    fc = 3.272e-5
    sc = _flat(10, ((0.0, 100.0), (0.0, 100.0)), infiltration_m_per_s=fc)
    sim = sc.build(vf.SM103Backend())
    vf.simulate_to_time(sim, 1000.0)
    got = vf.current_interior_state(sim)
    assert np.all(got.hu == 0.0) and np.all(got.hv == 0.0)
    assert abs(got.h.max() - (1.0 - fc * 1000)) <= 1e-10 and abs(got.h.min() - (1.0 - fc * 1000)) <= 1e-10


def test_dry_state_symmetry_gpu():
    sim = dry_circle(64).build(vf.SM103Backend())
    vf.simulate_to_time(sim, 0.05)
    assert vf.current_time(sim) == 0.05
    g = vf.current_interior_state(sim)
    check_symmetry(g.h, g.hu, g.hv, 1e-12)


@pytest.mark.parametrize("wet", [True, False])
def test_x_and_y_dam_breaks_bitwise_equal_gpu(wet):
    # test/test_swashes.jl:317-327
    sx = swashes_dam(512, wet, False).build(vf.SM103Backend())
    sy = swashes_dam(512, wet, True).build(vf.SM103Backend())
    vf.simulate_to_time(sx, 4.0)
    vf.simulate_to_time(sy, 4.0)
    assert sx.current_timestep == sy.current_timestep and sx.t == sy.t
    gx, gy = vf.current_interior_state(sx), vf.current_interior_state(sy)
    assert np.all(gx.hv == 0) and np.all(gy.hu == 0)
    assert np.array_equal(gx.h[:, 1], gy.h[1, :]) and np.array_equal(gx.hu[:, 1], gy.hv[1, :])


def test_wall_bc_mapping_gpu():
    # test/test_update_bc.jl:71-116 through set_current_state! on the device
    nx, ny = 10, 5
    grid = vf.CartesianGrid(nx, ny, gc=2, boundary=vf.WallBC())
    eq = vf.ShallowWaterEquations()
    be = vf.SM103Backend()
    sim = vf.Simulator(be, vf.ConservedSystem(be, vf.LinearReconstruction(), vf.CentralUpwind(eq), eq, grid),
                       vf.RungeKutta2(), grid)
    x = vf.cell_centers(grid)
    vf.set_current_state(sim, (x[:, :, 0], (x[:, :, 0] + x[:, :, 1]) * 10, x[:, :, 0] * (x[:, :, 1] - 5)))
    st = vf.current_state(sim)
    u = np.stack([st.h, st.hu, st.hv])
    I = slice(2, -2)
    for k, sx, sy in ((0, 1, 1), (1, -1, 1), (2, 1, -1)):
        assert np.array_equal(u[k, 1, I], sx * u[k, 2, I]) and np.array_equal(u[k, 0, I], sx * u[k, 3, I])
        assert np.array_equal(u[k, nx + 3, I], sx * u[k, nx, I]) and np.array_equal(u[k, nx + 2, I], sx * u[k, nx + 1, I])
        assert np.array_equal(u[k, I, 1], sy * u[k, I, 2]) and np.array_equal(u[k, I, 0], sy * u[k, I, 3])
        assert np.array_equal(u[k, I, ny + 3], sy * u[k, I, ny]) and np.array_equal(u[k, I, ny + 2], sy * u[k, I, ny + 1])


def test_ghosts_after_steps_match_oracle():
    sc = hills_rect(37, 29)
    sim, ora, _, _ = run_pair(sc, 30)
    st = vf.current_state(sim)
    want = ora.state()
    N1, N2 = sim.grid.size()
    mask = np.ones((N1, N2), bool)
    for a in (0, 1, N1 - 2, N1 - 1):
        for b in (0, 1, N2 - 2, N2 - 1):
            mask[a, b] = False  # corner ghosts are never read or written by the scheme
    for a, b in zip((st.h, st.hu, st.hv), want):
        assert np.array_equal(a[mask], b[mask])


@pytest.mark.parametrize("case,tol", [("dam", 2e-6), ("hills", 5e-4)])
def test_float32_error_against_float64_oracle(case, tol):
    """Float32 state: max-norm error relative to each field's scale, after the stated steps."""
    sc = S.circular_dam_break(256) if case == "dam" else hills_rect(128, 96, manning_n=None, rain_m_per_h=None,
                                                                     infiltration_m_per_s=None)
    steps = 200 if case == "dam" else 100
    sim = sc.build(vf.SM103Backend(np.float32))
    ora = oracle_from(sc)
    for _ in range(steps):
        vf.perform_step(sim, math.inf)
        ora.perform_step(math.inf)
    g = vf.current_interior_state(sim)
    w, hu, hv = ora.interior()
    assert max_rel(g.h, w) <= tol
    scale = max(np.abs(hu).max(), np.abs(hv).max())
    assert np.abs(g.hu - hu).max() <= 50 * tol * scale and np.abs(g.hv - hv).max() <= 50 * tol * scale


def test_time_order_of_the_steppers_gpu():
    # test/test_timesteppers.jl:70-87 on the device: forward Euler first order,
    # RK2 second order in time, with every step forced to the same dt
    from test_oracle_kats import smooth_bump, time_order

    def run(stepper, dt, T):
        sc = smooth_bump()
        sc.stepper = stepper
        sim = sc.build(vf.SM103Backend(np.float64))
        for _ in range(int(round(T / dt))):
            vf.perform_step(sim, dt)
            sim.t += sim.current_timestep
        w = vf.current_interior_state(sim).h.copy()
        sim.close()
        return w

    order = time_order(run)
    assert order["rk2"] == pytest.approx(2.0, abs=0.05)
    assert order["fe"] == pytest.approx(1.0, abs=0.1)
