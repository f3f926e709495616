"""The reference's tests for PeriodicBC, HortonInfiltration, TimeDependentRain,
FunctionalRain and NoReconstruction, run on the CPU oracle."""
import math
import random

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from oracle import vf_oracle as O
from volumefluxes_sm103 import scenarios as S
from vfhelpers import oracle_from
from test_oracle_kats import check_symmetry


@pytest.fixture(scope="module")
def lib():
    return O.load()


def test_periodic_bc_mapping(lib):
    # test/test_periodic_bc_2d.jl:26-66 (gc = 2)
    nx, ny, gc = 11, 8, 2
    N1, N2 = nx + 2 * gc, ny + 2 * gc
    u = -42.0 * np.ones((3, N1, N2))
    for j in range(gc, ny + gc):
        for i in range(gc, nx + gc):
            u[:, i, j] = (j + 1) * nx + (i + 1)
    buf = np.ascontiguousarray(u.transpose(0, 2, 1)).reshape(-1)
    assert lib.vfo_update_bc_periodic(buf.ctypes.data, nx, ny, gc) == 0
    out = buf.reshape(3, N2, N1).transpose(0, 2, 1)
    I = slice(gc, nx + gc)
    J = slice(gc, ny + gc)
    assert np.array_equal(out[:, I, J], u[:, I, J])
    for n in range(1, gc + 1):
        # 1-based: output[i, n] == output[i, end-(gc-n+1)-gc+1]; output[i, end-(gc-n)] == output[i, gc+n]
        assert np.array_equal(out[:, I, n - 1], out[:, I, N2 - (gc - n + 1) - gc])
        assert np.array_equal(out[:, I, N2 - (gc - n) - 1], out[:, I, gc + n - 1])
        assert np.array_equal(out[:, n - 1, J], out[:, N1 - (gc - n + 1) - gc, J])
        assert np.array_equal(out[:, N1 - (gc - n) - 1, J], out[:, gc + n - 1, J])
    assert out[0, 0, 0] == -42.0  # corners untouched


def test_deterministic_exp_accuracy(lib):
    rng = random.Random(5)
    xs = [0.0, -1.0, 1.0, -2.43e-3 * 1e6, -2.43e-3 * 1000.0, 709.0, -700.0, -744.0]
    xs += [rng.uniform(-50, 50) for _ in range(2000)] + [rng.uniform(-745, 709) for _ in range(500)]
    for x in xs:
        got, want = lib.vfo_exp(x), math.exp(x)
        if want == 0.0:
            assert got <= 5e-324 * 4
            continue
        assert abs(got - want) <= 2 * math.ulp(want), x


def dry_circle_periodic(n=64):
    # test/test_shallow_water_dry_states_2d.jl:31-53: CartesianGrid(64, 64; gc=2) defaults to PeriodicBC
    grid = vf.CartesianGrid(n, n, gc=2)
    c = vf.cell_centers(grid)
    r2 = (c[:, :, 0] - 0.5) ** 2 + (c[:, :, 1] - 0.5) ** 2
    w = 1 - np.sign(r2 - 0.01)
    z = np.zeros_like(w)
    return S.Scenario(name="dry_circle_periodic", nx=n, ny=n, extent=((0.0, 1.0), (0.0, 1.0)), B=None, w0=w,
                      hu0=z, hv0=z.copy(), cfl=0.25, bc="periodic")


def test_dry_state_symmetry_periodic():
    o = oracle_from(dry_circle_periodic())
    o.simulate_to_time(0.05)
    assert o.t == 0.05
    check_symmetry(*o.interior(), 1e-12)


def flat_lake(nx, extent, sources, bc="wall", t0=0.0, stepper="fe"):
    w = np.ones((nx, nx))
    z = np.zeros_like(w)
    return S.Scenario(name="flat", nx=nx, ny=nx, extent=extent, B=None, w0=w, hu0=z, hv0=z.copy(), cfl=0.25,
                      stepper=stepper, sources=sources, bc=bc, t0=t0)


def horton_case():
    # test/test_infiltration.jl:29-76: 10x10, gc=2, extent [0,100]^2, default (periodic) BC, t0 = 1e6
    grid = vf.CartesianGrid(10, 10, gc=2, extent=[[0.0, 100.0], [0.0, 100.0]])
    inf = vf.HortonInfiltration(grid, vf.SM103Backend())
    return flat_lake(10, ((0.0, 100.0), (0.0, 100.0)), [inf], bc="periodic", t0=1e6), inf


def test_horton_infiltration_drawdown():
    sc, inf = horton_case()
    assert np.all(inf.factor == 1.0) and inf.factor.shape == (14, 14)
    assert vf.compute_infiltration(inf, 0.0, (1, 1)) == inf.f0
    assert vf.compute_infiltration(inf, 1e6, (1, 1)) == inf.fc
    o = oracle_from(sc)
    o.simulate_to_time(1e6 + 1000)
    h, hu, hv = o.interior()
    assert np.all(hu == 0.0) and np.all(hv == 0.0)
    assert abs(h.max() - (1.0 - inf.fc * 1000)) <= 1e-10 and abs(h.min() - (1.0 - inf.fc * 1000)) <= 1e-10


def test_horton_factor_validation():
    # test/test_infiltration.jl:63-64
    with pytest.raises(vf.DomainError):
        vf.HortonInfiltration(vf.CartesianGrid(2, 2), vf.SM103Backend(), factor=np.ones((2, 2)))


TIME_RAIN = dict(rates=np.array([15.0, 0.3, 20.0]) * 0.001, times=np.array([0.0, 1.0, 2.0]) * 3600)


def test_time_dependent_rain_lookup():
    # test/test_rain.jl:61-66
    r = vf.TimeDependentRain(TIME_RAIN["rates"], TIME_RAIN["times"])
    assert vf.compute_rain(r, 10) == 0.015 / 3600.0
    assert vf.compute_rain(r, 3610) == 0.0003 / 3600.0
    assert vf.compute_rain(r, 7210) == 0.02 / 3600.0
    assert vf.compute_rain(r, 1.0e6) == 0.02 / 3600.0
    assert vf.compute_rain(r, 0.0) == 0.015 / 3600.0
    with pytest.raises(vf.DomainError):
        vf.TimeDependentRain([1.0, 2.0], [0.0])


@pytest.mark.parametrize("hours,expected,tol", [(1, 1.015, 1e-12), (2, 1.0153, 1e-4), (3, 1.0353, 1e-4)])
def test_time_dependent_rain_accumulation(hours, expected, tol):
    # test/test_rain.jl:79-90 (10x10 wall grid over [0,1000]^2, forward Euler)
    rain = vf.TimeDependentRain(TIME_RAIN["rates"], TIME_RAIN["times"])
    o = oracle_from(flat_lake(10, ((0.0, 1000.0), (0.0, 1000.0)), [rain]))
    o.simulate_to_time(hours * 3600.0)
    h, hu, hv = o.interior()
    assert np.all(hu == 0.0) and np.all(hv == 0.0)
    assert abs(h.max() - expected) <= tol and abs(h.min() - expected) <= tol


def functional(fn):
    grid = vf.CartesianGrid(10, 10, gc=2, boundary=vf.WallBC(), extent=[[0.0, 1000.0], [0.0, 1000.0]])
    return flat_lake(10, ((0.0, 1000.0), (0.0, 1000.0)), [vf.FunctionalRain(fn, grid)])


def constant_rain_fn(t, x, y):
    return 0.01 / 3600.0 + 0 * x


def timedependent_rain_fn(t, x, y):
    rate = 15.0 * 0.001 if t < 3600 else (0.3 * 0.001 if t < 7200 else 20.0 * 0.001)
    return rate / 3600 + 0 * x


def spatial_rain_fn(t, x, y):
    if 3600.0 < t < 7200.0:
        return 3 * (x / 500) * (y / 500) * 0.01 / 3600.0
    return 0.0 * x


def test_functional_rain():
    # test/test_rain.jl:98-146
    o = oracle_from(functional(constant_rain_fn))
    o.simulate_to_time(3 * 3600.0)
    h1 = o.interior()[0]
    assert abs(h1.max() - 1.03) <= 1e-12 and abs(h1.min() - 1.03) <= 1e-12
    o = oracle_from(functional(timedependent_rain_fn))
    o.simulate_to_time(3 * 3600.0)
    h3 = o.interior()[0]
    assert abs(h3.max() - 1.0353) <= 1e-4 and abs(h3.min() - 1.0353) <= 1e-4
    o = oracle_from(functional(spatial_rain_fn))
    o.simulate_to_time(3 * 3600.0)
    h5 = o.interior()[0]
    assert abs(h5.sum() - h1.sum()) <= 1e-2


def no_reconstruction_case(bottom: bool):
    grid = vf.CartesianGrid(32, 24, gc=2, boundary=vf.WallBC(), extent=[[0.0, 32.0], [0.0, 24.0]])
    f = vf.cell_faces(grid, interior=False)
    B = 0.1 * np.sin(f[:, :, 0] / 5.0) * np.cos(f[:, :, 1] / 7.0) if bottom else None
    Bc = 0.0 if B is None else 0.25 * (B[:-1, :-1] + B[1:, :-1] + B[:-1, 1:] + B[1:, 1:])[2:-2, 2:-2]
    w = np.maximum(1.0, Bc) + 0.2 * (np.arange(32)[:, None] < 8) * np.ones((32, 24))
    z = np.zeros_like(w)
    return S.Scenario(name="norec", nx=32, ny=24, extent=((0.0, 32.0), (0.0, 24.0)), B=B, w0=w, hu0=z, hv0=z.copy(),
                      cfl=0.25, stepper="fe", reconstruction="none", bottom_source=bottom)


def test_no_reconstruction_conserves_mass_on_a_flat_bottom():
    # With a sloping bottom the mirrored wall ghost keeps w but not B_cell, so the
    # reference moves water through the wall (src/reconstruction/noreconstruction.jl:42-45);
    # on a flat bottom the first-order scheme is conservative.
    o = oracle_from(no_reconstruction_case(bottom=False))
    v0 = o.interior()[0].sum()
    for _ in range(40):
        o.perform_step(math.inf)
    h, hu, hv = o.interior()
    assert np.all(np.isfinite(h)) and abs(h.sum() - v0) <= 1e-12 * v0


def test_neumann_bc_mapping_as_the_reference_writes_it(lib):
    # src/bc.jl:49-60 (gc = 2): left columns mirror the interior; right columns
    # copy ghost onto ghost; bottom rows take the top interior rows; top rows
    # copy ghost onto ghost. Corners untouched.
    nx, ny, gc = 9, 7, 2
    N1, N2 = nx + 2 * gc, ny + 2 * gc
    rng = np.random.default_rng(3)
    u = rng.standard_normal((3, N1, N2))
    buf = np.ascontiguousarray(u.transpose(0, 2, 1)).reshape(-1)
    assert lib.vfo_update_bc_neumann(buf.ctypes.data, nx, ny, gc) == 0
    out = buf.reshape(3, N2, N1).transpose(0, 2, 1)
    I, J = slice(gc, nx + gc), slice(gc, ny + gc)
    assert np.array_equal(out[:, I, J], u[:, I, J])
    assert np.array_equal(out[:, 0, J], u[:, 3, J]) and np.array_equal(out[:, 1, J], u[:, 2, J])
    assert np.array_equal(out[:, N1 - 2, J], u[:, N1 - 1, J]) and np.array_equal(out[:, N1 - 1, J], u[:, N1 - 1, J])
    assert np.array_equal(out[:, I, 0], u[:, I, N2 - 4]) and np.array_equal(out[:, I, 1], u[:, I, N2 - 3])
    assert np.array_equal(out[:, I, N2 - 2], u[:, I, N2 - 1]) and np.array_equal(out[:, I, N2 - 1], u[:, I, N2 - 1])
    assert out[0, 0, 0] == u[0, 0, 0] and out[0, N1 - 1, N2 - 1] == u[0, N1 - 1, N2 - 1]


def test_neumann_outflow_runs_and_stays_finite():
    from vfhelpers import hills_rect
    o = oracle_from(hills_rect(40, 30, bc="neumann"))
    for _ in range(30):
        o.perform_step(math.inf)
    h, hu, hv = o.interior()
    assert np.all(np.isfinite(h)) and np.all(np.isfinite(hu)) and np.all(np.isfinite(hv))
