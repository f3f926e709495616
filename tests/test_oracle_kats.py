"""The reference's own known-answer and property tests for this path, run on the CPU oracle.

These pin the oracle to VolumeFluxes.jl: the reference stores no golden fields,
so its test assertions (cited per test) are the anchor.
"""
import ctypes
import math
import random
from decimal import Decimal, getcontext

import numpy as np
import pytest

from oracle import vf_oracle as O
from vfhelpers import oracle_from
import volumefluxes_sm103 as vf
from volumefluxes_sm103 import scenarios as S


@pytest.fixture(scope="module")
def lib():
    return O.load()


def test_minmod_kats(lib):
    # test/test_minmod.jl:24-27
    assert lib.vfo_minmod(1, 2, 3) == 1
    assert lib.vfo_minmod(-1, -2, -3) == -1
    assert lib.vfo_minmod(1, -2, 3) == 0
    got = [lib.vfo_minmod(a, b, c) for a, b, c in zip([1, -2, -3], [3, -5, 2], [4, -3, 4])]
    assert got == [1, -2, 0]
    assert list(vf.minmod([1, -2, -3], [3, -5, 2], [4, -3, 4])) == [1, -2, 0]


def test_minmod_slope_definition(lib):
    # src/reconstruction/linearreconstruction.jl:37-43
    rng = random.Random(3)
    for _ in range(200):
        l, c, r = (rng.uniform(-2, 2) for _ in range(3))
        th = rng.choice([1.0, 1.2, 2.0])
        fwd, bwd = r - c, c - l
        want = lib.vfo_minmod(th * fwd, (fwd + bwd) / 2.0, th * bwd)
        assert lib.vfo_minmod_slope(l, c, r, th) == want


def _bottom_2x2():
    grid = vf.CartesianGrid(2, 2, gc=2, extent=[[0.0, 12.0], [0.0, 20.0]])
    f = vf.cell_faces(grid, interior=False)
    return grid, f[:, :, 0] + f[:, :, 1]


def test_bottom_topography_kats(lib):
    # test/test_bottom_topography.jl:77-109 (2D part)
    grid, B = _bottom_2x2()
    Bc = np.ascontiguousarray(B.T)
    W, H = B.shape
    look = lambda i, j, w: lib.vfo_bottom_lookup(Bc.ctypes.data, W, H, i, j, w)
    tol = 1e-10
    assert abs(look(3, 3, 0) - 8) < tol and abs(look(3, 4, 0) - 18) < tol
    assert abs(look(4, 3, 0) - 14) < tol and abs(look(4, 4, 0) - 24) < tol
    assert abs(look(3, 3, 1) - 5) < tol and abs(look(3, 3, 2) - 11) < tol
    assert abs(look(3, 3, 3) - 3) < tol and abs(look(3, 3, 4) - 13) < tol
    assert abs(look(4, 4, 1) - 21) < tol and abs(look(4, 4, 2) - 27) < tol
    assert abs(look(4, 4, 3) - 19) < tol and abs(look(4, 4, 4) - 29) < tol
    assert look(3, 4, 2) == look(4, 4, 1)
    assert look(4, 3, 4) == look(4, 4, 3)
    # the host API computes the same lookups
    bt = vf.BottomTopography2D(B, vf.SM103Backend(), grid)
    assert vf.B_cell(bt, 3, 3) == look(3, 3, 0)
    assert vf.B_face_left(bt, 4, 4, vf.XDIR) == look(4, 4, 1)
    assert vf.B_face_right(bt, 4, 4, vf.YDIR) == look(4, 4, 4)


def test_bottom_topography_validation():
    # test/test_bottom_topography.jl:58-59: wrong size is a DomainError
    grid, B = _bottom_2x2()
    with pytest.raises(vf.DomainError):
        vf.BottomTopography2D(B[1:, :], vf.SM103Backend(), grid)
    assert not vf.is_zero(vf.BottomTopography2D(B, vf.SM103Backend(), grid))
    assert vf.is_zero(vf.BottomTopography2D(np.zeros_like(B), vf.SM103Backend(), grid))
    assert vf.is_zero(vf.ConstantBottomTopography())
    assert not vf.is_zero(vf.ConstantBottomTopography(3.14))


def test_wall_bc_mapping(lib):
    # test/test_update_bc.jl:71-116
    nx, ny = 10, 5
    grid = vf.CartesianGrid(nx, ny, gc=2, boundary=vf.WallBC())
    x = vf.cell_centers(grid, interior=False)
    N1, N2 = grid.size()
    u = np.stack([x[:, :, 0], (x[:, :, 0] + x[:, :, 1]) * 10, x[:, :, 0] * (x[:, :, 1] - 5)], axis=0)
    orig = u.copy()
    buf = np.ascontiguousarray(u.transpose(0, 2, 1)).reshape(-1)
    assert lib.vfo_update_bc_wall(buf.ctypes.data, nx, ny, 2) == 0
    u = buf.reshape(3, N2, N1).transpose(0, 2, 1)
    I = slice(2, -2)
    assert np.array_equal(u[:, I, I], orig[:, I, I])
    for k, sx, sy in ((0, 1, 1), (1, -1, 1), (2, 1, -1)):
        assert np.array_equal(u[k, 1, I], sx * u[k, 2, I]) and np.array_equal(u[k, 0, I], sx * u[k, 3, I])
        assert np.array_equal(u[k, nx + 3, I], sx * u[k, nx, I]) and np.array_equal(u[k, nx + 2, I], sx * u[k, nx + 1, I])
        assert np.array_equal(u[k, I, 1], sy * u[k, I, 2]) and np.array_equal(u[k, I, 0], sy * u[k, I, 3])
        assert np.array_equal(u[k, I, ny + 3], sy * u[k, I, ny]) and np.array_equal(u[k, I, ny + 2], sy * u[k, I, ny + 1])
    # corner ghosts are never touched
    assert np.array_equal(u[:, :2, :2], orig[:, :2, :2])


def _exact_cbrt_rounded(x: float) -> float:
    """Nearest double to cbrt(x), by exact Decimal arithmetic and neighbour comparison."""
    getcontext().prec = 80
    X = Decimal(x)
    y = float(X ** (Decimal(1) / Decimal(3)))
    best, err = y, None
    for cand in (math.nextafter(y, -math.inf), y, math.nextafter(y, math.inf)):
        e = abs(Decimal(cand) ** 3 - X)
        if err is None or e < err:
            best, err = cand, e
    return best


def test_cbrt_correctly_rounded(lib):
    rng = random.Random(11)
    xs = [1.0, 8.0, 27.0, 2.0, 0.001, 1e-5, 5e-6, 3.0e-300, 5e-324, 1e300, 7.9999999999999991]
    xs += [rng.uniform(1e-6, 10.0) for _ in range(400)] + [10 ** rng.uniform(-300, 300) for _ in range(200)]
    for x in xs:
        want = _exact_cbrt_rounded(x)
        assert lib.vfo_cbrt(x) == want, x
        assert lib.vfo_cbrt(-x) == -want
    assert lib.vfo_cbrt(0.0) == 0.0 and math.copysign(1, lib.vfo_cbrt(-0.0)) == -1


def test_desingularize(lib):
    # src/equations/equation.jl:56
    eq = vf.ShallowWaterEquations()
    k = eq.desingularizing_kappa
    for h in (0.0, -0.0, 1e-7, 5e-6, 1e-5, 2e-5, 1.0, -3e-6, -1.0):
        assert lib.vfo_desingularize(h, k) == vf.desingularize(eq, h)
    assert lib.vfo_desingularize(0.0, k) == k / 2


def _lake(nx, extent, Bfun, w0=0.7, T=0.01):
    grid = vf.CartesianGrid(nx, nx, gc=2, boundary=vf.WallBC(), extent=extent)
    f = vf.cell_faces(grid, interior=False)
    B = Bfun(f[:, :, 0], f[:, :, 1])
    w = np.full((nx, nx), w0)
    z = np.zeros_like(w)
    sc = S.Scenario(name="lake", nx=nx, ny=nx, extent=tuple(map(tuple, extent)), B=B, w0=w, hu0=z, hv0=z.copy(),
                    cfl=0.2, stepper="fe", theta=2.0, bottom_source=True)
    return sc, T


LAKES = {
    # test/test_lake_at_rest_2d.jl:102-119
    "step": lambda: _lake(64, [[0.0, 10.0], [0.0, 10.0]], lambda x, y: np.where((x < 5.0) & (y < 5.0), 0.45, 0.55)),
    "bumpy": lambda: _lake(124, [[-2 * np.pi, 2 * np.pi], [-2 * np.pi, 2 * np.pi]],
                           lambda x, y: np.cos(x + y) - 0.5 - 1.5 * (np.sqrt(x * x + y * y) < 1.0)),
}


@pytest.mark.parametrize("case", sorted(LAKES))
def test_lake_at_rest(case):
    sc, T = LAKES[case]()
    o = oracle_from(sc)
    o.simulate_to_time(T)
    w, hu, hv = o.interior()
    assert np.abs(hu).max() <= 1e-14 and np.abs(hv).max() <= 1e-14
    assert np.abs(w - 0.7).max() <= 1e-14


def _flat(nx, extent, **kw):
    w = np.ones((nx, nx))
    z = np.zeros_like(w)
    args = dict(name="flat", nx=nx, ny=nx, extent=extent, B=None, w0=w, hu0=z, hv0=z.copy(), cfl=0.25, stepper="fe")
    args.update(kw)
    return S.Scenario(**args)


def test_rain_accumulation():
    # test/test_rain.jl:68-77: ConstantRain(0.01) for 3 h on a 10x10 lake
    sc = _flat(10, ((0.0, 1000.0), (0.0, 1000.0)), rain_m_per_h=0.01)
    o = oracle_from(sc)
    o.simulate_to_time(3 * 3600)
    assert abs(o.t - 3 * 3600) <= 1e-10
    w, hu, hv = o.interior()
    assert np.all(hu == 0.0) and np.all(hv == 0.0)
    assert abs(w.max() - (3 * 0.01 + 1.0)) <= 1e-12 and abs(w.min() - (3 * 0.01 + 1.0)) <= 1e-12


def test_infiltration_drawdown():
    # test/test_infiltration.jl:70-72 with the long-time Horton rate fc as a constant rate
    fc = 3.272e-5
    sc = _flat(10, ((0.0, 100.0), (0.0, 100.0)), infiltration_m_per_s=fc)
    o = oracle_from(sc)
    o.simulate_to_time(1000.0)
    w, hu, hv = o.interior()
    assert np.all(hu == 0.0) and np.all(hv == 0.0)
    assert abs(w.max() - (1.0 - fc * 1000)) <= 1e-10 and abs(w.min() - (1.0 - fc * 1000)) <= 1e-10


def dry_circle(n=64):
    grid = vf.CartesianGrid(n, n, gc=2, boundary=vf.WallBC())
    c = vf.cell_centers(grid)
    r2 = (c[:, :, 0] - 0.5) ** 2 + (c[:, :, 1] - 0.5) ** 2
    w = 1 - np.sign(r2 - 0.01)
    z = np.zeros_like(w)
    return S.Scenario(name="dry_circle", nx=n, ny=n, extent=((0.0, 1.0), (0.0, 1.0)), B=None, w0=w, hu0=z,
                      hv0=z.copy(), cfl=0.25)


def check_symmetry(h, hu, hv, tol):
    # test/test_shallow_water_dry_states_2d.jl:103-116
    nx, ny = h.shape
    xl, yl = nx // 3, ny // 3
    xr, yu = nx - xl + 1, ny - yl + 1
    xl, xr, yl, yu = xl - 1, xr - 1, yl - 1, yu - 1
    assert np.max(h[xl, :] - h[xr, :]) <= tol and np.max(h[:, yl] - h[:, yu]) <= tol
    assert np.max(hu[xl, :] + hu[xr, :]) <= tol and np.max(hu[:, yl] - hu[:, yu]) <= tol
    assert np.max(hv[xl, :] - hv[xr, :]) <= tol and np.max(hv[:, yl] + hv[:, yu]) <= tol


def test_dry_state_symmetry():
    sc = dry_circle(64)
    o = oracle_from(sc)
    o.simulate_to_time(0.05)
    assert o.t == 0.05
    check_symmetry(*o.interior(), 1e-12)


def swashes_dam(nx, wet: bool, transpose: bool):
    # test/test_swashes.jl:218-333: 2D-x (nx x 3) vs 2D-y (3 x nx) dam breaks, Swashes 4.1.1 / 4.1.2
    hl, hr = 0.005, (0.001 if wet else 0.0)
    L = 10.0
    xc = (np.arange(nx) + 0.5) * (L / nx)
    h1 = np.where(xc <= 5.0, hl, hr)
    w = np.repeat(h1[:, None], 3, axis=1)
    extent = ((0.0, L), (0.0, 5.0))
    if transpose:
        w, extent = w.T.copy(), ((0.0, 5.0), (0.0, L))
    z = np.zeros_like(w)
    return S.Scenario(name="swashes", nx=w.shape[0], ny=w.shape[1], extent=extent, B=None, w0=w, hu0=z,
                      hv0=z.copy(), cfl=0.1, stepper="fe", eq={"depth_cutoff": 1e-7, "desingularizing_kappa": 1e-7})


@pytest.mark.parametrize("wet", [True, False])
def test_x_and_y_dam_breaks_bitwise_equal(wet):
    ox = oracle_from(swashes_dam(128, wet, False))
    oy = oracle_from(swashes_dam(128, wet, True))
    ox.simulate_to_time(1.0)
    oy.simulate_to_time(1.0)
    assert ox.current_timestep == oy.current_timestep and ox.t == oy.t
    hx, hux, hvx = ox.interior()
    hy, huy, hvy = oy.interior()
    assert np.all(hvx == 0) and np.all(huy == 0)
    assert np.array_equal(hx[:, 1], hy[1, :]) and np.array_equal(hux[:, 1], hvy[1, :])


def test_mass_conserved_without_sources():
    o = oracle_from(S.circular_dam_break(64))
    w0 = o.interior()[0].sum()
    for _ in range(50):
        o.perform_step(math.inf)
    assert abs(o.interior()[0].sum() - w0) <= 1e-10 * w0


def smooth_bump(n=64):
    """A smooth wet bump on a flat bottom (no limiter switching near the crest
    matters at this amplitude): the time-order test's initial state."""
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    h0 = 1.0 + 0.1 * np.exp(-((X - 0.5) ** 2 + (Y - 0.45) ** 2) / 0.01)
    z = np.zeros_like(h0)
    return S.Scenario(name="bump", nx=n, ny=n, extent=((0.0, 1.0), (0.0, 1.0)), B=None, w0=h0, hu0=z, hv0=z.copy(),
                      cfl=0.2)


def time_order(run, T=0.0128, dts_div=(16, 32, 64, 128), ref_div=2048):
    """Observed order of a stepper in time, as test/test_timesteppers.jl:70-83
    measures it: errors at T against a fine RK2 reference, fitted in log-log.
    run(stepper, dt, T) returns w at T."""
    ref = run("rk2", T / ref_div, T)
    out = {}
    for st in ("rk2", "fe"):
        dts = [T / d for d in dts_div]
        errs = [float(np.abs(run(st, dt, T) - ref).max()) for dt in dts]
        out[st] = float(np.polyfit(np.log(dts), np.log(errs), 1)[0])
    return out


def _oracle_run(stepper, dt, T):
    sc = smooth_bump()
    sc.stepper = stepper
    o = oracle_from(sc)
    for _ in range(int(round(T / dt))):
        o.perform_step(dt)  # max_dt below the CFL step: every step is exactly dt
    return o.interior()[0]


def test_time_order_of_the_steppers():
    # test/test_timesteppers.jl:70-87: forward Euler is first order, RK2 second
    # order in time (here for the full shallow-water right-hand side, fixed dt)
    order = time_order(_oracle_run)
    assert order["rk2"] == pytest.approx(2.0, abs=0.05)
    assert order["fe"] == pytest.approx(1.0, abs=0.1)


def _friction_run(nx, ny, B=None, bottom_constant=0.0, elevate=0.0, bottom_source=False, T=0.05):
    """test/test_friction_1d.jl:25-43 in 2D: a Gaussian ridge along x,
    LinearReconstruction(1.05), CentralUpwind, RK2, the default
    ImplicitFriction (Cz = 0.03^2, friction_bh2021), CFL 0.2, to T = 0.05."""
    x = (np.arange(nx) + 0.5) / nx
    w0 = (np.exp(-(x - 0.5) ** 2 / 0.001) + 1.5 + elevate)[:, None] * np.ones((nx, ny))
    z = np.zeros_like(w0)
    o = O.OracleSim(nx=nx, ny=ny, cfl=0.2, stepper=O.STEPPER_RK2, theta=1.05, friction=O.FRICTION_BH2021,
                    friction_Cz=0.03 ** 2, B=B, bottom_constant=bottom_constant,
                    sources=[(O.SRC_BOTTOM, 0.0)] if bottom_source else [])
    o.set_interior(w0, z, z.copy())
    o.simulate_to_time(T)
    return o.interior()


def test_friction_run_is_invariant_under_a_raised_bottom():
    # test/test_friction_1d.jl:83-115: the same run with the bottom and the
    # initial surface raised by 1 (a constant bottom and a bottom field of
    # ones, both with SourceTermBottom) gives the flat-bottom depths and
    # momenta; the reference allows 1e-2 summed over the cells, the oracle
    # holds 1e-10 (what remains is the rounding of w + 1).
    nx, ny = 256, 4
    h_ref, hu_ref, _ = _friction_run(nx, ny)
    const = _friction_run(nx, ny, bottom_constant=1.0, elevate=1.0, bottom_source=True)
    field = _friction_run(nx, ny, B=np.ones((nx + 5, ny + 5)), elevate=1.0, bottom_source=True)
    for h, hu, hv in (const, field):
        assert np.sum(np.abs(h_ref - (h - 1.0))) <= 1e-10
        assert np.sum(np.abs(hu_ref - hu)) <= 1e-10
        assert np.all(hv == 0.0)
    # a bottom field of ones gives B_cell = ((1 + 1) + 1) + 1) / 4 = 1 exactly:
    # the constant and the field run are the same bits
    for a, b in zip(const, field):
        assert np.array_equal(a, b)
