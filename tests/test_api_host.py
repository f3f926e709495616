"""Host-side logic of the reference-mirroring API (no GPU calls)."""
import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import scenarios as S


def test_grid_defaults_follow_the_reference():
    # src/grid.jl:82-90: gc=1 and PeriodicBC by default
    g = vf.CartesianGrid(8, 4)
    assert g.gc == 1 and isinstance(g.boundary, vf.PeriodicBC)
    assert g.size() == (10, 6) and g.interior_size() == (8, 4)
    g = vf.CartesianGrid(8, 4, gc=2, boundary=vf.WallBC(), extent=[[0.0, 2.0], [1.0, 5.0]])
    assert g.delta == (0.25, 1.0) and vf.compute_dx(g) == 0.25 and vf.compute_dy(g) == 1.0


def test_cell_faces_use_julia_linrange():
    g = vf.CartesianGrid(3, 3, gc=2, extent=[[0.0, 0.3], [0.0, 1.0]])
    xf = vf.cell_faces(g, vf.XDIR)
    t = np.arange(4) / 3
    assert np.array_equal(xf, (1 - t) * 0.0 + t * 0.3)
    full = vf.cell_faces(g, interior=False)
    assert full.shape == (8, 8, 2)
    dx, dy = 0.3 / 3, 1.0 / 3
    assert full[0, 0, 0] == 0.0 - 2 * dx and full[-1, -1, 1] == 1.0 + 2 * dy
    c = vf.cell_centers(g)
    assert c.shape == (3, 3, 2)
    assert np.allclose(c[:, 0, 0], [0.05, 0.15, 0.25])
    assert np.allclose(vf.cell_center(g, (3, 3)), (0.05, 1 / 6), rtol=0, atol=1e-15)


def test_compute_rain_units():
    # test/test_rain.jl:55-59: ConstantRain takes m/h
    r = vf.ConstantRain(0.01)
    assert vf.compute_rain(r, 12.6, (12, 56)) == 0.01 / 3600.0
    assert vf.compute_infiltration(vf.ConstantInfiltration(2e-6)) == 2e-6


def test_friction_laws_match_reference_formulas():
    # src/friction.jl:30-43
    c, h, s = 0.0009, 0.7, 1.3
    assert vf.friction_bsa2012(c, h, s) == -c * s / (np.cbrt(h) * h)
    assert vf.friction_fcg2016(c, h, s) == -c * s / (np.cbrt(h) * h * h)
    assert vf.friction_bh2021(c, h, s) == -c * s / (h * h)
    f = vf.ImplicitFriction()
    assert f.Cz == 0.03 ** 2 and f.friction_function is vf.friction_bh2021


def test_conserved_system_compatibility():
    # src/equations/equation.jl:74-84
    g = vf.CartesianGrid(4, 4, gc=2, boundary=vf.WallBC())
    B = np.ones((9, 9))
    eq = vf.ShallowWaterEquations(vf.BottomTopography2D(B, vf.SM103Backend(), g))
    with pytest.raises(vf.ArgumentError):
        vf.ConservedSystem(vf.SM103Backend(), vf.LinearReconstruction(), vf.CentralUpwind(eq), eq, g)
    vf.ConservedSystem(vf.SM103Backend(), vf.LinearReconstruction(), vf.CentralUpwind(eq), eq, g,
                       vf.SourceTermBottom())
    with pytest.raises(vf.DomainError):
        vf.ShallowWaterEquations(vf.BottomTopography2D(np.ones((8, 9)), vf.SM103Backend(), g))


class _OtherBC(vf.BoundaryCondition):
    pass


@pytest.mark.parametrize("change", ["other_bc", "gc1", "pure_backend"])
def test_unsupported_configurations_raise(change):
    be = vf.SM103Backend()
    g = vf.CartesianGrid(8, 8, gc=1 if change == "gc1" else 2,
                         boundary=_OtherBC() if change == "other_bc" else vf.WallBC())
    eq = vf.ShallowWaterEquations()
    rec = vf.LinearReconstruction()
    sys_ = vf.ConservedSystem(be, rec, vf.CentralUpwind(eq), eq, g)
    with pytest.raises(vf.ArgumentError):
        vf.Simulator(object() if change == "pure_backend" else be, sys_, vf.RungeKutta2(), g)


class _FakeSim:
    def __init__(self):
        self.current_timestep = 0.5


def test_interval_writer_fires_like_the_reference():
    # src/callbacks.jl:49-55
    calls = []
    w = vf.IntervalWriter(step=1.0, writer=lambda t, s: calls.append(t))
    sim = _FakeSim()
    for t in (0.5, 1.0, 1.5, 2.0, 2.5):
        w(t, sim)
    # fires when t + dt >= current_t, then current_t += step
    assert calls == [0.5, 1.0, 1.5, 2.5]
    assert w.current_t == 4.0
    m = vf.MultipleCallbacks([w])
    m(3.0, sim)
    assert calls[-1] == 2.5
    m(3.5, sim)
    assert calls[-1] == 3.5


def test_splitmix64_known_values():
    # splitmix64 first outputs for seed 1234567 (a published test vector)
    rng = S.SplitMix64(1234567)
    assert [rng.next_u64() for _ in range(3)] == [6457827717110365317, 3203168211198807973, 9817491932198370423]


def test_scenarios_shapes():
    sc = S.hills_wet_dry(64, length=64.0)
    assert sc.B.shape == (69, 69) and sc.w0.shape == (64, 64)
    Bc = 0.25 * (sc.B[:-1, :-1] + sc.B[1:, :-1] + sc.B[:-1, 1:] + sc.B[1:, 1:])[2:-2, 2:-2]
    assert np.all(sc.w0 >= Bc) and np.any(sc.w0 == Bc)  # dry islands exist


def test_grid_coordinates_2d():
    # test/test_grid_2d.jl:25-85: a 10 x 6 grid over [0,10] x [0,6] with gc = 2
    nx, ny, gc = 10, 6, 2
    g = vf.CartesianGrid(nx, ny, extent=[[0.0, nx], [0.0, ny]], gc=gc)
    dx, dy = vf.compute_dx(g), vf.compute_dy(g)
    faces, centers = vf.cell_faces(g), vf.cell_centers(g)
    assert np.array_equal(faces[:, :, 0], np.arange(nx + 1.0)[:, None] * np.ones((1, ny + 1)))
    assert np.array_equal(faces[:, :, 1], np.ones((nx + 1, 1)) * np.arange(ny + 1.0)[None, :])
    assert np.array_equal(centers[:, :, 0], (np.arange(nx) + 0.5)[:, None] * np.ones((1, ny)))
    assert np.array_equal(centers[:, :, 1], np.ones((nx, 1)) * (np.arange(ny) + 0.5)[None, :])
    assert np.array_equal(vf.cell_faces(g, vf.XDIR), np.arange(nx + 1.0))
    assert np.array_equal(vf.cell_faces(g, vf.YDIR), np.arange(ny + 1.0))
    assert np.array_equal(vf.cell_centers(g, vf.XDIR), np.arange(nx) + 0.5)
    assert np.array_equal(vf.cell_centers(g, vf.YDIR), np.arange(ny) + 0.5)
    faces_gc = vf.cell_faces(g, interior=False)
    assert np.allclose(faces_gc[2:-2, 2:-2], faces, rtol=0, atol=1e-14)
    cells_gc = vf.cell_centers(g, interior=False)
    assert np.allclose(cells_gc[2:-2, 2:-2], centers, rtol=0, atol=1e-14)
    for j in (1, 2):
        for i in (1, 2):
            assert np.allclose(faces_gc[i - 1, j - 1], (-3 + i, -3 + j), rtol=0, atol=1e-14)
            assert np.allclose(faces_gc[-i, -j], (nx + (gc - i + 1), ny + (gc - j + 1)), rtol=0, atol=1e-14)
            assert np.allclose(cells_gc[i - 1, j - 1], (-3 + i + dx / 2, -3 + j + dy / 2), rtol=0, atol=1e-14)
            assert np.allclose(cells_gc[-i, -j], (nx + (gc - i) + dx / 2, ny + (gc - j) + dy / 2), rtol=0, atol=1e-14)
