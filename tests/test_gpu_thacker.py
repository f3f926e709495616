"""Thacker's paraboloid oscillations (SWASHES 4.2.2.a/b, test/swashes.jl:87-125,
227-310, run as test/run_swashes_2d.jl:31-45 runs them) on the device: a
quarter period on 64^2 cells under forward Euler and RK2, both kernel
designs, bit for bit the oracle's run (every dt too). With
tests/test_oracle_thacker.py, which shows the oracle converging to the exact
solutions, this ties the device to an analytic 2D wet/dry solution the
reference holds."""
import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import scenarios as S
from test_oracle_thacker import L, bottom, exact, radius
from vfhelpers import oracle_from

pytestmark = pytest.mark.gpu


def thacker(case, nx, stepper):
    grid = vf.CartesianGrid(nx, nx, gc=2, boundary=vf.WallBC(), extent=[[0.0, L], [0.0, L]])
    f = vf.cell_faces(grid, interior=False)
    B = bottom(radius(f[:, :, 0], f[:, :, 1]))
    c = vf.cell_centers(grid)
    x, y = c[:, :, 0], c[:, :, 1]
    d = L / nx
    Bc = 0.25 * (bottom(radius(x - d / 2, y - d / 2)) + bottom(radius(x - d / 2, y + d / 2))
                 + bottom(radius(x + d / 2, y - d / 2)) + bottom(radius(x + d / 2, y + d / 2)))
    w0, hu0, hv0, period = exact(case, 0.0, x, y, Bc)
    sc = S.Scenario(name=f"thacker_{case}", nx=nx, ny=nx, extent=((0.0, L), (0.0, L)), B=B, w0=w0, hu0=hu0, hv0=hv0,
                    cfl=0.1, stepper=stepper, bottom_source=True,
                    eq={"depth_cutoff": 1e-4, "desingularizing_kappa": 1e-4})
    return sc, 0.25 * period


@pytest.mark.parametrize("case", ["4.2.2.a_radial", "4.2.2.b_planar"])
@pytest.mark.parametrize("stepper", ["fe", "rk2"])
@pytest.mark.parametrize("variant", ["march", "tile"])
def test_thacker_on_the_device_equals_the_oracle(case, stepper, variant, monkeypatch):
    monkeypatch.setenv("VF_KERNELS", variant)
    sc, t_end = thacker(case, 64, stepper)
    sim = sc.build(vf.SM103Backend(np.float64))
    ora = oracle_from(sc)
    vf.simulate_to_time(sim, t_end)
    steps = ora.simulate_to_time(t_end)
    assert steps > 20 and sim.t == ora.t
    got = vf.current_interior_state(sim)
    for name, a, b in zip(("h", "hu", "hv"), (got.h, got.hu, got.hv), ora.interior()):
        assert np.array_equal(a, b), f"{name}: {int((a != b).sum())} cells differ"
    sim.close()
