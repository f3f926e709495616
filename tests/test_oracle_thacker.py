"""The oracle against the 2D analytic wet/dry solutions the reference holds:
Thacker's oscillations in a paraboloid bowl, SWASHES 4.2.2.a (radially
symmetric) and 4.2.2.b (planar surface), as test/swashes.jl:87-125 defines
them, test/swashes.jl:227-301 writes their exact states and
test/swashes.jl:305-310 their bottom, and test/run_swashes_2d.jl:31-45 runs
them: gc = 2, WallBC, depth_cutoff = desingularizing_kappa = 1e-4,
LinearReconstruction(1.2), CentralUpwind, SourceTermBottom, CFL 0.1, forward
Euler (and RK2 here), started from the exact state at t = 0.

These pin the 2D machinery the 1D dam breaks do not reach: the practical
reconstruction's wet/dry clauses on a curved bottom, the central-upwind flux
at a moving shoreline in both directions, the bottom source and the dry
clamp. At 50², 100² and 200² cells, a quarter of an oscillation period in:
the L1 depth error falls at better than first order (measured 1.18-1.20 for
the planar surface, 1.38-1.53 for the radial case) and the water volume is
conserved to round-off. The exact solutions are restated from the published
formulas (Thacker 1981; Delestre et al. 2013).
"""
import math

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from oracle import vf_oracle as O

G, A, L, H0 = 9.81, 1.0, 4.0, 0.1  # gravity, bowl radius a, domain side, bowl depth h0
NX = (50, 100, 200)


def bottom(r):
    """b(r) = -h0 (1 - r^2/a^2)."""
    return -H0 * (1.0 - r * r / (A * A))


def radius(x, y):
    return np.sqrt((x - L / 2) ** 2 + (y - L / 2) ** 2)


def exact(case, t, x, y, Bc):
    """(w, hu, hv) at time t and the period of one oscillation. Depths below
    the bottom are clipped to dry cells, w = max(w, B_cell), as the
    reference's initial and reference states are."""
    if case == "4.2.2.b_planar":
        eta = 0.5
        om = math.sqrt(2 * G * H0) / A
        u, v = -eta * om * math.sin(om * t), eta * om * math.cos(om * t)
        w = (eta * H0 / A**2) * (2 * (x - L / 2) * math.cos(om * t) + 2 * (y - L / 2) * math.sin(om * t) - eta)
        w = np.maximum(w, Bc)
        h = w - Bc
        return w, u * h, v * h, 2 * math.pi / om
    r0 = 0.8
    om = math.sqrt(8 * G * H0) / A
    a_ = (A * A - r0 * r0) / (A * A + r0 * r0)
    den = 1 - a_ * math.cos(om * t)
    t1 = math.sqrt(1 - a_ * a_) / den - 1.0
    t2 = (1 - a_ * a_) / den**2 - 1.0
    vel = 0.5 * om * a_ * math.sin(om * t) / den
    w = np.maximum(H0 * (t1 - (radius(x, y) ** 2 / A**2) * t2), Bc)
    h = w - Bc
    return w, vel * (x - L / 2) * h, vel * (y - L / 2) * h, 2 * math.pi / om


def run(case, nx, stepper):
    """L1 depth error and relative volume change a quarter period in."""
    grid = vf.CartesianGrid(nx, nx, gc=2, boundary=vf.WallBC(), extent=[[0.0, L], [0.0, L]])
    f = vf.cell_faces(grid, interior=False)  # corners of the total grid, ghosts included
    B = bottom(radius(f[:, :, 0], f[:, :, 1]))
    c = vf.cell_centers(grid)
    x, y = c[:, :, 0], c[:, :, 1]
    d = L / nx
    Bc = 0.25 * (bottom(radius(x - d / 2, y - d / 2)) + bottom(radius(x - d / 2, y + d / 2))
                 + bottom(radius(x + d / 2, y - d / 2)) + bottom(radius(x + d / 2, y + d / 2)))
    w0, hu0, hv0, period = exact(case, 0.0, x, y, Bc)
    o = O.OracleSim(nx=nx, ny=nx, extent=((0.0, L), (0.0, L)), cfl=0.1, stepper=stepper, depth_cutoff=1e-4,
                    desingularizing_kappa=1e-4, theta=1.2, B=B, sources=[(O.SRC_BOTTOM, 0.0)])
    o.set_interior(w0, hu0, hv0)
    t_end = 0.25 * period
    o.simulate_to_time(t_end)
    w, hu, hv = o.interior()
    we, _, _, _ = exact(case, t_end, x, y, Bc)
    area = d * d
    err = float(np.sum(np.abs(w - we)) * area)
    m0, m1 = float(np.sum(w0 - Bc) * area), float(np.sum(w - Bc) * area)
    assert np.all(w - Bc >= -1e-15), "negative depth"
    return err, (m1 - m0) / m0, m0


@pytest.mark.parametrize("case", ["4.2.2.a_radial", "4.2.2.b_planar"])
@pytest.mark.parametrize("stepper", [O.STEPPER_FE, O.STEPPER_RK2], ids=["forward_euler", "rk2"])
def test_thacker_paraboloid_converges_to_the_analytic_solution(case, stepper):
    res = [run(case, nx, stepper) for nx in NX]
    errs = np.array([r[0] for r in res])
    order = np.log2(errs[:-1] / errs[1:])
    assert np.all(order >= 1.0), (case, errs, order)
    for err, dm, m0 in res:
        assert abs(dm) < 1e-12, (case, dm)  # volume conserved to round-off (no sources, no clamp gain here)
    # at 200^2 cells the depth error is below 1% of the water volume
    assert errs[-1] <= 1e-2 * res[-1][2], (case, errs[-1], res[-1][2])
