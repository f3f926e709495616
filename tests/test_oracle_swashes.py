"""The oracle against analytic solutions the reference holds: the SWASHES dam
breaks 4.1.1 (wet, Stoker's solution) and 4.1.2 (dry, Ritter's solution) of
Delestre et al. (2013), which test/swashes.jl:130-180 implements and
test/test_swashes.jl:218-330 runs in 2D on an nx x 3 grid with WallBC,
LinearReconstruction(1.2), CentralUpwind, depth_cutoff = kappa = 1e-7 and
CFL 0.1.

The properties and known answers of tests/test_oracle_kats.py pin single
operators; these runs pin the assembled central-upwind flux, reconstruction
and stepping: at four resolutions the L1 error of h and hu against the exact
solution falls at first order (the order a shock and a rarefaction corner
allow), in both time steppers. The exact solutions are restated here from
the published formulas."""
import math

import numpy as np
import pytest

from oracle import vf_oracle as O

G = 9.81
CASES = {
    # name: (hl, hr, cm, t_end); SWASHES 4.1.1 / 4.1.2, x0 = 5, L = 10
    "4.1.1_wet": (0.005, 0.001, 0.1578324867, 6.0),
    "4.1.2_dry": (0.005, 0.0, 0.0, 4.0),
}
NX = (100, 200, 400, 800)


def dam_break_exact(x, t, hl, hr, cm, x0=5.0):
    """(h, u) of the 1D dam break at time t: still water left of the
    rarefaction head xA, the rarefaction fan up to xB, then (wet bed) the
    constant state cm^2/g up to the shock xC and the still right state."""
    c = math.sqrt(G * hl)
    xA, xB = x0 - t * c, x0 + t * (2 * c - 3 * cm)
    fan_h = (4.0 / (9.0 * G)) * (c - (x - x0) / (2 * t)) ** 2
    fan_u = (2.0 / 3.0) * ((x - x0) / t + c)
    h = np.where(x < xA, hl, np.where(x < xB, fan_h, hr))
    u = np.where(x < xA, 0.0, np.where(x < xB, fan_u, 0.0))
    if hr > 0:
        xC = x0 + t * (2 * cm * cm * (c - cm)) / (cm * cm - G * hr)
        mid = (x >= xB) & (x < xC)
        h = np.where(mid, cm * cm / G, h)
        u = np.where(mid, 2 * (c - cm), u)
    return h, u


def l1_errors(case, nx, stepper):
    hl, hr, cm, t_end = CASES[case]
    dx = 10.0 / nx
    xc = (np.arange(nx) + 0.5) * dx
    w0 = np.where(xc < 5.0, hl, hr)[:, None] * np.ones((nx, 3))
    o = O.OracleSim(nx=nx, ny=3, extent=((0.0, 10.0), (0.0, 5.0)), cfl=0.1, stepper=stepper, depth_cutoff=1e-7,
                    desingularizing_kappa=1e-7, theta=1.2)
    o.set_interior(w0, np.zeros_like(w0), np.zeros_like(w0))
    o.simulate_to_time(t_end)
    w, hu, hv = o.interior()
    h_ex, u_ex = dam_break_exact(xc, t_end, hl, hr, cm)
    # the three rows are identical and carry no transverse momentum
    assert np.array_equal(w[:, 0], w[:, 1]) and np.array_equal(w[:, 1], w[:, 2])
    assert np.all(hv == 0.0)
    return (float(np.sum(np.abs(w[:, 1] - h_ex)) * dx), float(np.sum(np.abs(hu[:, 1] - h_ex * u_ex)) * dx))


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("stepper", [O.STEPPER_FE, O.STEPPER_RK2], ids=["forward_euler", "rk2"])
def test_dam_break_converges_to_the_analytic_solution(case, stepper):
    errs = np.array([l1_errors(case, nx, stepper) for nx in NX])  # (resolution, [h, hu])
    hl = CASES[case][0]
    mass = 5.0 * (hl + CASES[case][1])  # initial water volume per unit width
    for k in range(2):
        order = np.log2(errs[:-1, k] / errs[1:, k])
        assert np.all(order >= 0.8), (case, k, errs[:, k], order)
    # at 800 cells the depth error is below 0.2 % of the water volume
    assert errs[-1, 0] <= 2e-3 * mass, errs[-1, 0]
