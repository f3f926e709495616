"""The Float64 tile kernels stage their tiles with TMA copies and write the
stage pass's output tile with a tensor store by default; with VF_TMA=0 the
same kernels load and store the plain way. Both must give the same bits, ghost
cells included, on full and partial tiles (interior widths of every residue
mod 4, since a tensor store's clipping is coarser than one element), with and
without friction and bottom arrays, for every boundary kind."""
import math
import os

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import scenarios as S
from vfhelpers import hills_rect

pytestmark = pytest.mark.gpu


def run(sc, steps, tma: bool):
    old = os.environ.get("VF_TMA")
    os.environ["VF_TMA"] = "1" if tma else "0"
    try:
        sim = sc.build(vf.SM103Backend(np.float64))  # the tensor maps are made with the handle
    finally:
        if old is None:
            del os.environ["VF_TMA"]
        else:
            os.environ["VF_TMA"] = old
    dts = []
    for _ in range(steps):
        vf.perform_step(sim, math.inf)
        dts.append(sim.current_timestep)
        sim.t += sim.current_timestep
    st = vf.current_state(sim)  # ghost cells included
    out = (np.array(dts), st.h.copy(), st.hu.copy(), st.hv.copy())
    sim.close()
    return out


CASES = {
    "hills_wall_partial_tiles": (lambda: hills_rect(77, 45), 80),
    "hills_periodic": (lambda: hills_rect(64, 48, bc="periodic"), 60),
    "hills_neumann": (lambda: hills_rect(70, 45, bc="neumann"), 60),
    "dam_break_flat_no_friction": (lambda: S.circular_dam_break(96), 80),
    "hills_wet_dry_256": (lambda: S.hills_wet_dry(256), 40),
    "tiny_2x2": (lambda: hills_rect(2, 2), 20),
    "width_33": (lambda: hills_rect(33, 21), 12),
    "width_34": (lambda: hills_rect(34, 20), 12),
    "width_35": (lambda: hills_rect(35, 19), 12),
    "width_36": (lambda: hills_rect(36, 18), 12),
    "width_35_periodic": (lambda: hills_rect(35, 17, bc="periodic"), 12),
    "width_33_neumann": (lambda: hills_rect(33, 19, bc="neumann"), 12),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_tma_matches_plain_loads(case):
    make, steps = CASES[case]
    a = run(make(), steps, tma=True)
    b = run(make(), steps, tma=False)
    for x, y, name in zip(a, b, ("dt", "w", "hu", "hv")):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64)), f"{case}: {name} differs"


def test_bounded_tile_wait_gives_up_and_returns():
    """The wait the TMA kernels use for their copies ends on its own when the
    copy never completes (a barrier nothing completes), and succeeds at once
    when it does; the kernel returns either way and the context stays usable."""
    import ctypes as C
    from volumefluxes_sm103 import _native as N
    lib = N.load()
    out = C.c_int32(-1)
    N.check(lib, None, lib.vf_selftest_tile_wait(0, 0, 2000, C.byref(out)))
    assert out.value == 1
    N.check(lib, None, lib.vf_selftest_tile_wait(0, 1, 2000, C.byref(out)))
    assert out.value == 0
    sim = S.circular_dam_break(32).build(vf.SM103Backend(np.float64))  # the device still steps afterwards
    vf.perform_step(sim, math.inf)
    assert np.isfinite(vf.current_interior_state(sim).h).all()
    sim.close()
