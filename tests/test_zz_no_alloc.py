"""vf_water_volume_static: the water volume without any device allocation.

Some callers cannot let a library call cudaMalloc -- their device memory is
owned by another allocator that must account for every byte (CUDA.jl's pool,
a framework's caching allocator), or they run loops that cannot afford the
synchronisation an allocation may imply. This test plays such a caller: the
state, the bottom and the one-double result live in buffers its own allocator
(torch) made, the entry point is called through the C ABI, and the result is
compared with the allocating entry point vf_water_volume on the same state, on
two calls in a row (the static scratch keeps the previous call's contents), in
both precisions, with a corner bottom and with a constant one, on the default
stream and on a stream of the caller's.
"""
import ctypes as C
import math

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import _native as N
from volumefluxes_sm103 import scenarios as S
from vfhelpers import hills_rect

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # the Float64 tolerance used throughout the tests


def _case(bottom: str):
    if bottom == "corners":
        return hills_rect(120, 90)  # rain and infiltration: the volume changes between the calls
    sc = S.circular_dam_break(96)
    from dataclasses import replace
    # a constant bottom of 0.1 that is not exact in Float32, with rain so the volume changes
    return replace(sc, sources=[vf.SourceTermBottom(), vf.ConstantRain(36.0)], eq={}, meta={"bottom_constant": 0.1})


def _build(sc, real):
    be = vf.SM103Backend(real)
    if sc.B is None and "bottom_constant" in sc.meta:
        grid = sc.grid()
        eq = vf.ShallowWaterEquations(vf.ConstantBottomTopography(sc.meta["bottom_constant"]))
        system = vf.ConservedSystem(be, vf.LinearReconstruction(), vf.CentralUpwind(eq), eq, grid,
                                    sc.source_terms(), None)
        sim = vf.Simulator(be, system, vf.RungeKutta2(), grid, cfl=sc.cfl)
        vf.set_current_state(sim, (sc.w0 + 0.1, sc.hu0, sc.hv0))
        return sim
    return sc.build(be)


@pytest.mark.parametrize("real", [np.float64, np.float32])
@pytest.mark.parametrize("bottom", ["corners", "constant"])
@pytest.mark.parametrize("on_stream", [False, True])
def test_static_volume_matches_allocating_entry_point_on_two_calls(real, bottom, on_stream):
    torch = pytest.importorskip("torch")
    sc = _case(bottom)
    sim = _build(sc, real)
    lib = N.load()
    tdt = torch.float64 if real == np.float64 else torch.float32
    rb = 8 if real == np.float64 else 4
    const = sc.B is None
    B = None if const else torch.from_numpy(np.ascontiguousarray(sc.B.T).astype(real)).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    dx, dy = sim.grid.delta
    stream = torch.cuda.Stream() if on_stream else None
    tol = REL_TOL if real == np.float64 else 1e-12  # both sums are Float64 over the same Float32 values
    got = []
    for _ in range(2):
        for _ in range(10):
            vf.perform_step(sim, math.inf)
        st = vf.current_state(sim)
        dense = np.ascontiguousarray(np.stack([st.h.T, st.hu.T, st.hv.T])).astype(real)  # (3, N2, N1): x fastest
        state = torch.from_numpy(dense).cuda()
        torch.cuda.synchronize()
        rc = lib.vf_water_volume_static(C.c_void_p(state.data_ptr()), None if const else C.c_void_p(B.data_ptr()),
                                        sc.nx, sc.ny, 2, rb, dx, dy, int(const),
                                        sc.meta.get("bottom_constant", 0.0), C.c_void_p(out.data_ptr()),
                                        None if stream is None else C.c_void_p(stream.cuda_stream))
        assert rc == N.VF_OK, lib.vf_last_error(None)
        torch.cuda.synchronize()
        value = float(out.item())
        assert value == pytest.approx(vf.water_volume(sim), rel=tol)
        got.append(value)
    assert got[0] != got[1]
    sim.close()


def test_static_volume_rejects_grids_beyond_its_scratch():
    lib = N.load()
    rc = lib.vf_water_volume_static(C.c_void_p(16), None, 4, N.VF_STATIC_MAX_ROWS + 1, 2, 8, 1.0, 1.0, 1, 0.0,
                                    C.c_void_p(16), None)
    assert rc == N.VF_EINVAL
    assert b"VF_STATIC_MAX_ROWS" in lib.vf_last_error(None)
