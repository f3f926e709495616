"""vf_water_volume_static: the water volume without any device allocation.

Some callers cannot let a library call cudaMalloc -- their device memory is
owned by another allocator that must account for every byte (CUDA.jl's pool,
a framework's caching allocator), or they run loops that cannot afford the
synchronisation an allocation may imply. This test plays such a caller: the
state, the bottom and the one-double result live in buffers its own allocator
(torch) made, the entry point is called through the C ABI, and the result is
compared with the allocating entry point vf_water_volume on the same state, on
two calls in a row (the static scratch keeps the previous call's contents).
"""
import ctypes as C
import math

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import _native as N
from vfhelpers import hills_rect

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # the Float64 tolerance used throughout the tests


def test_static_volume_matches_allocating_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    sc = hills_rect(120, 90)  # rain and infiltration: the volume changes between the calls
    sim = sc.build(vf.SM103Backend(np.float64))
    lib = N.load()
    B = torch.from_numpy(np.ascontiguousarray(sc.B.T)).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    dx, dy = sim.grid.delta
    got = []
    for _ in range(2):
        for _ in range(10):
            vf.perform_step(sim, math.inf)
        st = vf.current_state(sim)
        dense = np.ascontiguousarray(np.stack([st.h.T, st.hu.T, st.hv.T]))  # (3, N2, N1): x fastest
        state = torch.from_numpy(dense).cuda()
        torch.cuda.synchronize()
        rc = lib.vf_water_volume_static(C.c_void_p(state.data_ptr()), C.c_void_p(B.data_ptr()), sc.nx, sc.ny, 2, 8,
                                        dx, dy, 0, 0.0, C.c_void_p(out.data_ptr()), None)
        assert rc == N.VF_OK, lib.vf_last_error(None)
        torch.cuda.synchronize()
        value = float(out.item())
        assert value == pytest.approx(vf.water_volume(sim), rel=REL_TOL)
        got.append(value)
    assert got[0] != got[1]


def test_static_volume_rejects_grids_beyond_its_scratch():
    lib = N.load()
    rc = lib.vf_water_volume_static(C.c_void_p(16), None, 4, N.VF_STATIC_MAX_ROWS + 1, 2, 8, 1.0, 1.0, 1, 0.0,
                                    C.c_void_p(16), None)
    assert rc == N.VF_EINVAL
    assert b"VF_STATIC_MAX_ROWS" in lib.vf_last_error(None)
