"""The CUDA library reproduces the committed golden fixtures bit for bit in
Float64, step by step through perform_step."""
import math
import sys
from pathlib import Path

import numpy as np
import pytest

import volumefluxes_sm103 as vf

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import make_golden as G  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_library_matches_golden(name):
    ref = np.load(Path(G.HERE) / f"{name}.npz")
    sim = G.scenario(name).build(vf.SM103Backend(np.float64))
    dts = []
    for _ in range(G.CASES[name]):
        vf.perform_step(sim, math.inf)
        dts.append(vf.current_timestep(sim))
        sim.t += vf.current_timestep(sim)
    assert np.array_equal(np.asarray(dts), ref["dts"])
    st = vf.current_interior_state(sim)
    for a, b in zip((st.h, st.hu, st.hv), (ref["w"], ref["hu"], ref["hv"])):
        assert np.array_equal(a, b)
