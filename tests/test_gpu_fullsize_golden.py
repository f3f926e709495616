"""Float64 parity at the measured configuration's full size and length: the
4096 x 4096 wet/dry hills workload over its 1000 RK2 steps, against the oracle's
record in tests/golden/hills_wet_dry_4096_rk2_1000.npz (made by
tests/golden/make_fullsize.py; the fields themselves are too large to store).

At every step the dt must equal the oracle's; at steps 1, 2, 10, 100, 300 and
1000 each interior field must hash to the oracle's SHA-256 (bitwise equality).
Should a hash differ, the stated tolerance still decides: every stored row and
column within 1e-12 relative max-norm of the oracle's, and the field sums and
max-norms likewise. The run takes about 35 s on a GB300.
"""
import hashlib
import math
from pathlib import Path

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import scenarios as S

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "hills_wet_dry_4096_rk2_1000.npz"
F64_TOL = 1e-12  # relative max-norm, per field
FIELDS = ("w", "hu", "hv")


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


@pytest.fixture(scope="module")
def golden():
    if not GOLDEN.exists():
        pytest.fail(f"missing golden record {GOLDEN.name}: run tests/golden/make_fullsize.py")
    return np.load(GOLDEN)


def test_terrain_regenerates_bit_for_bit(golden):
    sc = S.hills_wet_dry(4096)
    assert sha(sc.B) == str(golden["B_sha"])
    assert sha(sc.w0) == str(golden["w0_sha"])


def test_1000_steps_at_4096_match_the_oracle(golden):
    sc = S.hills_wet_dry(4096)
    sim = sc.build(vf.SM103Backend(np.float64))
    dts = golden["dts"]
    cps = [int(c) for c in golden["checkpoints"]]
    hashes_equal = True
    for k in range(1, len(dts) + 1):
        vf.perform_step(sim, math.inf)
        assert vf.current_timestep(sim) == dts[k - 1], f"dt differs at step {k}"
        sim.t += vf.current_timestep(sim)
        if k not in cps:
            continue
        c = cps.index(k)
        g = vf.current_interior_state(sim)
        for name, a in zip(FIELDS, (g.h, g.hu, g.hv)):
            if sha(a) != str(golden[f"{name}_sha"][c]):
                hashes_equal = False
            scale = float(golden[f"{name}_max"][c])
            assert abs(float(np.abs(a).max()) - scale) <= F64_TOL * scale, (name, k)
            assert abs(float(np.sum(a, dtype=np.float64)) - float(golden[f"{name}_sum"][c])) <= \
                F64_TOL * scale * a.size, (name, k)
            if k == cps[-1]:
                rows = np.stack([a[:, j] for j in golden["rows"]])
                cols = np.stack([a[i, :] for i in golden["cols"]])
                assert np.abs(rows - golden[f"{name}_rows"]).max() <= F64_TOL * scale, name
                assert np.abs(cols - golden[f"{name}_cols"]).max() <= F64_TOL * scale, name
    # the kernels reproduce the reference path bit for bit, not just within the tolerance
    assert hashes_equal
    sim.close()
