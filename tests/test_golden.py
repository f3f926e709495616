"""The oracle reproduces the committed golden fixtures bit for bit
(tests/golden/make_golden.py made them from the oracle; the oracle itself is
pinned by the reference's known-answer tests)."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import make_golden as G  # noqa: E402


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_oracle_matches_golden(name):
    ref = np.load(Path(G.HERE) / f"{name}.npz")
    dts, w, hu, hv = G.run_oracle(name)
    assert np.array_equal(dts, ref["dts"])
    for a, b in zip((w, hu, hv), (ref["w"], ref["hu"], ref["hv"])):
        assert np.array_equal(a, b)
