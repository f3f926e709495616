"""The integer-pipe Float64 division (volumefluxes.jl_gb300/csrc/vf_idiv.cuh) compiled for
the host and compared bit for bit with IEEE division, including with a deliberately
perturbed reciprocal seed (the device seed is a different approximation)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("scale", [None, "1.0001f", "0.9999f"])
def test_integer_division_is_ieee_exact(tmp_path, scale):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "idiv_check"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{ROOT / 'volumefluxes.jl_gb300' / 'csrc'}",
           str(ROOT / "tests" / "native" / "idiv_check.cpp"), "-o", str(exe)]
    if scale:
        cmd.insert(1, f"-DVF_IDIV_SEED_SCALE={scale}")
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe), "3000000", "17"], capture_output=True, text=True)
    bad, fast = (int(v) for v in out.stdout.split()[-2:])
    assert bad == 0, out.stdout
    assert fast > 2_900_000
