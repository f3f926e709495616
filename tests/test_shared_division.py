"""The shared-divisor Float64 division (volumefluxes.jl_gb300/csrc/vf_sdiv.cuh)
compiled for the host and compared bit for bit with IEEE division, with the
host's seed and with deliberately poor seeds (the device seed differs); the
exact rounding test must make every accepted quotient the IEEE one."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("scale", [None, "1.001", "0.97"])
def test_shared_division_is_ieee_exact(tmp_path, scale):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "sdiv_check"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{ROOT / 'volumefluxes.jl_gb300' / 'csrc'}",
           str(ROOT / "tests" / "native" / "sdiv_check.cpp"), "-o", str(exe)]
    if scale:
        cmd.insert(1, f"-DVF_SDIV_SEED_SCALE={scale}")
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe), "1500000", "23"], capture_output=True, text=True)
    bad, fast = (int(v) for v in out.stdout.split()[-2:])
    assert bad == 0, out.stdout
    if scale != "0.97":  # a 3% seed leaves y too far from 1/b: nearly everything falls back, still exact
        assert fast > 0.6 * 4 * 1_500_000, fast  # the rest are outside the fast range (extreme exponents, zeros)
