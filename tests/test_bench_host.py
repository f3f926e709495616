"""Host-side logic of bench.py: the roofline arithmetic, the per-cell figures
read from the committed ncu summaries, the kernel names it reports, and the
CPU-baseline timer on a small grid. No GPU is touched."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402
from volumefluxes_sm103 import scenarios  # noqa: E402


def test_profile_tables_cover_the_reported_kernels():
    traffic = bench.profile_table("traffic")
    inst = bench.profile_table("fp64_inst_per_cell")
    for key in (("stage", "f64"), ("flux", "f64"), ("stage", "f32"), ("flux", "f32")):
        assert key in traffic and traffic[key] > 0, key
    # measured DRAM bytes per cell are at least the design's words (Float64 8 B, Float32 4 B)
    assert traffic[("stage", "f64")] >= bench.WORDS_STAGE_PASS * 8 * 0.9
    assert traffic[("flux", "f64")] >= bench.WORDS_FLUX_PASS * 8 * 0.9
    assert ("stage", "f64") in inst and 300 < inst[("stage", "f64")] < 1000


def test_roofline_arithmetic():
    sc = scenarios.Scenario(name="t", nx=1000, ny=2000, extent=((0.0, 1.0), (0.0, 1.0)), B=None,
                            w0=None, hu0=None, hv0=None, cfl=0.25)
    traffic = {("stage", "f64"): 90.0}
    r = bench.roofline(sc, "f64", ms_flux=1.0, ms_stage=2.0, peak=5000.0, peak_kind="measured", traffic=traffic)
    cells = 1000 * 2000
    alg = bench.WORDS_STAGE_PASS * 8 * cells
    assert r["algorithmic_bytes"] == alg
    assert r["achieved"] == pytest.approx(alg / 2e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 5000.0)
    assert r["traffic"] == pytest.approx(90.0 * cells)
    assert r["bound"] == "hbm" and r["launch_ms"] == 2.0
    # the dominant kernel is the slower one
    r2 = bench.roofline(sc, "f32", ms_flux=3.0, ms_stage=2.0, peak=5000.0, peak_kind="measured", traffic={})
    assert r2["algorithmic_bytes"] == bench.WORDS_FLUX_PASS * 4 * cells and r2["traffic"] is None


def test_fp64_pipe_roofline():
    sc = scenarios.Scenario(name="t", nx=100, ny=100, extent=((0.0, 1.0), (0.0, 1.0)), B=None,
                            w0=None, hu0=None, hv0=None, cfl=0.25)
    r = bench.fp64_roofline(sc, 2.0, 2000.0, {("stage", "f64"): 500.0})
    assert r["achieved"] == pytest.approx(500.0 * 1e4 / 2e-3)
    assert r["peak"] == pytest.approx(bench.FP64_INST_PER_CLK_SM * bench.N_SMS * 2000.0e6)
    assert "developed" in r["window"]
    assert bench.fp64_roofline(sc, 2.0, 2000.0, {}) is None
    assert bench.fp64_roofline(sc, None, 2000.0, {("stage", "f64"): 500.0}) is None


def test_field_errors():
    ref = (np.array([[2.0, 4.0]]), np.array([[0.001, -0.002]]), np.zeros((1, 2)))
    got = (np.array([[2.0, 4.0 + 4e-12]]), np.array([[0.001, -0.002 + 2e-12]]), np.zeros((1, 2)))
    e = bench.field_errors(got, ref)
    assert e["w"]["rel_field"] == pytest.approx(1e-12) and e["w"]["rel_state"] == pytest.approx(1e-12)
    assert e["hu"]["rel_field"] == pytest.approx(1e-9) and e["hu"]["rel_state"] == pytest.approx(5e-13)
    assert e["hv"]["max_abs"] == 0.0


def test_kernel_names_follow_the_switches(monkeypatch):
    monkeypatch.delenv("VF_KERNELS", raising=False)
    monkeypatch.delenv("VF_TMA", raising=False)
    assert bench.kernel_names("f64") == {"flux": "k_flux_tma<double>", "stage": "k_stage2_tma<double>"}
    assert bench.kernel_names("f32")["stage"] == "k_stage_march<float,24>"
    monkeypatch.setenv("VF_TMA", "0")
    assert bench.kernel_names("f64")["stage"] == "k_stage2<double>"
    monkeypatch.setenv("VF_KERNELS", "march")
    assert bench.kernel_names("f64")["flux"] == "k_flux_march<double,40>"


def test_cpu_baseline_timer_small_grid():
    sc = scenarios.hills_wet_dry(48)
    o = bench.oracle_sim(sc)
    rate, threads, steps, el = bench.cpu_rate(sc, 0, None, budget_s=0.2, max_steps=3, threads=1, o=o)
    assert threads == 1 and 1 <= steps <= 3 and el > 0 and rate == pytest.approx(48 * 48 * steps / el)


def test_reference_arm_prints_its_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--n", "64", "--steps", "2",
                          "--warmup", "1", "--cpu-budget", "1"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "cell-updates/s" and line["value"] > 0
    assert line["cpu_baseline"]["cores"] >= 1 and line["e2e"]["h2d_bytes_per_step"] == 0
    # the same config object as the library's arm prints for this workload
    assert line["config"] == bench.bench_config(scenarios.hills_wet_dry(64), "f64", 1)
