"""The seeded synthetic workloads the bench and the GPU tests run: their draws
stay inside the stated distributions (the configurations' shapes, sizes and
value ranges) and are reproducible. No GPU is touched."""
import numpy as np
import pytest

from volumefluxes_sm103 import scenarios as S


def test_small_configuration_is_the_circular_dam_break():
    sc = S.circular_dam_break(256)
    assert (sc.nx, sc.ny, sc.cfl, sc.stepper, sc.bc) == (256, 256, 0.2, "rk2", "wall")
    assert sc.extent == ((0.0, 1.0), (0.0, 1.0)) and sc.B is None
    x = (np.arange(256) + 0.5) / 256
    r = np.hypot(x[:, None] - 0.5, x[None, :] - 0.5)
    assert np.array_equal(sc.w0, np.where(r < 0.15, 2.0, 1.0))
    assert not sc.hu0.any() and not sc.hv0.any()
    assert sc.rain_m_per_h is None and sc.manning_n is None


def test_wet_dry_hills_follow_the_configuration():
    sc = S.hills_wet_dry(256)
    assert sc.meta == {"seed": 20240901, "n_hills": 64}
    assert sc.B.shape == (256 + 5, 256 + 5)
    Bc = 0.25 * (sc.B[:-1, :-1] + sc.B[1:, :-1] + sc.B[:-1, 1:] + sc.B[1:, 1:])[2:-2, 2:-2]
    assert np.array_equal(sc.w0, np.maximum(1.5, Bc))
    assert (Bc > 1.5).any() and (Bc < 1.5).any()  # dry islands and wet ground
    assert sc.rain_m_per_h == pytest.approx(0.036) and sc.infiltration_m_per_s == 2e-6
    assert sc.manning_n == 0.03 and sc.cfl == 0.25 and sc.bottom_source
    # the bottom is the planar slope plus non-negative hills of at most 64 * 4 m
    f = S.hill_bottom(256, 256, sc.extent, 0, 1)
    assert ((sc.B - f) >= 0).all() and (sc.B - f).max() <= 64 * 4.0
    assert np.array_equal(S.hills_wet_dry(256).B, sc.B)  # reproducible


def test_ensemble_draws():
    specs = S.ensemble_specs()
    assert len(specs) == 256
    sides = np.array([s.side for s in specs])
    assert sides.min() >= 64 and sides.max() <= 1024
    logs = np.log(sides)
    assert abs(np.median(logs) - np.log(256.0)) < 0.35  # log-uniform over [64, 1024]: median 256
    assert all(8 <= s.n_hills <= 32 for s in specs)
    assert all(0.0 <= s.rain_m_per_s <= 5e-5 and 0.01 <= s.manning_n <= 0.08 and 0.0 <= s.h0 <= 2.0 for s in specs)
    assert all(10.0 <= s.endtime <= 600.0 and float(np.float32(s.endtime)) == s.endtime for s in specs)
    assert [s.seed for s in S.ensemble_specs()] == [s.seed for s in specs]
    m = S.ensemble_member(specs[0])
    assert m.nx == specs[0].side and m.eq["depth_cutoff"] == S.ENSEMBLE_DEPTH_CUTOFF
    Bc = 0.25 * (m.B[:-1, :-1] + m.B[1:, :-1] + m.B[:-1, 1:] + m.B[1:, 1:])[2:-2, 2:-2]
    assert np.allclose(m.w0 - Bc, specs[0].h0)


def test_serving_draws():
    specs = S.serving_specs()
    assert len(specs) == 48
    assert all(128 <= s.spec.side <= 2048 for s in specs)
    reals = {s.real for s in specs}
    assert reals == {"f32", "f64"}
    assert all(2.0 <= s.spec.endtime <= 20.0 for s in specs)


def test_differentiation_case():
    case = S.differentiation_case(128)
    sc = case.scenario
    assert case.gauges.shape == (32, 2) and case.gauges.min() >= 0 and case.gauges.max() < 128
    assert sc.manning_n == 0.03 and sc.rain_m_per_h == pytest.approx(2e-5 * 3600)
    d = case.B_target - sc.B
    assert np.abs(d).max() <= 8 * 0.1 and np.abs(d).max() > 0
