"""The reference-facing API on the GPU: device time loop, callbacks, volume, state I/O, errors."""
import math

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import scenarios as S
from vfhelpers import hills_rect, oracle_from

pytestmark = pytest.mark.gpu


def test_device_loop_equals_host_loop():
    sc = hills_rect(80, 60)
    a = sc.build(vf.SM103Backend())
    b = sc.build(vf.SM103Backend())
    T = 2.0
    vf.simulate_to_time(a, T)                               # device-resident loop
    seen = []
    vf.simulate_to_time(b, T, callback=lambda t, s: seen.append(t))  # per-step host loop
    assert a.t == b.t == T
    assert a.current_timestep == b.current_timestep
    ga, gb = vf.current_interior_state(a), vf.current_interior_state(b)
    assert np.array_equal(ga.h, gb.h) and np.array_equal(ga.hu, gb.hu) and np.array_equal(ga.hv, gb.hv)
    ora = oracle_from(sc)
    n = ora.simulate_to_time(T)
    assert n == len(seen) and ora.t == T
    assert np.array_equal(ga.h, ora.interior()[0])


def test_interval_writer_fires_at_the_same_times_on_both_loops():
    sc = hills_rect(48, 48)
    a = sc.build(vf.SM103Backend())
    b = sc.build(vf.SM103Backend())
    ta, tb = [], []
    wa = vf.IntervalWriter(step=0.25, writer=lambda t, s: ta.append((t, float(vf.current_interior_state(s).h.sum()))))
    wb = vf.IntervalWriter(step=0.25, writer=lambda t, s: tb.append((t, float(vf.current_interior_state(s).h.sum()))))
    vf.simulate_to_time(a, 1.5, callback=wa)                        # device loop, stops when the writer is due
    vf.simulate_to_time(b, 1.5, callback=vf.MultipleCallbacks([wb, lambda t, s: None]))  # per-step loop
    assert ta == tb and len(ta) >= 6


def test_maximum_timestep_and_match_endtime():
    sc = hills_rect(40, 40)
    sim = sc.build(vf.SM103Backend())
    vf.simulate_to_time(sim, 0.3, maximum_timestep=0.001)
    assert sim.t == pytest.approx(0.3, abs=1e-12)
    assert sim.current_timestep <= 0.001
    ora = oracle_from(sc)
    ora.simulate_to_time(0.3, maximum_timestep=0.001)
    assert ora.t == sim.t
    assert np.array_equal(vf.current_interior_state(sim).h, ora.interior()[0])
    sim2 = sc.build(vf.SM103Backend())
    vf.simulate_to_time(sim2, 0.3, match_endtime=False)
    assert sim2.t >= 0.3


def test_water_volume_matches_host_sum():
    sc = hills_rect(70, 50)
    sim = sc.build(vf.SM103Backend())
    for _ in range(20):
        vf.perform_step(sim, math.inf)
    g = vf.current_interior_state(sim)
    Bc = 0.25 * (sc.B[:-1, :-1] + sc.B[1:, :-1] + sc.B[:-1, 1:] + sc.B[1:, 1:])[2:-2, 2:-2]
    dx, dy = sim.grid.delta
    want = float(((g.h - Bc) * dx * dy).sum())
    assert vf.water_volume(sim) == pytest.approx(want, rel=1e-12)


def test_state_roundtrip_and_reupload():
    sc = hills_rect(33, 21)
    sim = sc.build(vf.SM103Backend())
    for _ in range(5):
        vf.perform_step(sim, math.inf)
    full = vf.current_state(sim)
    inner = vf.current_interior_state(sim)
    assert np.array_equal(full.h[2:-2, 2:-2], inner.h)
    other = sc.build(vf.SM103Backend())
    vf.set_current_state(other, inner)
    for s in (sim, other):
        vf.perform_step(s, math.inf)
    assert np.array_equal(vf.current_interior_state(sim).h, vf.current_interior_state(other).h)


def test_stepping_before_a_state_is_an_error():
    grid = vf.CartesianGrid(8, 8, gc=2, boundary=vf.WallBC())
    eq = vf.ShallowWaterEquations()
    be = vf.SM103Backend()
    sim = vf.Simulator(be, vf.ConservedSystem(be, vf.LinearReconstruction(), vf.CentralUpwind(eq), eq, grid),
                       vf.RungeKutta2(), grid)
    with pytest.raises(vf._native.NativeError):
        vf.perform_step(sim, 1.0)


def test_kernels_are_the_compute_path():
    sim = S.circular_dam_break(32).build(vf.SM103Backend())
    n0 = sim.launch_count()
    vf.simulate_to_time(sim, 0.01)
    assert sim.launch_count() > n0
    assert vf.library_path().name == "libvfsm103.so"


def test_sample_cells_reads_gauges_without_a_download():
    from vfhelpers import hills_rect
    sim = hills_rect(70, 45).build(vf.SM103Backend())
    vf.simulate_to_time(sim, 2.0)
    cells = np.array([[0, 0], [69, 44], [10, 30], [35, 7]])
    s = vf.sample_cells(sim, cells)
    full = vf.current_interior_state(sim)
    for k, (i, j) in enumerate(cells):
        assert s.h[k] == full.h[i, j] and s.hu[k] == full.hu[i, j] and s.hv[k] == full.hv[i, j]
    with pytest.raises(vf.ArgumentError):
        vf.sample_cells(sim, [[70, 0]])


def test_gauge_recorder_in_an_interval_writer():
    from vfhelpers import hills_rect
    sim = hills_rect(48, 40).build(vf.SM103Backend())
    rec = vf.GaugeRecorder([[5, 5], [40, 30]])
    vf.simulate_to_time(sim, 3.0, callback=vf.IntervalWriter(step=1.0, writer=rec))
    assert len(rec.times) >= 3 and all(v.shape == (2,) for v in rec.values)
    assert rec.times == sorted(rec.times)
