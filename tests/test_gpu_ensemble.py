"""The batched ensemble (vf_batch_*): many simulations to their own end times in
one set of cluster launches.

Float64: every member ends bitwise where the plain device loop (vf_simulate)
ends on the same scenario, and where the oracle ends. Both precisions: a
member's result is the same alone and in a mix with other members, whatever
cluster size runs it.
"""
import math

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import ensemble as E
from volumefluxes_sm103 import _native as N
from volumefluxes_sm103 import scenarios as S
from vfhelpers import oracle_from, hills_rect
from test_gpu_parity import assert_bitwise, nonsquare_step
from test_gpu_next_rows import terrain_sources
from test_oracle_next_rows import dry_circle_periodic

pytestmark = pytest.mark.gpu


def small_member(i, side=None, endtime=None):
    spec = S.ensemble_specs(16, seed=77)[i]
    if side is not None:
        spec.side = side
    if endtime is not None:
        spec.endtime = endtime
    return S.ensemble_member(spec), spec.endtime


MIXED = {
    # name: (scenario factory, end time [s])
    "hills_97x45_rk2": (lambda: hills_rect(97, 45), 3.0),
    "hills_64x48_fe": (lambda: hills_rect(64, 48, stepper="fe"), 2.0),
    "hills_periodic_70x45": (lambda: hills_rect(70, 45, bc="periodic"), 2.5),
    "norec_50x41": (lambda: hills_rect(50, 41, reconstruction="none"), 2.0),
    "time_rain_horton_64x48": (lambda: terrain_sources(64, 48), 3.0),
    "dam_break_256": (lambda: S.circular_dam_break(256), 0.02),
    "step_13x7": (lambda: nonsquare_step(13, 7), 0.05),
    "dry_circle_periodic_64": (lambda: dry_circle_periodic(64), 0.02),
    "hills_neumann_70x45": (lambda: hills_rect(70, 45, bc="neumann"), 2.5),
}


def interior(sim):
    g = vf.current_interior_state(sim)
    return g.h.copy(), g.hu.copy(), g.hv.copy()


def test_float64_members_match_the_plain_loop_and_the_oracle():
    names = sorted(MIXED)
    scen = [MIXED[k][0]() for k in names]
    ends = [MIXED[k][1] for k in names]
    batch = [sc.build(vf.SM103Backend()) for sc in scen]
    res = E.simulate_batch(batch, ends)
    for name, sc, T, sim, r in zip(names, scen, ends, batch, res):
        assert r.status == N.VF_BATCH_OK, name
        plain = sc.build(vf.SM103Backend())
        vf.simulate_to_time(plain, T)
        assert sim.t == plain.t == T, name
        assert sim.current_timestep == plain.current_timestep, name
        got = vf.current_interior_state(sim)
        assert_bitwise(got, interior(plain))
        if sc.nx * sc.ny <= 64 * 64:
            ora = oracle_from(sc)
            ora.simulate_to_time(T)
            assert ora.o.t == T
            assert_bitwise(got, ora.interior())


@pytest.mark.parametrize("tiles_per_cta", [1, 4, 64])
def test_cluster_sizes_give_the_same_float64_result(tiles_per_cta):
    """Clusters of 16, 4 and 1 CTAs split the 256x160 grid's 80 tiles differently;
    the dt reduction through distributed shared memory is exact, so all agree
    with the plain loop bit for bit."""
    sc = hills_rect(256, 160)
    sim = sc.build(vf.SM103Backend())
    opt = E.BatchOptions(tiles_per_cta=tiles_per_cta)
    c = E.cluster_size(sim, opt)
    assert c == {1: 16, 4: 16, 64: 2}[tiles_per_cta]
    (r,) = E.simulate_batch([sim], 4.0, options=opt)
    assert r.status == N.VF_BATCH_OK and r.steps > 10
    plain = sc.build(vf.SM103Backend())
    vf.simulate_to_time(plain, 4.0)
    assert_bitwise(vf.current_interior_state(sim), interior(plain))


@pytest.mark.parametrize("real", [np.float64, np.float32])
def test_member_is_the_same_alone_and_in_the_mix(real):
    members = [small_member(i) for i in range(6)]
    members = [(sc, min(T, 8.0 if real == np.float64 else 30.0)) for sc, T in members]
    probe, Tp = members[2]
    alone = probe.build(vf.SM103Backend(real))
    (ra,) = E.simulate_batch([alone], Tp)
    mix = [sc.build(vf.SM103Backend(real)) for sc, _ in members]
    rm = E.simulate_batch(mix, [T for _, T in members], options=E.BatchOptions(tiles_per_cta=2))
    assert ra.status == rm[2].status == N.VF_BATCH_OK
    assert (ra.t, ra.steps, ra.last_dt) == (rm[2].t, rm[2].steps, rm[2].last_dt)
    a, m = interior(alone), interior(mix[2])
    for x, y in zip(a, m):
        assert np.array_equal(x, y)


def test_float32_members_state_their_error_against_the_float64_oracle():
    sc = hills_rect(64, 48)
    T = 2.0
    s32 = sc.build(vf.SM103Backend(np.float32))
    (r,) = E.simulate_batch([s32], T)
    assert r.status == N.VF_BATCH_OK
    o64, o32 = oracle_from(sc, 8), oracle_from(sc, 4)
    o64.simulate_to_time(T)
    o32.simulate_to_time(T)
    w64 = o64.interior()[0]
    err_ref = np.abs(o32.interior()[0] - w64).max()
    err = np.abs(vf.current_interior_state(s32).h - w64).max()
    assert err <= 2 * err_ref + 1e-5, (err, err_ref)


def test_max_steps_and_watchdog_statuses():
    sc = hills_rect(64, 48)
    sim = sc.build(vf.SM103Backend())
    (r,) = E.simulate_batch([sim], 100.0, max_steps=7)
    assert r.status == N.VF_BATCH_MAX_STEPS and r.steps == 7 and r.t < 100.0
    plain = sc.build(vf.SM103Backend())
    for _ in range(7):
        vf.perform_step(plain, 100.0 - plain.t)
        plain.t += plain.current_timestep
    assert r.t == plain.t
    assert_bitwise(vf.current_interior_state(sim), interior(plain))
    # A watchdog far below one step's time stops the member before its first
    # update: state and time unchanged.
    sim2 = sc.build(vf.SM103Backend())
    before = interior(sim2)
    (r2,) = E.simulate_batch([sim2], 100.0, options=E.BatchOptions(time_limit_s=1e-9))
    assert r2.status == N.VF_BATCH_TIMEOUT and r2.steps == 0 and r2.t == 0.0
    for x, y in zip(before, interior(sim2)):
        assert np.array_equal(x, y)


def test_nonblocking_poll_and_collect():
    members = [small_member(i, endtime=5.0)[0] for i in range(4)]
    sims = [sc.build(vf.SM103Backend(np.float32)) for sc in members]
    run = E.BatchRun(sims, 5.0)
    run.wait()
    assert run.n_done() == 4
    assert all(run.is_done(i) for i in range(4))
    r1 = run.collect(1)
    assert r1.t == 5.0 and sims[1].t == 5.0
    out = run.finish()
    assert all(o.status == N.VF_BATCH_OK for o in out)
    # handles are usable again after collection
    vf.perform_step(sims[0], math.inf)


def test_batch_rejects_duplicates_and_unready_handles():
    sc = hills_rect(32, 32)
    sim = sc.build(vf.SM103Backend())
    with pytest.raises(vf.ArgumentError):
        E.simulate_batch([sim, sim], 1.0)


@pytest.mark.parametrize("real", [np.float64, np.float32])
def test_wide_members_match_narrow_members_and_the_plain_loop(real):
    """Members above wide_cells run the whole-grid kernels fed in graph chunks,
    so they end bit for bit where the plain loop ends. In Float64 the cluster
    path agrees bit for bit too; in Float32 (multiply-add contraction decided
    per kernel) it agrees to rounding."""
    scen = [hills_rect(200, 150), hills_rect(64, 48), hills_rect(130, 70, stepper="fe")]
    T = 3.0
    wide = [sc.build(vf.SM103Backend(real)) for sc in scen]
    rw = E.simulate_batch(wide, T, options=E.BatchOptions(wide_cells=9000))  # the first and third go wide
    narrow = [sc.build(vf.SM103Backend(real)) for sc in scen]
    rn = E.simulate_batch(narrow, T, options=E.BatchOptions(wide_cells=-1))
    for k, (sc, a, b, x, y) in enumerate(zip(scen, wide, narrow, rw, rn)):
        assert x.status == y.status == N.VF_BATCH_OK and x.t == y.t == T
        plain = sc.build(vf.SM103Backend(real))
        vf.simulate_to_time(plain, T)
        assert plain.t == x.t
        if k != 1 or real == np.float64:  # wide (or Float64): the plain loop's kernels
            assert_bitwise(vf.current_interior_state(a), interior(plain))
        if real == np.float64:
            assert (x.steps, x.last_dt) == (y.steps, y.last_dt)
            assert_bitwise(vf.current_interior_state(a), interior(b))
        else:
            d = np.abs(vf.current_interior_state(a).h - vf.current_interior_state(b).h).max()
            assert d <= 1e-3, d


def test_wide_member_max_steps_is_exact():
    sc = hills_rect(200, 150)
    sim = sc.build(vf.SM103Backend())
    (r,) = E.simulate_batch([sim], 100.0, max_steps=37, options=E.BatchOptions(wide_cells=1))
    assert r.status == N.VF_BATCH_MAX_STEPS and r.steps == 37
    other = sc.build(vf.SM103Backend())
    (q,) = E.simulate_batch([other], 100.0, max_steps=37, options=E.BatchOptions(wide_cells=-1))
    assert (q.steps, q.t) == (37, r.t)
    assert_bitwise(vf.current_interior_state(sim), interior(other))
