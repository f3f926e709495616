"""The serving engine (vf_server_*): requests admitted by HBM budget and run
with continuous batching give the results of plain simulate_to_time runs, and a
request's result is the same alone and in a mix of overlapping requests."""
import time

import numpy as np
import pytest

import volumefluxes_sm103 as vf
from volumefluxes_sm103 import _native as N
from volumefluxes_sm103 import scenarios as S
from volumefluxes_sm103.serving import Server
from vfhelpers import hills_rect

pytestmark = pytest.mark.gpu

GB = 1 << 30


def requests(n, seed=5, side_cap=200):
    out = []
    for k, sp in enumerate(S.ensemble_specs(n, seed=seed)):
        sp.side = min(sp.side, side_cap)
        real = np.float32 if k % 2 == 0 else np.float64
        out.append((S.ensemble_member(sp), real, min(sp.endtime, 6.0 if real == np.float64 else 20.0)))
    return out


def wait_for(srv, cond, timeout=60.0):
    t0 = time.time()
    while not cond(srv.stats()):
        assert time.time() - t0 < timeout, srv.stats()
        time.sleep(0.0005)


def drain(srv, tickets, timeout=300.0):
    done = {}
    t0 = time.time()
    while len(done) < len(tickets):
        for tk in srv.poll():
            done[tk] = srv.result(tk)
        assert time.time() - t0 < timeout, "server did not drain"
        time.sleep(0.001)
    return [done[t] for t in tickets]


def plain(sc, real, T):
    sim = sc.build(vf.SM103Backend(real))
    vf.simulate_to_time(sim, T)
    g = vf.current_interior_state(sim)
    return sim.t, (g.h.copy(), g.hu.copy(), g.hv.copy())


def test_served_results_equal_plain_runs():
    reqs = requests(6)
    with Server(8 * GB) as srv:
        tickets = [srv.submit(sc, real, T) for sc, real, T in reqs]
        res = drain(srv, tickets)
        assert srv.stats()["used_bytes"] == 0
    for (sc, real, T), r in zip(reqs, res):
        assert r.status == N.VF_BATCH_OK and r.t == T
        t, want = plain(sc, real, T)
        assert t == r.t
        for a, b in zip((r.state.h, r.state.hu, r.state.hv), want):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("real", [np.float64, np.float32])
def test_request_is_the_same_alone_and_in_the_mix(real):
    probe = hills_rect(96, 80)
    T = 4.0 if real == np.float64 else 10.0
    with Server(8 * GB) as srv:
        (alone,) = drain(srv, [srv.submit(probe, real, T)])
    others = requests(5, seed=9)
    with Server(8 * GB) as srv:
        first = [srv.submit(sc, r, t) for sc, r, t in others[:3]]
        wait_for(srv, lambda st: st["running"] == 3)  # the first three run
        mid = srv.submit(probe, real, T)  # arrives while they run
        last = [srv.submit(sc, r, t) for sc, r, t in others[3:]]
        res = drain(srv, first + [mid] + last)
        assert srv.stats()["launches"] >= 2
    mixed = res[3]
    assert (mixed.t, mixed.steps, mixed.last_dt) == (alone.t, alone.steps, alone.last_dt)
    for a, b in zip((mixed.state.h, mixed.state.hu, mixed.state.hv), (alone.state.h, alone.state.hu, alone.state.hv)):
        assert np.array_equal(a, b)


def test_admission_waits_for_memory():
    sc = hills_rect(128, 128)
    need = 0
    with Server(1 << 40) as srv:  # measure one request's charge
        tk = srv.submit(sc, np.float64, 30.0)
        wait_for(srv, lambda st: st["running"] == 1)
        need = srv.stats()["used_bytes"]
        drain(srv, [tk])
    assert need > 0
    with Server(2 * need + need // 2) as srv:  # room for two at a time
        tickets = [srv.submit(sc, np.float64, 30.0) for _ in range(5)]
        wait_for(srv, lambda st: st["running"] == 2)
        st = srv.stats()
        assert st["queued"] == 3 and st["used_bytes"] == 2 * need
        res = drain(srv, tickets)
        assert max(r.admit_s for r in res[2:]) >= min(r.done_s for r in res[:2])  # admitted as memory freed
        assert srv.stats()["used_bytes"] == 0
    assert all(r.status == N.VF_BATCH_OK and r.t == 30.0 for r in res)
    assert all(np.array_equal(r.state.h, res[0].state.h) for r in res)
