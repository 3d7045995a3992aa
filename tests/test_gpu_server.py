"""Served form: continuous batching under an HBM budget.  Every result must be
the same bits as the scene stepped alone in a one-scene world, whatever else
was resident, however the resident set was re-laid out around it and
whether the server's world grew in the meantime."""
import numpy as np
import pytest

from fluidgrid_gb300 import World, Server, FluidGridError, build, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _alone(spec, steps):
    w = World([spec])
    w.step(steps)
    p, v = w.download()
    w.close()
    return p, v


def _mix():
    ss = scenes.batched_scenes(seed=77, count=6, nmin=2048, nmax=12000)  # odd scenes carry a body
    steps = [5, 9, 3, 12, 7, 4]
    arrive = [0, 0, 2, 3, 3, 6]  # server step at which each request is submitted
    return ss, steps, arrive


def _run(server, ss, steps, arrive):
    ids = {}
    k = 0
    max_active = 0
    while len(ids) < len(ss) or not all(server.done(i) for i in ids.values()):
        for s, a in enumerate(arrive):
            if a == k and s not in ids:
                ids[s] = server.submit(ss[s], steps[s])
        info = server.step()
        max_active = max(max_active, info["active_scenes"])
        k += 1
        assert k < 200
    return ids, max_active


@pytest.mark.parametrize("graphs,via_host,depth", [(True, False, 0), (False, False, 0), (True, True, 0),
                                                   (True, False, 3), (False, True, 2)])
def test_results_equal_scene_alone(graphs, via_host, depth):
    """Every request's result equals its scene stepped alone: with and without
    graph replay, through host-parked growth, and with fg_server_step leaving
    up to `depth` steps running on the device."""
    ss, steps, arrive = _mix()
    with Server(budget_bytes=64 << 30, use_graphs=graphs, grow_via_host=via_host, pipeline_depth=depth) as srv:
        ids, max_active = _run(srv, ss, steps, arrive)
        assert max_active >= 3  # the scenes really overlapped on the device
        for s, rid in ids.items():
            info = srv.request(rid)
            assert info["steps_done"] == steps[s] and info["done_s"] >= info["admit_s"] >= info["submit_s"]
            p, v = srv.result(rid)
            pa, va = _alone(ss[s], steps[s])
            assert np.array_equal(p.view(np.uint32), pa.view(np.uint32)), s
            assert np.array_equal(v.view(np.uint32), va.view(np.uint32)), s


def test_budget_bounds_the_resident_set():
    ss, steps, arrive = _mix()
    with Server(budget_bytes=64 << 30) as probe:
        rids = [probe.submit(sp, 1) for sp in ss]
        probe.step()
        charge = [probe.request(r)["resident_bytes"] for r in rids]
    budget = int(2.2 * max(charge))  # two to three scenes at a time
    assert sum(charge) > budget
    with Server(budget_bytes=budget) as srv:
        ids = [srv.submit(s, n) for s, n in zip(ss, steps)]
        seen = 0
        while not all(srv.done(i) for i in ids):
            info = srv.step()
            assert info["resident_bytes"] <= budget
            seen = max(seen, info["active_scenes"])
        assert seen >= 2
        for s, rid in enumerate(ids):
            p, v = srv.result(rid)
            pa, _ = _alone(ss[s], steps[s])
            assert np.array_equal(p.view(np.uint32), pa.view(np.uint32)), s


def test_scene_larger_than_budget_is_refused():
    spec = scenes.dam_break_small()
    with Server(budget_bytes=1 << 20) as srv:
        with pytest.raises(FluidGridError):
            srv.submit(spec, 10)
    with Server(max_particles=1000) as srv:
        with pytest.raises(FluidGridError):
            srv.submit(spec, 10)


def test_particle_limit_queues_requests():
    ss, steps, arrive = _mix()
    limit = max(s.n for s in ss) + 100
    with Server(max_particles=limit) as srv:
        ids = [srv.submit(s, n) for s, n in zip(ss, steps)]
        while not all(srv.done(i) for i in ids):
            info = srv.step()
            assert info["active_particles"] <= limit
        st = srv.stats()
        assert st["queued"] == 0 and st["active"] == 0 and st["resident_bytes"] == 0
        assert st["particle_steps"] == sum(s.n * n for s, n in zip(ss, steps))


def _blocks(sizes, seed=5):
    rng = np.random.default_rng(seed)
    return [scenes.dam_break_request(n, 0, rng, name="block_%d" % k) for k, n in enumerate(sizes)]


def test_time_budget_bounds_the_resident_particles():
    """With a per-step time budget the server admits only as many particles
    as its learned rate says fit one step in the budget; without one it
    admits everything that fits the other budgets at once.  Results stay the
    scene alone's bits."""
    ss = _blocks([65536] * 8)
    steps = [6] * 8
    total = sum(s.n for s in ss)
    with Server(target_step_ms=0, max_particles=0) as free:
        ids = [free.submit(s, n) for s, n in zip(ss, steps)]
        info = free.step()
        assert info["active_particles"] == total
        while not all(free.done(i) for i in ids):
            free.step()
    with Server(target_step_ms=0.12, max_particles=0) as srv:
        ids = [srv.submit(s, n) for s, n in zip(ss, steps)]
        most = 0
        while not all(srv.done(i) for i in ids):
            info = srv.step()
            most = max(most, info["active_particles"])
        # predicted 0.1 ms + 0.9 ns per particle: one scene fits 0.12 ms, two
        # do not, and steps of fewer than 100k particles teach no new rate
        assert most == 65536
        for k in (0, 7):
            p, v = srv.result(ids[k])
            pa, va = _alone(ss[k], steps[k])
            assert np.array_equal(p.view(np.uint32), pa.view(np.uint32)), k


def test_reservation_backfills_only_requests_done_in_time():
    """When the oldest request does not fit it gets a reservation: a younger
    request passes it only if it is done before the oldest can fit
    (backfilling).  Without reservations (head_wait_s beyond the run) any
    younger request that fits passes it."""
    ss = _blocks([12000, 15000, 2000, 2000])
    steps = [4, 3, 3, 10]  # A runs 4 steps; C (3 steps) can finish before B fits, D (10) cannot
    order = {}
    for wait in (0.0, 1e9):
        with Server(max_particles=20000, target_step_ms=0, head_wait_s=wait) as srv:
            ids = [srv.submit(s, n) for s, n in zip(ss, steps)]
            while not all(srv.done(i) for i in ids):
                srv.step()
            order[wait] = [srv.request(i)["admit_s"] for i in ids]
            for k in range(4):
                p, v = srv.result(ids[k])
                pa, _ = _alone(ss[k], steps[k])
                assert np.array_equal(p.view(np.uint32), pa.view(np.uint32)), k
    a, b, c, d = order[0.0]
    assert c < b          # C is backfilled: it is done before B fits
    assert b <= d         # D would still be running: it waits behind B
    a, b, c, d = order[1e9]
    assert d < b          # no reservation: D passes B


def test_active_lists_the_resident_requests():
    ss = _blocks([3000, 4000, 5000])
    with Server() as srv:
        ids = [srv.submit(s, n) for s, n in zip(ss, (2, 4, 6))]
        assert srv.active() == []
        srv.step()
        assert sorted(srv.active()) == sorted(ids)
        srv.step()
        srv.step()
        assert sorted(srv.active()) == sorted(ids[1:])
        while not all(srv.done(i) for i in ids):
            srv.step()
        assert srv.active() == []
