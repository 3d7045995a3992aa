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
