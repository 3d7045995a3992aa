"""bench.py's multi-rank host path on CPU: two gloo ranks (the scene does not
shard, so ranks are independent replicas; the only communication is the
host barrier and the max/sum of the timings)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_info()
    d = bench.Dist(w)
    d.barrier()
    mx = d.reduce(10.0 + rank, "max")
    sm = d.reduce(1.5 * (rank + 1), "sum")
    d.barrier()
    d.close()
    q.put((r, w, local, mx, sm))


def test_two_gloo_ranks_reduce_max_and_sum():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[:3] for o in out] == [(0, 2, 0), (1, 2, 1)]
    for o in out:
        assert o[3] == 11.0 and o[4] == 4.5


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        workload = "dam_break_16k"
        steps = 1
        warmup = 0
        gpus = 2
    assert bench.run_reference(A(), rank=1, world=2) == 0  # other ranks exit without work
