"""The multi-rank plumbing of bench.py on CPU: world_size 2 over gloo (one
process per GPU on one node; replicas, so the only collectives are the
barrier around the timed region and the max-over-ranks of the step time)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    w, r, local, dist = bench.dist_setup()
    bench.barrier(dist)
    ms = bench.max_over_ranks(dist, 2.0 + 3.0 * r)  # rank 1 is the slow one
    val = bench.job_throughput(1000.0, w, ms)
    bench.barrier(dist)
    dist.destroy_process_group()
    out.put((r, w, local, ms, val))


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1]
    for r, w, local, ms, val in res:
        assert w == 2 and local == r
        assert ms == 5.0                          # the max over ranks, on every rank
        assert val == pytest.approx(2 * 1000.0 / 5e-3)  # whole-job units / slowest rank's time


def test_single_process_defaults(monkeypatch):
    import sys
    sys.path.insert(0, ROOT)
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    import bench
    assert bench.dist_setup() == (1, 0, 0, None)
    assert bench.max_over_ranks(None, 3.5) == 3.5
    assert bench.job_throughput(500.0, 1, 2.0) == pytest.approx(250000.0)
