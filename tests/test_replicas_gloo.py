"""The N > 1 path of bench.py on CPU: two gloo ranks (one replica each, no data-path collective)
agree on the maximum time and the summed value, as the timed region does on GPUs with NCCL."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import bench
    dist = bench.Dist(world)
    try:
        assert dist.backend == "gloo"
        dist.barrier()
        ms = [10.0, 12.5][rank]            # per-rank timed region
        units = [100.0, 100.0][rank]       # each replica's units per step
        t = dist.max(ms)
        v = dist.sum(units) / (t / 1e3)    # whole-job throughput over the slowest rank
        out.put((rank, t, v))
    finally:
        dist.close()


def test_two_gloo_replicas_reduce_time_and_value():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    for rank, t, v in res:
        assert t == pytest.approx(12.5)
        assert v == pytest.approx(200.0 / 12.5e-3)
