"""The multi-GPU form of bench.py is replicas only: each rank evaluates its own
field and the job time is the slowest rank's.  The cross-rank aggregation is
tested here with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r took (r + 1) seconds for 3 steps of 10 pairs each
    value, total = bench.aggregate(float(rank + 1), 3, 10.0, world, dist)
    out.put((rank, value, total))
    dist.destroy_process_group()


def test_replica_aggregation_takes_slowest_rank_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
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
    for _, value, total in res:
        assert total == 2.0                    # max over ranks
        assert value == 2 * 3 * 10.0 / 2.0     # whole-job pairs/s


def test_single_process_aggregation():
    import bench
    assert bench.aggregate(2.0, 4, 5.0, 1, None) == (10.0, 2.0)
