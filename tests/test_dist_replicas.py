"""world_size-2 gloo test (CPU) of the replica aggregation used by
bench.py --gpus N: max over ranks of the time, sum of the work."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    from les_gb300.dist import aggregate
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank            # rank 1 is the slow one
    pts = 1000 * (rank + 1)
    out = aggregate(ms, pts)
    dist.destroy_process_group()
    q.put((rank, out))


def test_replica_aggregation_two_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        ms, pts, rate = res[r]
        assert ms == 150.0 and pts == 3000.0
        assert abs(rate - 3000.0 / 0.150) < 1e-6
