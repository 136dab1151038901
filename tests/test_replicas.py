"""bench.py's multi-GPU arm runs independent replicas of the well (the
single-well step does not shard).  Its host-side aggregation -- the slowest
rank's time and the sum of the units all ranks processed -- is checked here
with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    t, u = bench.reduce_replicas(dist, 10.0 + 5.0 * rank, 1000 * (rank + 1), device="cpu")
    q.put((rank, t, u))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, t, u in res:
        assert t == 15.0          # the slowest rank's time
        assert u == 3000.0        # units of both ranks


def test_single_process_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_replicas(None, 7.5, 42) == (7.5, 42.0)
