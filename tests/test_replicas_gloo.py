"""Replica timing across ranks (the N > 1 path of bench.py), with two gloo ranks
on the CPU: max of the per-rank times, sum of the per-rank particle updates."""
import os
import socket

import torch.multiprocessing as mp

from cmag_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    secs, units = replicas.aggregate(dist, seconds=1.0 + rank, units=100.0 * (rank + 1))
    q.put((rank, secs, units, replicas.replica_seed(1973, rank)))
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, secs, units, seed in out:
        assert secs == 2.0 and units == 300.0
    assert out[0][3] != out[1][3]


def test_single_process_passthrough():
    assert replicas.aggregate(None, 1.5, 10) == (1.5, 10.0)
