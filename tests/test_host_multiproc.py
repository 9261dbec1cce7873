"""CPU, world_size 2 (gloo): the benchmark's multi-rank timing path.

The FFT path runs as independent replicas per GPU (one grid per rank, no
data-path collective); what crosses ranks is only the barrier and the
max-over-ranks reduction of the step time, exercised here on gloo."""
import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(0.5 + rank)
    units = bench.sum_over_ranks(10)
    q.put((rank, t, units))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, units in res:
        assert t == pytest.approx(1.5)
        assert units == 20
