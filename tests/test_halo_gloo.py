"""CPU, world sizes 2 and 4 (gloo): the halo-update driver (gbfft.update_halo)
exchanging with real point-to-point messages between processes, a numpy box
copy standing in for the GPU kernel; every rank's halo-extended array must
equal the oracle's (oracle/halo.py) on the cells the reference defines, bit
for bit -- periodic and non-periodic dimensions, all three pencils, halo
levels 1 and 2."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from halo_cases import CASES


def _worker(rank, world, port, case, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import gbfft
    from halo_cases import global_field, np_copy, oracle, piece
    grid, p_row, p_col, pencil, level, periodic = case
    g = global_field(grid)
    ds, arrs, masks = oracle(g, grid, p_row, p_col, pencil, level, periodic)
    d = ds[rank]
    out = gbfft.update_halo(torch.from_numpy(piece(g, d, pencil)), level, d, pencil, periodic, copy=np_copy)
    got = out.numpy()
    ok = got.shape == arrs[rank].shape and np.array_equal(got[masks[rank]], arrs[rank][masks[rank]])
    q.put((rank, ok))
    dist.destroy_process_group()


@pytest.mark.parametrize("case", [c for c in CASES if c[1] * c[2] > 1])
def test_update_halo_gloo(case):
    world = case[1] * case[2]
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, case, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(ok for _, ok in res), res
