"""CPU, world sizes 2 and 4 (gloo): the multi-rank transpose driver
(gbfft.transpose_dist) on real process groups -- the row / column groups of
a p_row x p_col grid, the ALLTOALLV counts and displacements of the C ABI
(gbfft_decomp_counts) -- with the oracle's restated pack / unpack standing
in for the GPU kernels on CPU tensors.  Every rank transposes its piece of
a global array x -> y -> z -> y -> x and must hold its slice of the global
array, bit for bit, after every step."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _oracle_pack(kind, src, send, dist_, disp):
    from oracle import transpose as T
    send.copy_(torch.from_numpy(T.mem_split(kind, src.numpy(), dist_, disp, send.numel())))


def _oracle_unpack(kind, recv, dst, dist_, disp):
    from oracle import transpose as T
    dst.copy_(torch.from_numpy(T.mem_merge(kind, recv.numpy(), tuple(dst.shape), dist_, disp)))


def _slice(g, d, pencil):
    st, en = getattr(d, pencil + "st"), getattr(d, pencil + "en")
    return g[st[2] - 1:en[2], st[1] - 1:en[1], st[0] - 1:en[0]]


def _worker(rank, world, port, layout, grid, dtype, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import gbfft
    p_row, p_col = layout
    nx, ny, nz = grid
    groups = gbfft.pencil_groups(p_row, p_col)
    d = gbfft.Decomp(nx, ny, nz, p_row, p_col, rank)
    rng = np.random.default_rng(11)
    g = rng.uniform(-1, 1, (nz, ny, nx))
    if dtype.startswith("complex"):
        g = g + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    g = g.astype(dtype)
    cur = torch.from_numpy(np.ascontiguousarray(_slice(g, d, "x")))
    ok = True
    for kind, to in ((gbfft.X_TO_Y, "y"), (gbfft.Y_TO_Z, "z"), (gbfft.Z_TO_Y, "y"), (gbfft.Y_TO_X, "x")):
        dst = torch.empty(d.shape(to), dtype=cur.dtype)
        gbfft.transpose_dist(kind, cur, dst, d, groups, pack=_oracle_pack, unpack=_oracle_unpack)
        ok = ok and np.array_equal(dst.numpy(), _slice(g, d, to))
        cur = dst
    q.put((rank, ok))
    dist.destroy_process_group()


def _run(world, layout, grid, dtype):
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, layout, grid, dtype, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(ok for _, ok in res), res


@pytest.mark.parametrize("layout", [(1, 2), (2, 1)])
def test_transpose_chain_two_ranks(layout):
    _run(2, layout, (17, 13, 11), "float64")


def test_transpose_chain_four_ranks_complex():
    _run(4, (2, 2), (17, 13, 11), "complex128")


def test_transpose_chain_four_ranks_slab_single():
    _run(4, (1, 4), (9, 8, 10), "complex64")
