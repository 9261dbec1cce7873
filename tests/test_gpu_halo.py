"""GPU: the halo update (gbfft.update_halo) with its device box copies
(gbfft_box_copy) through the C ABI.  Every rank of the grid runs in its own
host thread of this one process (one GPU; the device work of all threads is
ordered on the default stream, no kernel waits for another), exchanging its
slabs through an in-process mailbox in update_halo's message batches; each rank's
halo-extended array must equal the oracle's (oracle/halo.py) on the cells
the reference defines, bit for bit.  Boxes outside an array are rejected
before any launch."""
import threading

import numpy as np
import pytest

from halo_cases import CASES, global_field, oracle, piece

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


class Mailbox:
    """The batches of point-to-point messages of all ranks, in lockstep."""

    def __init__(self, nranks):
        self.barrier = threading.Barrier(nranks)
        self.box = {}
        self.lock = threading.Lock()

    def exchange(self, rank):
        def fn(sends, recvs):
            with self.lock:
                for t, peer in sends:
                    if t is not None and peer is not None:
                        self.box[(rank, peer)] = t
            self.barrier.wait()
            for t, peer in recvs:
                if t is not None and peer is not None:
                    t.copy_(self.box[(peer, rank)])
            self.barrier.wait()
            with self.lock:
                for t, peer in sends:
                    if t is not None and peer is not None:
                        self.box.pop((rank, peer), None)
            self.barrier.wait()
        return fn


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("dtype", [np.float64, np.complex64])
def test_update_halo_gpu(case, dtype):
    import gbfft
    grid, p_row, p_col, pencil, level, periodic = case
    g = global_field(grid)
    if np.iscomplexobj(np.zeros(1, dtype)):
        g = g + 0.5j * g
    g = g.astype(dtype)
    ds, arrs, masks = oracle(g, grid, p_row, p_col, pencil, level, periodic)
    n = len(ds)
    mb = Mailbox(n)
    outs = [None] * n
    errs = []

    def run(r):
        try:
            x = torch.from_numpy(piece(g, ds[r], pencil)).cuda()
            outs[r] = gbfft.update_halo(x, level, ds[r], pencil, periodic, exchange=mb.exchange(r))
        except Exception as e:  # pragma: no cover - reported below
            errs.append(e)
            mb.barrier.abort()

    threads = [threading.Thread(target=run, args=(r,)) for r in range(n)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=120)
    assert not errs, errs
    torch.cuda.synchronize()
    for r in range(n):
        got = outs[r].cpu().numpy()
        assert got.shape == arrs[r].shape
        assert np.array_equal(got[masks[r]], arrs[r][masks[r]])


def test_box_outside_the_array_is_rejected():
    import gbfft
    a = torch.zeros((4, 5, 6), device="cuda")
    b = torch.zeros((4, 5, 6), device="cuda")
    before = gbfft.launch_count()
    with pytest.raises(gbfft.GbfftError, match="outside"):
        gbfft.box_copy(a, [1, 0, 0], b, [0, 0, 0], [6, 5, 4])
    with pytest.raises(gbfft.GbfftError, match="outside"):
        gbfft.box_copy(a, [0, 0, 0], b, [0, 0, 1], [6, 5, 4])
    assert gbfft.launch_count() == before
