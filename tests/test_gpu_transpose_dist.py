"""GPU: the pack / unpack kernels of the multi-rank transposes
(gbfft_transpose_pack / _unpack) through the C ABI.

Every rank of an emulated p_row x p_col grid runs in this one process (one
GPU, no rank waits for another): its pencil is packed on the GPU, the send
buffers are exchanged by slicing, and the received buffer is unpacked on the
GPU.  Each send buffer must equal the oracle's restated mem_split bit for
bit, and each rank's pencil after x -> y -> z -> y -> x must equal its slice
of the global array (the reference's test2d chain).  Blocks that would reach
past a buffer are rejected before any launch."""
import numpy as np
import pytest

from oracle import transpose as T
from test_decomp import LAYOUTS, _slice, emulated_chain

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _gpu_pack(checked):
    def pack(kind, a, dist, disp, size):
        import gbfft
        src = torch.from_numpy(np.ascontiguousarray(a)).cuda()
        send = torch.full((size,), 7, dtype=src.dtype, device="cuda")
        gbfft.transpose_pack(kind, src, send, dist, disp)
        torch.cuda.synchronize()
        out = send.cpu().numpy()
        ref = T.mem_split(kind, a, dist, disp, size)
        checked.append(np.array_equal(out, ref))
        return out
    return pack


def _gpu_unpack(kind, buf, shape, dist, disp):
    import gbfft
    recv = torch.from_numpy(buf).cuda()
    dst = torch.empty(shape, dtype=recv.dtype, device="cuda")
    gbfft.transpose_unpack(kind, recv, dst, dist, disp)
    torch.cuda.synchronize()
    return dst.cpu().numpy()


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex64, np.complex128])
@pytest.mark.parametrize("grid", [(17, 13, 11), (64, 48, 40)])
def test_gpu_pack_unpack_chain(layout, dtype, grid):
    nx, ny, nz = grid
    rng = np.random.default_rng(nx + ny + nz)
    g = rng.uniform(-1, 1, (nz, ny, nx))
    if np.iscomplexobj(np.zeros(1, dtype)):
        g = g + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    g = g.astype(dtype)
    checked = []
    steps = emulated_chain(g, *layout, _gpu_pack(checked), _gpu_unpack)
    assert checked and all(checked)
    for to, pencils, ds in steps:
        for r, d in enumerate(ds):
            assert np.array_equal(pencils[r], _slice(g, d, to))


def test_blocks_past_the_buffer_are_rejected_before_launch():
    import gbfft
    src = torch.zeros((4, 6, 8), dtype=torch.float32, device="cuda")
    send = torch.zeros(4 * 6 * 8 - 1, dtype=torch.float32, device="cuda")  # one element short
    before = gbfft.launch_count()
    with pytest.raises(gbfft.GbfftError, match="past the end"):
        gbfft.transpose_pack(gbfft.X_TO_Y, src, send, [4, 4], [0, 4 * 6 * 4])
    with pytest.raises(gbfft.GbfftError, match="add up"):
        gbfft.transpose_pack(gbfft.X_TO_Y, src, torch.zeros(500, device="cuda"), [4, 3], [0, 96])
    assert gbfft.launch_count() == before
