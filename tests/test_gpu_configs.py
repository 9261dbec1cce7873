"""GPU: the benchmark configurations at their full sizes, against the FP64
oracle, through the C ABI.

  * 256^3 complex64 c2c, forward and backward, both formats (seeded uniform
    [-1, 1) real and imaginary parts, seed 2): rel-L2 <= 2e-6 against the
    oracle's double build on the same (complex64-rounded) input;
  * the 64 uneven FP32 grids of the batched benchmark (each dimension from
    {32, 48, 64, 96, 128, 192, 256}, format by a seeded coin), forward in one
    persistent launch, every grid against the oracle's double build, then
    forward + backward replayed from a CUDA graph (the real arrays become
    nx ny nz times the input).
"""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


@pytest.fixture(scope="module", autouse=True)
def _threads():
    O.set_threads(os.cpu_count() or 1)


@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
def test_c2c_256_cubed_complex64_against_fp64_oracle(fmt):
    import gbfft
    n = 256
    rng = np.random.default_rng(2)
    a = (rng.uniform(-1, 1, (n, n, n)) + 1j * rng.uniform(-1, 1, (n, n, n))).astype(np.complex64)
    e = gbfft.Engine(fmt, n, n, n, prec=gbfft.PREC_SINGLE)
    x = torch.from_numpy(a).cuda()
    y = torch.empty_like(x)
    e.c2c(x, y, gbfft.FORWARD)
    torch.cuda.synchronize()
    ref = O.fft3d_c2c(a.astype(np.complex128), fmt, O.FORWARD, prec="d")
    assert rel(y.cpu().numpy(), ref) <= 2e-6
    # backward from the oracle's spectrum rounded to complex64
    s = ref.astype(np.complex64)
    refb = O.fft3d_c2c(s.astype(np.complex128), fmt, O.BACKWARD, prec="d")
    xs = torch.from_numpy(s).cuda()
    e.c2c(xs, y, gbfft.BACKWARD)
    torch.cuda.synchronize()
    assert rel(y.cpu().numpy(), refb) <= 2e-6
    assert torch.equal(xs.cpu(), torch.from_numpy(s))  # c2c leaves its input alone
    e.close()


def test_batch_of_64_uneven_grids_against_fp64_oracle():
    import bench
    import gbfft
    dims = bench.batch_dims()
    assert len(dims) == 64
    rng = np.random.default_rng(7)
    batch = gbfft.Batch()
    items = []
    for nx, ny, nz, fmt in dims:
        e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
        a = rng.uniform(-1, 1, (nz, ny, nx)).astype(np.float32)
        x = torch.from_numpy(a).cuda()
        s = e.empty_spectral()
        batch.add(e, x, s)
        items.append((e, a, x, s, fmt))
    assert batch.info()["persistent"]
    batch.run(1)
    torch.cuda.synchronize()
    batch.status()
    worst = 0.0
    for e, a, x, s, fmt in items:
        ref = O.fft3d_r2c(a.astype(np.float64), fmt, prec="d")
        worst = max(worst, rel(s.cpu().numpy(), ref))
    assert worst <= 2e-6
    stream = torch.cuda.Stream()
    batch.graph_build(stream)
    batch.graph_launch(stream)
    stream.synchronize()
    batch.status()
    for e, a, x, s, fmt in items:
        n = e.nx * e.ny * e.nz
        assert rel((x / n).cpu().numpy(), a) <= 1e-6
    batch.close()
