"""GPU: cluster launches of the one-shot kernels (gbfft_engine_set_cluster)
give the same transform: clusters of 2, 4 and 8 CTAs, with and without the
start barrier, tile counts that are not multiples of the cluster size (the
grid is padded with CTAs that own no line), both formats, against the FP64
oracle (FP32 tolerance)."""
import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 2e-6  # rel-L2 against the FP64 oracle (FP32 data)
KINDS = ("r2c", "c2r", "c2c_x", "c2c_y", "c2c_z")


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("ctas,sync", [(2, 0), (2, 1), (4, 1), (8, 1), (8, 0)])
@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("shape", [(1024, 1024, 8), (130, 512, 64), (64, 256, 1024), (1000, 33, 512)])
def test_cluster_launch_matches_oracle(ctas, sync, fmt, shape):
    import gbfft
    nx, ny, nz = shape
    x = np.random.default_rng(nx + ny + nz + ctas + sync + fmt).standard_normal((nz, ny, nx))
    e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    for k in KINDS:
        e.set_cluster(k, ctas, sync)
    assert e.cluster()["c2c_y"] == (ctas, sync)
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    s = e.empty_spectral()
    e.r2c(xd, s)
    assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= TOL
    y = e.empty_physical()
    e.c2r(s, y)
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= TOL
    e.close()


def test_cluster_launch_c2c_with_tiles():
    import gbfft
    nx, ny, nz = 40, 1024, 512
    rng = np.random.default_rng(4)
    a = rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    ref = O.fft3d_c2c(a.copy(), 1, -1)
    e = gbfft.Engine(1, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    ad = torch.from_numpy(a.astype(np.complex64)).cuda()
    for ctas in (2, 4):
        for k in KINDS:
            e.set_cluster(k, ctas, 1)
        for lines in (0, 4, 16):
            for k in ("c2c_y", "c2c_z"):
                e.set_tile(k, lines)
            out = torch.empty_like(ad)
            e.c2c(ad, out, -1)
            assert rel(out.cpu().numpy(), ref) <= TOL, (ctas, lines)
            back = torch.empty_like(ad)
            e.c2c(out, back, 1)
            assert rel(back.cpu().numpy() / (nx * ny * nz), a) <= TOL, (ctas, lines)
    e.close()


def test_cluster_size_is_validated():
    import gbfft
    e = gbfft.Engine(1, 256, 256, 4, prec=gbfft.PREC_SINGLE)
    with pytest.raises(gbfft.GbfftError):
        e.set_cluster("c2c_y", 3)
    e.close()
