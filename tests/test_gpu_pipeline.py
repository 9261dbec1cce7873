"""GPU: pipelined persistent passes (gbfft_engine_set_pipeline) give the
same transform as the one-shot kernels: every pass kind, both formats,
contiguous and strided lines of 256, 512 and 1024 points, line counts that
leave ragged last tiles, against the FP64 oracle (FP32 tolerance)."""
import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 2e-6  # rel-L2 against the FP64 oracle (FP32 data)
KINDS = ("r2c", "c2r", "c2c_x", "c2c_y", "c2c_z")


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("depth", [2, 3])
@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("shape", [(1024, 256, 64), (256, 1024, 18), (512, 30, 512), (6, 256, 1024), (20, 512, 9)])
def test_pipelined_r2c_c2r_matches_oracle(depth, fmt, shape):
    import gbfft
    nx, ny, nz = shape
    x = np.random.default_rng(nx + ny + nz + depth + fmt).standard_normal((nz, ny, nx))
    e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    for k in KINDS:
        e.set_pipeline(k, depth)
    assert all(e.pipeline()[k] == depth for k in KINDS)
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    s = e.empty_spectral()
    e.r2c(xd, s)
    assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= TOL
    y = e.empty_physical()
    e.c2r(s, y)
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= TOL
    e.close()


@pytest.mark.parametrize("depth", [2, 3])
@pytest.mark.parametrize("shape", [(1024, 512, 20), (256, 7, 1024)])
def test_pipelined_c2c_matches_oracle(depth, shape):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(depth)
    a = rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    e = gbfft.Engine(1, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    for k in KINDS:
        e.set_pipeline(k, depth)
    ad = torch.from_numpy(a.astype(np.complex64)).cuda()
    out = torch.empty_like(ad)
    e.c2c(ad, out, -1)
    assert rel(out.cpu().numpy(), O.fft3d_c2c(a.copy(), 1, -1)) <= TOL
    back = torch.empty_like(ad)
    e.c2c(out, back, 1)
    assert rel(back.cpu().numpy() / (nx * ny * nz), a) <= TOL
    e.close()


@pytest.mark.parametrize("lines", [1, 2, 4, 8, 16, 32])
def test_pipelined_tile_heights(lines):
    import gbfft
    nx, ny, nz = 1024, 1024, 3
    x = np.random.default_rng(lines).standard_normal((nz, ny, nx))
    e = gbfft.Engine(1, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    for k in KINDS:
        e.set_pipeline(k, 3)
        try:
            e.set_tile(k, lines)
        except gbfft.GbfftError:
            pass
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    s = e.empty_spectral()
    e.r2c(xd, s)
    assert rel(s.cpu().numpy(), O.fft3d_r2c(x, 1)) <= TOL
    y = e.empty_physical()
    e.c2r(s, y)
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= TOL
    e.close()


def test_pipeline_depth_is_validated():
    import gbfft
    e = gbfft.Engine(1, 256, 256, 4, prec=gbfft.PREC_SINGLE)
    with pytest.raises(gbfft.GbfftError):
        e.set_pipeline("c2c_y", 5)
    e.close()

