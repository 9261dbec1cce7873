"""GPU: the split-precision tensor-core form (GBFFT_FORM_SPLIT).

Axes of 256, 512 and 1024 points run their radix-16 stages as FP16 hi+lo
DFT-matrix products on the tensor cores with FP32 accumulation; other axes
run the plain FP32 kernels.  The form must stay within rel-L2 1e-6 of the
FP64 oracle, forward and round trip (the same bar as the plain FP32 form
plus a small margin: the split keeps about 22 bits per operand)."""
import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-6  # rel-L2 against the FP64 oracle, forward and round trip


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def split_engine(fmt, nx, ny, nz):
    import gbfft
    return gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE, form=gbfft.FORM_SPLIT)


@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("shape", [(256, 256, 256), (1024, 64, 512), (512, 1024, 32), (64, 512, 1024)])
def test_split_r2c_c2r_matches_fp64_oracle(fmt, shape):
    nx, ny, nz = shape
    x = np.random.default_rng(nx + ny + nz + fmt).uniform(-1, 1, (nz, ny, nx))
    e = split_engine(fmt, nx, ny, nz)
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    s = e.empty_spectral()
    e.r2c(xd, s)
    torch.cuda.synchronize()
    assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= TOL
    y = e.empty_physical()
    e.c2r(s, y)
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= TOL
    e.status()
    e.close()


@pytest.mark.parametrize("shape", [(256, 256, 64), (1024, 8, 512)])
def test_split_c2c_forward_backward(shape):
    nx, ny, nz = shape
    rng = np.random.default_rng(7)
    a = rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    e = split_engine(1, nx, ny, nz)
    ad = torch.from_numpy(a.astype(np.complex64)).cuda()
    out = torch.empty_like(ad)
    e.c2c(ad, out, -1)
    assert rel(out.cpu().numpy(), O.fft3d_c2c(a.copy(), 1, -1)) <= TOL
    back = torch.empty_like(ad)
    e.c2c(out, back, 1)
    assert rel(back.cpu().numpy() / (nx * ny * nz), a) <= TOL
    e.close()


@pytest.mark.parametrize("fmt,shape", [(1, (20, 256, 7)), (1, (1024, 5, 3)), (3, (6, 5, 1024)), (3, (9, 3, 512))])
def test_split_ragged_tiles(fmt, shape):
    # line counts that are not multiples of the 4 (contiguous) or 8
    # (strided) lines of a tile, and odd real line counts (r2c pairs)
    nx, ny, nz = shape
    x = np.random.default_rng(11).standard_normal((nz, ny, nx))
    e = split_engine(fmt, nx, ny, nz)
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    s = e.empty_spectral()
    e.r2c(xd, s)
    assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= TOL
    y = e.empty_physical()
    e.c2r(s, y)
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= TOL
    e.close()


def test_split_is_exactly_scale_invariant():
    # every butterfly is scaled by a power of two before the FP16 split, so
    # scaling the input by 2^k scales the spectrum by exactly 2^k
    nx, ny, nz = 256, 64, 512
    x = np.random.default_rng(5).standard_normal((nz, ny, nx)).astype(np.float32)
    e = split_engine(1, nx, ny, nz)
    s0, s1, s2 = e.empty_spectral(), e.empty_spectral(), e.empty_spectral()
    xd = torch.from_numpy(x).cuda()
    e.r2c(xd, s0)
    e.r2c(xd * 2.0 ** 60, s1)
    e.r2c(xd * 2.0 ** -60, s2)
    assert torch.equal(s1, s0 * 2.0 ** 60)
    assert torch.equal(s2, s0 * 2.0 ** -60)
    e.close()


def test_split_rejects_double_precision():
    import gbfft
    with pytest.raises(gbfft.GbfftError):
        gbfft.Engine(1, 256, 256, 256, prec=gbfft.PREC_DOUBLE, form=gbfft.FORM_SPLIT)


def test_split_and_plain_agree_closely():
    import gbfft
    nx, ny, nz = 1024, 128, 256
    x = torch.randn((nz, ny, nx), device="cuda", generator=torch.Generator("cuda").manual_seed(3))
    p = gbfft.Engine(1, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    q = split_engine(1, nx, ny, nz)
    sp, sq = p.empty_spectral(), q.empty_spectral()
    p.r2c(x, sp)
    q.r2c(x, sq)
    d = float(torch.linalg.vector_norm(sp - sq) / torch.linalg.vector_norm(sp))
    assert d <= TOL
    p.close()
    q.close()


@pytest.mark.parametrize("fmt,shape", [(1, (256, 48, 27)), (3, (96, 50, 512)), (1, (48, 40, 27))])
def test_split_on_non_power_of_two_axes(fmt, shape):
    # only the 256-, 512- and 1024-point axes have split stages; the other
    # axes of the same engine run the plain FP32 kernels (a grid with none,
    # like 48 x 40 x 27, is the plain form throughout)
    nx, ny, nz = shape
    x = np.random.default_rng(17).uniform(-1, 1, (nz, ny, nx))
    e = split_engine(fmt, nx, ny, nz)
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    s = e.empty_spectral()
    e.r2c(xd, s)
    assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= TOL
    y = e.empty_physical()
    e.c2r(s, y)
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= TOL
    e.status()
    e.close()
