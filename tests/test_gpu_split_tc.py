"""GPU: the tcgen05 split-precision form (GBFFT_FORM_SPLIT_TC).  Strided
c2c passes of 1024 points run as two 32-point DFT products on the
5th-generation tensor cores (FP16 hi + lo operands in shared memory, FP32
accumulators in tensor memory); the other passes run as in the mma.sync
split form.  Every case against the FP64 oracle at rel-L2
<= 1e-6 (the accuracy bar a split-precision form must meet), with the tcgen05 kernel's
launch counter showing it ran: r2c / c2r in both formats with ragged line
counts (a tile of 4 lines partly past the array), per-row and flat-plane z
passes, c2c forward and backward along y and z, in place."""
import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-6


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def _engine(fmt, nx, ny, nz):
    import gbfft
    return gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE, form=gbfft.FORM_SPLIT_TC)


@pytest.mark.parametrize("fmt,shape", [(O.PHYSICAL_IN_X, (66, 1024, 12)), (O.PHYSICAL_IN_Z, (66, 1024, 10)),
                                       (O.PHYSICAL_IN_X, (30, 12, 1024)), (O.PHYSICAL_IN_X, (256, 1024, 64)),
                                       (O.PHYSICAL_IN_X, (34, 12, 1024)), (O.PHYSICAL_IN_X, (128, 1024, 256))])
def test_tc_form_r2c_c2r(fmt, shape):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + ny + nz + fmt)
    x = rng.standard_normal((nz, ny, nx)) + 3.0 * np.cos(2 * np.pi * 5 * np.arange(ny) / ny)[None, :, None]
    e = _engine(fmt, nx, ny, nz)
    before = gbfft.tc_pass_count()
    s = e.empty_spectral()
    e.r2c(torch.from_numpy(x.astype(np.float32)).cuda(), s)
    y = e.empty_physical()
    e.c2r(s, y)
    torch.cuda.synchronize()
    e.status()
    assert gbfft.tc_pass_count() > before
    assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= TOL
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= TOL
    e.close()


@pytest.mark.parametrize("shape", [(32, 1024, 8), (16, 8, 1024), (6, 1024, 5), (5, 4, 1024)])
def test_tc_form_c2c(shape):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * ny + nz)
    a = (rng.standard_normal((nz, ny, nx)) + 1j * rng.standard_normal((nz, ny, nx))).astype(np.complex64)
    e = _engine(O.PHYSICAL_IN_X, nx, ny, nz)
    x = torch.from_numpy(a).cuda()
    for isign in (gbfft.FORWARD, gbfft.BACKWARD):
        before = gbfft.tc_pass_count()
        ref = O.fft3d_c2c(a.astype(np.complex128), O.PHYSICAL_IN_X, isign)
        out = torch.empty_like(x)
        e.c2c(x, out, isign)
        z = x.clone()
        e.c2c(z, z, isign)  # in place
        torch.cuda.synchronize()
        e.status()
        assert gbfft.tc_pass_count() >= before + 2
        assert rel(out.cpu().numpy(), ref) <= TOL
        assert rel(z.cpu().numpy(), ref) <= TOL
    e.close()


def test_tc_form_is_scale_invariant():
    """One power of two scales each tile before the FP16 split: scaling the
    input by 2^k scales the output by exactly 2^k."""
    import gbfft
    nx, ny, nz = 16, 1024, 4
    a = (np.random.default_rng(5).standard_normal((nz, ny, nx)) * (1 + 1j)).astype(np.complex64)
    e = _engine(O.PHYSICAL_IN_X, nx, ny, nz)
    outs = []
    for k in (0, 20, -30):
        x = torch.from_numpy(a * np.float32(2.0 ** k)).cuda()
        o = torch.empty_like(x)
        e.c2c(x, o, gbfft.FORWARD)
        torch.cuda.synchronize()
        outs.append(o.cpu().numpy() / np.float32(2.0 ** k))
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    e.close()
