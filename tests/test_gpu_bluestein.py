"""GPU: axis lengths with a prime factor above 256 -- inside one shared-memory
tile or beyond it -- run the chirp-z transform (Bluestein: two power-of-two
FFTs of a convolution of length >= 2n - 1) instead of a direct-sum stage.
Every case through the C ABI, r2c / c2r and c2c in both directions, the
prime axis contiguous (x) and strided (y, z), against pocketfft in FP64 and
the FP64 oracle (the reference's Glassman FFT, whose one stage over a large
prime builds its twiddles by a recurrence: its own distance from pocketfft
is added to the tolerance, as in the long-axis tests).  Tolerances: rel-L2
<= 1e-12 in double, <= 1e-6 in single (the direct sum this replaces reached
1.6e-6 on 8191 points in single)."""
import numpy as np
import pytest

from oracle import oracle as O
from test_gpu_long import _engine, pocket_c2c, pocket_c2r, pocket_r2c, rel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {"d": 1e-12, "s": 1e-6}


def check(got, oracle, pocket, prec):
    assert rel(got, pocket) <= TOL[prec]
    assert rel(got, oracle) <= TOL[prec] + rel(oracle, pocket)


# 257 (the smallest prime above the threshold), 1009, 4099, 8191 (one tile
# in FP32), 2 * 1009 and 3 * 997 (a large prime factor beside small ones),
# 16411 (beyond one tile); on every axis
C2C_CASES = [((257, 3, 2), "s"), ((1009, 2, 3), "d"), ((3, 4099, 2), "s"), ((2, 3, 2991), "d"),
             ((8191, 2, 2), "s"), ((2, 2018, 3), "s"), ((3, 2, 4099), "d"), ((16411, 2, 1), "s")]


@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
@pytest.mark.parametrize("shape,prec", C2C_CASES)
def test_chirp_z_c2c(fmt, shape, prec):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + 5 * ny + 11 * nz + fmt)
    a = rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    a = a.astype(np.complex128 if prec == "d" else np.complex64)
    e = _engine(fmt, shape, prec)
    x = torch.from_numpy(a).cuda()
    for isign in (gbfft.FORWARD, gbfft.BACKWARD):
        ref = O.fft3d_c2c(a.astype(np.complex128), fmt, isign, prec="d")
        pk = pocket_c2c(a, isign)
        y = torch.empty_like(x)
        e.c2c(x, y, isign)
        torch.cuda.synchronize()
        check(y.cpu().numpy(), ref, pk, prec)
        z = x.clone()
        e.c2c(z, z, isign)  # in place
        torch.cuda.synchronize()
        check(z.cpu().numpy(), ref, pk, prec)
    e.status()
    e.close()


# the prime axis as the real axis (odd line counts: a pair with one real
# line) and as a c2c axis of a real transform
REAL_CASES = [(O.PHYSICAL_IN_X, (1009, 3, 5), "s"), (O.PHYSICAL_IN_X, (4099, 2, 3), "d"),
              (O.PHYSICAL_IN_Z, (3, 5, 8191), "s"), (O.PHYSICAL_IN_X, (6, 2018, 3), "d"),
              (O.PHYSICAL_IN_Z, (7, 3, 2991), "s"), (O.PHYSICAL_IN_X, (16, 9, 257), "s"),
              (O.PHYSICAL_IN_X, (16411, 3, 1), "d")]


@pytest.mark.parametrize("fmt,shape,prec", REAL_CASES)
def test_chirp_z_r2c_c2r(fmt, shape, prec):
    nx, ny, nz = shape
    rng = np.random.default_rng(3 * nx + ny + nz + fmt)
    rt, ct = (np.float64, np.complex128) if prec == "d" else (np.float32, np.complex64)
    x = rng.uniform(-1, 1, (nz, ny, nx)).astype(rt)
    ref = O.fft3d_r2c(x.astype(np.float64), fmt, prec="d")
    e = _engine(fmt, shape, prec)
    spec = e.empty_spectral()
    e.r2c(torch.from_numpy(x).cuda(), spec)
    torch.cuda.synchronize()
    check(spec.cpu().numpy(), ref, pocket_r2c(x, fmt), prec)
    # c2r of a non-Hermitian spectrum: the reference's rule decides
    s = (ref + 0.3 * (rng.standard_normal(ref.shape) + 1j * rng.standard_normal(ref.shape))).astype(ct)
    refb = O.fft3d_c2r(s.astype(np.complex128), nx, ny, nz, fmt, prec="d")
    sd = torch.from_numpy(s).cuda()
    back = e.empty_physical()
    e.c2r(sd, back)
    torch.cuda.synchronize()
    check(back.cpu().numpy(), refb, pocket_c2r(s, shape, fmt), prec)
    assert torch.equal(sd.cpu(), torch.from_numpy(s))  # the input is preserved
    e.status()
    e.close()


def test_chirp_z_skip_flags():
    """A skipped prime axis is left alone; the others are transformed."""
    import gbfft
    nx, ny, nz = 12, 1009, 10
    rng = np.random.default_rng(1009)
    a = (rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))).astype(np.complex64)
    for skip in ((False, True, False), (True, False, True)):
        e = _engine(O.PHYSICAL_IN_X, (nx, ny, nz), "s", skip=skip)
        x = torch.from_numpy(a).cuda()
        y = torch.empty_like(x)
        e.c2c(x, y, gbfft.FORWARD)
        torch.cuda.synchronize()
        ref = O.fft3d_c2c(a.astype(np.complex128), O.PHYSICAL_IN_X, O.FORWARD, skip=skip, prec="d")
        assert rel(y.cpu().numpy(), ref) <= TOL["s"]
        e.close()
