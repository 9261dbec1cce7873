"""GPU: axes longer than one shared-memory tile -- more than 8192 points, or
FP64 lines whose two tile buffers do not fit -- run stage by stage through
global memory (the long-axis path), for any length: powers of two, mixed
radices and primes up to 256 as direct-sum stages, larger primes as the
chirp-z transform (the reference's SPCFFT takes any N:
src/glassman.f90:29-67).  Every case through the C ABI against the
FP64 oracle and against pocketfft (numpy) in FP64.  Tolerances as the parity
tests, rel-L2 <= 1e-12 in double, <= 2e-6 in single, against pocketfft; and
against the oracle the same plus the oracle's own distance from pocketfft:
on a large prime the reference's one Glassman stage builds its twiddles by a
recurrence across the whole prime (src/glassman.f90:84-96) and is accurate
to only about 1e-9 in double (8209 points: 5.8e-10), while the GPU's direct
sum uses exactly rounded twiddles.

Also strided passes with more planes than one launch's grid allows (a z
pass over more than 65535 rows), which run as several launches.
"""
import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {"d": 1e-12, "s": 2e-6}


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def check(got, oracle, pocket, prec):
    assert rel(got, pocket) <= TOL[prec]
    assert rel(got, oracle) <= TOL[prec] + rel(oracle, pocket)


def pocket_c2c(a, isign):
    a = a.astype(np.complex128)
    return np.fft.fftn(a) if isign < 0 else np.fft.ifftn(a) * a.size


def pocket_r2c(x, fmt):
    return np.fft.rfftn(x.astype(np.float64), axes=(0, 1, 2) if fmt == O.PHYSICAL_IN_X else (2, 1, 0))


def pocket_c2r(s, shape, fmt):
    nx, ny, nz = shape
    if fmt == O.PHYSICAL_IN_X:
        return np.fft.irfftn(s.astype(np.complex128), s=(nz, ny, nx), axes=(0, 1, 2)) * (nx * ny * nz)
    return np.fft.irfftn(s.astype(np.complex128), s=(nx, ny, nz), axes=(2, 1, 0)) * (nx * ny * nz)


def _engine(fmt, shape, prec, skip=None):
    import gbfft
    nx, ny, nz = shape
    return gbfft.Engine(fmt, nx, ny, nz, skip=skip, prec=gbfft.PREC_DOUBLE if prec == "d" else gbfft.PREC_SINGLE)


# one long axis each: 2^14; 2^4 5^4 = 10000 (mixed radix); 8209 (prime:
# the chirp-z path); 73 * 137 = 10001 (two generic prime stages)
C2C_CASES = [((16384, 3, 2), "s"), ((16384, 2, 2), "d"), ((5, 10000, 3), "s"), ((4, 3, 9000), "d"),
             ((8209, 2, 2), "s"), ((3, 10001, 2), "s"), ((2, 2, 8209), "d")]


@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
@pytest.mark.parametrize("shape,prec", C2C_CASES)
def test_long_axis_c2c_against_oracle(fmt, shape, prec):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + 3 * ny + 7 * nz + fmt)
    a = rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    ct = np.complex128 if prec == "d" else np.complex64
    a = a.astype(ct)
    e = _engine(fmt, shape, prec)
    x = torch.from_numpy(a).cuda()
    for isign in (gbfft.FORWARD, gbfft.BACKWARD):
        ref = O.fft3d_c2c(a.astype(np.complex128), fmt, isign, prec="d")
        pk = pocket_c2c(a, isign)
        y = torch.empty_like(x)
        e.c2c(x, y, isign)
        torch.cuda.synchronize()
        check(y.cpu().numpy(), ref, pk, prec)
        # in place
        z = x.clone()
        e.c2c(z, z, isign)
        torch.cuda.synchronize()
        check(z.cpu().numpy(), ref, pk, prec)
    e.close()


# the long axis as the real axis (x for PHYSICAL_IN_X, z for PHYSICAL_IN_Z),
# even and odd lengths, odd line counts (a line pair with one real line),
# and as a c2c axis of an r2c engine
REAL_CASES = [(O.PHYSICAL_IN_X, (16384, 3, 3), "s"), (O.PHYSICAL_IN_X, (10001, 2, 3), "d"),
              (O.PHYSICAL_IN_X, (8191, 3, 2), "d"), (O.PHYSICAL_IN_Z, (3, 3, 16384), "s"),
              (O.PHYSICAL_IN_Z, (5, 2, 9001), "d"), (O.PHYSICAL_IN_X, (6, 16384, 3), "s"),
              (O.PHYSICAL_IN_Z, (7, 2, 10000), "s")]


@pytest.mark.parametrize("fmt,shape,prec", REAL_CASES)
def test_long_axis_r2c_c2r_against_oracle(fmt, shape, prec):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 5 + ny + nz + fmt)
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
    e.close()


@pytest.mark.parametrize("skip_y", [False, True])
def test_more_planes_than_one_launch(skip_y):
    """A z pass over 70000 rows (ny = 2^4 5^4 7, itself a long axis unless
    skipped) runs as two launches of at most 65535 planes."""
    import gbfft
    nx, ny, nz = 16, 70000, 3
    rng = np.random.default_rng(70000)
    a = (rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))).astype(np.complex64)
    skip = (False, skip_y, False)
    e = _engine(O.PHYSICAL_IN_X, (nx, ny, nz), "s", skip=skip)
    x = torch.from_numpy(a).cuda()
    y = torch.empty_like(x)
    e.c2c(x, y, gbfft.FORWARD)
    torch.cuda.synchronize()
    ref = O.fft3d_c2c(a.astype(np.complex128), O.PHYSICAL_IN_X, O.FORWARD, skip=skip, prec="d")
    assert rel(y.cpu().numpy(), ref) <= TOL["s"]
    e.close()
