"""CPU: the oracle (restated generic backend) pinned against pocketfft and
against the reference's own known-answer tests."""
import numpy as np
import pytest

from oracle import oracle as O
import refcases as RC
from backends import OracleBackend

SIZES_1D = [1, 2, 3, 4, 5, 6, 7, 8, 9, 11, 12, 13, 15, 16, 17, 18, 25, 27, 29, 32, 48, 49, 64,
            96, 100, 121, 128, 243, 256, 360, 400, 1024]


@pytest.mark.parametrize("n", SIZES_1D)
def test_spcfft_double_matches_pocketfft(n):
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    f = O.fft1d(x, -1)
    b = O.fft1d(x, 1)
    assert np.linalg.norm(f - np.fft.fft(x)) <= 1e-13 * np.linalg.norm(np.fft.fft(x))
    assert np.linalg.norm(b - n * np.fft.ifft(x)) <= 1e-13 * np.linalg.norm(np.fft.fft(x))


def test_spcfft_single_build_accuracy():
    # The reference's single generic build (complex(real32) twiddle
    # recurrence) is far less accurate than FP32 rounding: ~1e-5 at n=400.
    rng = np.random.default_rng(5)
    x = (rng.uniform(-1, 1, 400) + 1j * rng.uniform(-1, 1, 400)).astype(np.complex64)
    f = O.fft1d(x, -1, prec="s")
    ref = np.fft.fft(x.astype(np.complex128))
    rel = np.linalg.norm(f - ref) / np.linalg.norm(ref)
    assert 1e-7 < rel < 1e-4


@pytest.mark.parametrize("shape", [(17, 13, 11), (16, 12, 10), (1, 5, 4), (6, 1, 1)])
@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
def test_fft3d_against_pocketfft(shape, fmt):
    nx, ny, nz = shape
    rng = np.random.default_rng(sum(shape) + fmt)
    x = rng.uniform(-1, 1, (nz, ny, nx))
    s = O.fft3d_r2c(x, fmt)
    if fmt == O.PHYSICAL_IN_X:
        ref = np.fft.rfftn(x, axes=(0, 1, 2))
    else:
        ref = np.fft.rfftn(x.transpose(2, 1, 0), axes=(0, 1, 2)).transpose(2, 1, 0)
    assert s.shape == O.spectral_shape(nx, ny, nz, fmt)
    assert np.allclose(s, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    y = O.fft3d_c2r(s.copy(), nx, ny, nz, fmt)
    assert np.allclose(y / (nx * ny * nz), x, atol=1e-13)
    c = x + 1j * rng.uniform(-1, 1, x.shape)
    f = O.fft3d_c2c(c.copy(), fmt, O.FORWARD)
    assert np.allclose(f, np.fft.fftn(c), atol=1e-12 * np.abs(f).max())


def test_c2r_ignores_imag_of_dc_and_nyquist():
    # src/fft_generic.f90:318-330 keeps only the real part after the
    # Hermitian fill, so Im of bin 0 and bin n/2 has no effect.
    nx, ny, nz = 8, 3, 2
    rng = np.random.default_rng(3)
    s = rng.standard_normal((nz, ny, nx // 2 + 1)) + 1j * rng.standard_normal((nz, ny, nx // 2 + 1))
    a = O.fft3d_c2r(s.copy(), nx, ny, nz, O.PHYSICAL_IN_X, skip=(False, True, True))
    s2 = s.copy()
    s2[..., 0] = s2[..., 0].real
    s2[..., nx // 2] = s2[..., nx // 2].real
    b = O.fft3d_c2r(s2, nx, ny, nz, O.PHYSICAL_IN_X, skip=(False, True, True))
    assert np.allclose(a, b, atol=1e-14)


def test_inplace_destroys_input_and_copy_preserves_it():
    rng = np.random.default_rng(9)
    c = rng.standard_normal((5, 4, 3)) + 1j * rng.standard_normal((5, 4, 3))
    keep = c.copy()
    O.fft3d_c2c(c, O.PHYSICAL_IN_X, O.FORWARD, inplace=False)
    assert np.array_equal(c, keep)
    O.fft3d_c2c(c, O.PHYSICAL_IN_X, O.FORWARD, inplace=True)
    assert not np.array_equal(c, keep)


# ---- the reference's example programs, run on the oracle ----------------
@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("fmt", [RC.PHYSICAL_IN_X, RC.PHYSICAL_IN_Z])
@pytest.mark.parametrize("skip", [None, (True, False, True)])
def test_reference_fft_c2c(prec, fmt, skip):
    err, thr = RC.fft_c2c(OracleBackend(prec), 17, 13, 11, fmt, prec, skip=skip)
    assert err <= thr, (err, thr)


@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("fmt", [RC.PHYSICAL_IN_X, RC.PHYSICAL_IN_Z])
@pytest.mark.parametrize("skip", [None, (True, False, True)])
def test_reference_fft_r2c(prec, fmt, skip):
    err, thr = RC.fft_r2c(OracleBackend(prec), 17, 13, 11, fmt, prec, skip=skip)
    assert err <= thr, (err, thr)


@pytest.mark.parametrize("prec", ["d", "s"])
def test_reference_fft_grid_x(prec):
    # fft_grid_x: the FFT grid differs from the decomposition grid
    err, thr = RC.fft_r2c(OracleBackend(prec), 17, 13, 11, RC.PHYSICAL_IN_X, prec)
    assert err <= thr


@pytest.mark.parametrize("prec", ["d", "s"])
def test_reference_multiple_grids(prec):
    b = OracleBackend(prec)
    nx, ny, nz = 17, 13, 11
    for (fmt, sx, sy, sz) in [(RC.PHYSICAL_IN_X, nx, ny, nz), (RC.PHYSICAL_IN_Z, nx, ny, nz),
                              (RC.PHYSICAL_IN_X, nx, ny + 2, nz + 16),
                              (RC.PHYSICAL_IN_Z, nx + 16, ny + 2, nz)]:
        e, t = RC.multigrid_c2c(b, sx, sy, sz, fmt, prec)
        assert e <= t, ("c2c", fmt, sx, sy, sz, e, t)
        e, t = RC.multigrid_r2c(b, sx, sy, sz, fmt, prec)
        assert e <= t, ("r2c", fmt, sx, sy, sz, e, t)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex64, np.complex128])
def test_reference_test2d_chain(dtype):
    assert all(RC.test2d_chain(OracleBackend("d"), 17, 13, 11, dtype))
