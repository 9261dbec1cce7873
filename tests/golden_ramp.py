"""Closed-form forward spectra of the reference's own test field.

The reference's FFT example programs fill the X-pencil with
f(i, j, k) = i/nx * j/ny * k/nz, 1-based (examples/fft_physical_x/fft_r2c_x.f90:65-72;
the c2c programs use f + i f, examples/fft_physical_x/fft_c2c_x.f90:64-73).  Its
unnormalised forward 3D DFT is the product of three exact 1D spectra, stored
rounded once to complex128 in tests/golden/ramp_dft.npz (generated by
tests/golden/make_ramp_golden.py with mpmath).  Arrays here use the numpy view
of a Fortran (nx, ny, nz) pencil: shape (nz, ny, nx).
"""
import os

import numpy as np

_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ramp_dft.npz")
_cache = None

PHYSICAL_IN_X = 1
PHYSICAL_IN_Z = 3


def spectrum_1d(n):
    """g_n(k) = sum_m (m+1)/n exp(-2 pi i m k / n), k = 0..n-1 (complex128)."""
    global _cache
    if _cache is None:
        with np.load(_PATH) as z:
            _cache = {k: z[k] for k in z.files}
    return _cache["n%d" % n]


def lengths():
    spectrum_1d(11)
    return sorted(int(k[1:]) for k in _cache)


def field(nx, ny, nz, dtype=np.float64):
    """The reference's test field in working precision, evaluated left to
    right as the Fortran expression i/nx*j/ny*k/nz is."""
    t = np.dtype(dtype).type
    i = np.arange(1, nx + 1, dtype=dtype)[None, None, :]
    j = np.arange(1, ny + 1, dtype=dtype)[None, :, None]
    k = np.arange(1, nz + 1, dtype=dtype)[:, None, None]
    return ((((i / t(nx)) * j) / t(ny)) * k) / t(nz)


def r2c_spectrum(nx, ny, nz, fmt):
    """Exact r2c spectrum of field(): (nz, ny, nx//2+1) for PHYSICAL_IN_X,
    (nz//2+1, ny, nx) for PHYSICAL_IN_Z."""
    gx, gy, gz = spectrum_1d(nx), spectrum_1d(ny), spectrum_1d(nz)
    if fmt == PHYSICAL_IN_X:
        gx = gx[: nx // 2 + 1]
    else:
        gz = gz[: nz // 2 + 1]
    return gz[:, None, None] * gy[None, :, None] * gx[None, None, :]


def c2c_spectrum(nx, ny, nz):
    """Exact forward c2c spectrum of field() + i field(), shape (nz, ny, nx)."""
    gx, gy, gz = spectrum_1d(nx), spectrum_1d(ny), spectrum_1d(nz)
    return (1 + 1j) * (gz[:, None, None] * gy[None, :, None] * gx[None, None, :])
