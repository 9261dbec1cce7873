"""CPU: the oracle's forward spectra against the exact spectra of the
reference's own test field (tests/golden_ramp.py).

This pins the oracle's forward transform -- not only its round trip, which
any invertible transform passes -- to a reference-derived closed form:
rel-L2 <= 1e-13 in double; <= 5e-6 in single, where the restated Glassman
stages build their twiddles by the reference's single-precision recurrence
OMEGA = DELTA * OMEGA (src/glassman.f90:84-96; 1.9e-6 on 17 x 13 x 11).
"""
import numpy as np
import pytest

import golden_ramp as G
from oracle import oracle as O


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def test_fixture_matches_the_closed_form_in_float64():
    for n in G.lengths():
        g = G.spectrum_1d(n)
        k = np.arange(1, n)
        # cot(pi k / n) = -cot(pi (n - k) / n): evaluate on the short side
        kk = np.minimum(k, n - k)
        cot = np.cos(np.pi * kk / n) / np.sin(np.pi * kk / n) * np.where(k <= n - k, 1.0, -1.0)
        assert g[0] == (n + 1) / 2
        assert np.allclose(g[1:].real, -0.5, rtol=0, atol=1e-15)
        assert np.max(np.abs(g[1:].imag - cot / 2) / np.abs(g).max()) < 1e-14


def test_fixture_matches_a_direct_dft():
    for n in (11, 13, 17, 64, 243):
        f = np.arange(1, n + 1) / n
        assert rel(np.fft.fft(f), G.spectrum_1d(n)) < 1e-14


@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
@pytest.mark.parametrize("shape", [(17, 13, 11), (64, 17, 13), (11, 64, 17)])
def test_oracle_r2c_matches_the_exact_spectrum(fmt, shape):
    nx, ny, nz = shape
    exact = G.r2c_spectrum(nx, ny, nz, fmt)
    got = O.fft3d_r2c(G.field(nx, ny, nz), fmt, prec="d")
    assert rel(got, exact) <= 1e-13
    got_s = O.fft3d_r2c(G.field(nx, ny, nz, np.float32), fmt, prec="s")
    assert rel(got_s, exact) <= 5e-6


@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
def test_oracle_c2c_matches_the_exact_spectrum(fmt):
    nx, ny, nz = 17, 13, 11
    f = G.field(nx, ny, nz)
    got = O.fft3d_c2c(np.ascontiguousarray(f + 1j * f), fmt, O.FORWARD, prec="d")
    assert rel(got, G.c2c_spectrum(nx, ny, nz)) <= 1e-13


def test_oracle_backward_of_the_exact_spectrum_is_the_field():
    """c2r of the exact spectrum, divided by nx ny nz, gives the field back
    (the reference's own round-trip check, from the other side)."""
    nx, ny, nz = 17, 13, 11
    for fmt in (O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z):
        spec = np.ascontiguousarray(G.r2c_spectrum(nx, ny, nz, fmt))
        back = O.fft3d_c2r(spec, nx, ny, nz, fmt, prec="d") / (nx * ny * nz)
        assert np.abs(back - G.field(nx, ny, nz)).max() <= 1e-13
