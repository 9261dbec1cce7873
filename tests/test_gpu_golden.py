"""GPU: forward spectra against the exact spectra of the reference's own test
field, f(i, j, k) = i/nx * j/ny * k/nz (tests/golden_ramp.py), through the
C ABI.

This pins the GPU path's forward transform to a reference-derived closed
form at every size the fixture covers, including the 1024 x 1024 x 512 FP32
grid in both formats.  Tolerances (relative L2 over the whole spectrum):
<= 1e-12 in double, <= 2e-6 in single, as in the oracle parity tests.
"""
import numpy as np
import pytest

import golden_ramp as G

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {8: 1e-12, 4: 2e-6}


def _field(nx, ny, nz, prec):
    return torch.from_numpy(G.field(nx, ny, nz, np.float64 if prec == 8 else np.float32)).cuda()


def _exact_dev(nx, ny, nz, fmt):
    """Exact spectrum built on the device in complex128 (outer product of
    the three 1D spectra), so that large grids need no host copy."""
    gx, gy, gz = (torch.from_numpy(G.spectrum_1d(n)).cuda() for n in (nx, ny, nz))
    if fmt == G.PHYSICAL_IN_X:
        gx = gx[: nx // 2 + 1]
    elif fmt == G.PHYSICAL_IN_Z:
        gz = gz[: nz // 2 + 1]
    return gz[:, None, None] * gy[None, :, None] * gx[None, None, :]


def _rel(got, exact):
    d = got.to(torch.complex128) - exact
    return float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(exact))


SMALL = [(17, 13, 11), (64, 17, 13), (11, 64, 17), (13, 11, 64)]
MEDIUM = [(384, 400, 243), (360, 270, 210), (256, 256, 256)]


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("fmt", [G.PHYSICAL_IN_X, G.PHYSICAL_IN_Z])
@pytest.mark.parametrize("shape", SMALL + MEDIUM)
def test_r2c_matches_the_exact_spectrum(prec, fmt, shape):
    import gbfft
    nx, ny, nz = shape
    e = gbfft.Engine(fmt, nx, ny, nz, prec=prec)
    x = _field(nx, ny, nz, prec)
    spec = e.empty_spectral()
    e.r2c(x, spec)
    torch.cuda.synchronize()
    exact = _exact_dev(nx, ny, nz, fmt)
    assert _rel(spec, exact) <= TOL[prec]
    # backward from the exact spectrum (rounded to the engine's type): the
    # field again after dividing by nx ny nz
    back = e.empty_physical()
    e.c2r(exact.to(spec.dtype).contiguous(), back)
    torch.cuda.synchronize()
    err = float((back.double() / (nx * ny * nz) - x.double()).abs().max())
    assert err <= (1e-13 if prec == 8 else 2e-6)
    e.close()


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("fmt", [G.PHYSICAL_IN_X, G.PHYSICAL_IN_Z])
@pytest.mark.parametrize("shape", SMALL + [(256, 256, 256)])
def test_c2c_matches_the_exact_spectrum(prec, fmt, shape):
    import gbfft
    nx, ny, nz = shape
    e = gbfft.Engine(fmt, nx, ny, nz, prec=prec)
    f = _field(nx, ny, nz, prec)
    x = torch.complex(f, f)
    out = torch.empty_like(x)
    e.c2c(x, out, gbfft.FORWARD)
    torch.cuda.synchronize()
    exact = (1 + 1j) * _exact_dev(nx, ny, nz, None)
    assert _rel(out, exact) <= TOL[prec]
    e.close()


@pytest.mark.parametrize("fmt", [G.PHYSICAL_IN_X, G.PHYSICAL_IN_Z])
def test_large_fp32_grid_matches_the_exact_spectrum(fmt):
    """The benchmark's 1024 x 1024 x 512 FP32 grid, r2c then c2r."""
    import gbfft
    nx, ny, nz = 1024, 1024, 512
    e = gbfft.Engine(fmt, nx, ny, nz, prec=4)
    x = _field(nx, ny, nz, 4)
    spec = e.empty_spectral()
    e.r2c(x, spec)
    torch.cuda.synchronize()
    exact = _exact_dev(nx, ny, nz, fmt)
    assert _rel(spec, exact) <= TOL[4]
    del exact
    back = e.empty_physical()
    e.c2r(spec, back)
    torch.cuda.synchronize()
    d = back.double() / (nx * ny * nz) - x.double()
    assert float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(x.double())) <= 2e-6
    e.close()


@pytest.mark.parametrize("form", ["split", "split_tc"])
def test_large_fp32_grid_split_forms_within_1e6(form):
    """The split-precision forms at the benchmark's 1024 x 1024 x 512 FP32
    grid (PHYSICAL_IN_X): the forward spectrum within rel-L2 1e-6 of the exact
    one (the accuracy bar a split-precision form must meet), and the round trip."""
    import gbfft
    nx, ny, nz = 1024, 1024, 512
    f = gbfft.FORM_SPLIT if form == "split" else gbfft.FORM_SPLIT_TC
    before = gbfft.tc_pass_count()
    e = gbfft.Engine(G.PHYSICAL_IN_X, nx, ny, nz, prec=4, form=f)
    x = _field(nx, ny, nz, 4)
    spec = e.empty_spectral()
    e.r2c(x, spec)
    torch.cuda.synchronize()
    exact = _exact_dev(nx, ny, nz, G.PHYSICAL_IN_X)
    assert _rel(spec, exact) <= 1e-6
    del exact
    back = e.empty_physical()
    e.c2r(spec, back)
    torch.cuda.synchronize()
    d = back.double() / (nx * ny * nz) - x.double()
    assert float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(x.double())) <= 2e-6
    if form == "split_tc":
        assert gbfft.tc_pass_count() >= before + 2  # both y passes ran on tcgen05
    e.status()
    e.close()
