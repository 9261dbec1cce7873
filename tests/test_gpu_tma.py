"""GPU: 1024-point y passes staged by bulk tensor copies (gbfft_engine_set_tma)
against the oracle, and against the one-shot kernel they stand in for (same
plan, same twiddle table, same butterflies; the two kernels agree to
rounding -- rel-L2 <= 1e-6 -- since the compiler may fuse the complex
multiply-adds into FMAs differently in each).

Covered: both plans of 1024 points (16 and 32 points a thread); ragged last
tiles (line counts that are not a multiple of the tile's lines, and fewer
lines than one tile); one plane; c2c in both directions and formats; r2c /
c2r in the padded work area (pad=1, 2) and in Z-format rows; the
1024 x 1024 x 512 FP32 grid with the padded layout against the exact spectrum
of the reference's test field.
Tolerance against the FP64 oracle: relative L2 <= 2e-6 (single precision).
"""
import numpy as np
import pytest

import golden_ramp as G
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 2e-6


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def _engine(fmt, shape, tma, pad=None):
    import gbfft
    nx, ny, nz = shape
    e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    e.set_tma(tma)
    if pad is not None:
        e.set_layout(pad=pad, flat=True)
    return e


# every shape has at least one eligible strided pass: y passes over rows of
# an even number of values, z passes over rows of a multiple of 16 values
# (shape, points a thread of the y plan): rows of an even number of values
C2C_SHAPES = [((64, 1024, 6), 32), ((64, 1024, 6), 16), ((30, 1024, 3), 16), ((6, 1024, 2), 32),
              ((2, 1024, 4), 16), ((10, 1024, 1), 16), ((1024, 1024, 2), 16)]


@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
@pytest.mark.parametrize("shape,ey", C2C_SHAPES)
def test_c2c_tma_against_oracle_and_one_shot(fmt, shape, ey):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 7 + ny * 3 + nz + fmt)
    a = (rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))).astype(np.complex64)
    x = torch.from_numpy(a).cuda()
    for isign in (gbfft.FORWARD, gbfft.BACKWARD):
        ref = O.fft3d_c2c(a.astype(np.complex128), fmt, isign, prec="d")
        outs = []
        for tma in (True, False):
            e = _engine(fmt, shape, tma)
            e.set_plan(1, ey)
            y = torch.empty_like(x)
            c0 = gbfft.tma_pass_count()
            e.c2c(x, y, isign)
            torch.cuda.synchronize()
            e.status()
            ran = gbfft.tma_pass_count() - c0
            assert ran == (1 if tma else 0)  # the y pass
            outs.append(y.cpu().numpy())
            e.close()
        assert rel(outs[0], ref) <= TOL
        assert rel(outs[0], outs[1]) <= 1e-6


# (format, shape, pad, TMA passes of one r2c + c2r): X-format y passes run
# it in the padded work area (pad=1 both directions, pad=2 c2r only),
# Z-format y passes over rows of an even number of values
REAL_CASES = [(O.PHYSICAL_IN_X, (1024, 1024, 6), 1, 2), (O.PHYSICAL_IN_X, (62, 1024, 5), 1, 2),
              (O.PHYSICAL_IN_X, (1022, 1024, 2), 1, 2), (O.PHYSICAL_IN_X, (512, 1024, 3), 2, 1),
              (O.PHYSICAL_IN_X, (512, 1024, 3), 0, 0), (O.PHYSICAL_IN_Z, (64, 1024, 10), 0, 2),
              (O.PHYSICAL_IN_Z, (34, 1024, 7), 0, 2), (O.PHYSICAL_IN_Z, (256, 1024, 9), 1, 2)]


@pytest.mark.parametrize("fmt,shape,pad,expect", REAL_CASES)
def test_r2c_c2r_tma_against_oracle_and_one_shot(fmt, shape, pad, expect):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + ny + nz + fmt + pad)
    x = rng.uniform(-1, 1, (nz, ny, nx)).astype(np.float32)
    ref = O.fft3d_r2c(x.astype(np.float64), fmt, prec="d")
    s = (ref + 0.25 * (rng.standard_normal(ref.shape) + 1j * rng.standard_normal(ref.shape))).astype(np.complex64)
    refb = O.fft3d_c2r(s.astype(np.complex128), nx, ny, nz, fmt, prec="d")
    got = {}
    for tma in (True, False):
        e = _engine(fmt, shape, tma, pad)
        e.set_plan(1, 16)
        e.set_layout(pad=pad, flat=True)
        xd = torch.from_numpy(x).cuda()
        spec = e.empty_spectral()
        c0 = gbfft.tma_pass_count()
        e.r2c(xd, spec)
        sd = torch.from_numpy(s).cuda()
        back = e.empty_physical()
        e.c2r(sd, back)
        torch.cuda.synchronize()
        e.status()
        ran = gbfft.tma_pass_count() - c0
        assert ran == (expect if tma else 0)
        assert torch.equal(sd.cpu(), torch.from_numpy(s))  # c2r keeps its input
        got[tma] = (spec.cpu().numpy(), back.cpu().numpy())
        e.close()
    assert rel(got[True][0], ref) <= TOL
    assert rel(got[True][1], refb) <= TOL
    assert rel(got[True][0], got[False][0]) <= 1e-6
    assert rel(got[True][1], got[False][1]) <= 1e-6


def test_large_grid_padded_layout_against_exact_spectrum():
    """1024 x 1024 x 512 FP32, PHYSICAL_IN_X, padded work rows: both y passes
    run the bulk-tensor-copy kernel; r2c against the exact spectrum of the
    reference's test field, c2r back to the field."""
    import gbfft
    nx, ny, nz = 1024, 1024, 512
    e = _engine(O.PHYSICAL_IN_X, (nx, ny, nz), True, pad=1)
    e.set_plan(1, 16)
    e.set_layout(pad=1, flat=True)
    x = torch.from_numpy(G.field(nx, ny, nz, np.float32)).cuda()
    spec = e.empty_spectral()
    c0 = gbfft.tma_pass_count()
    e.r2c(x, spec)
    torch.cuda.synchronize()
    assert gbfft.tma_pass_count() - c0 == 1
    gx, gy, gz = (torch.from_numpy(G.spectrum_1d(n)).cuda() for n in (nx, ny, nz))
    exact = gz[:, None, None] * gy[None, :, None] * gx[None, None, : nx // 2 + 1]
    d = spec.to(torch.complex128) - exact
    assert float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(exact)) <= TOL
    del d, exact
    back = e.empty_physical()
    e.c2r(spec, back)
    torch.cuda.synchronize()
    e.status()
    assert gbfft.tma_pass_count() - c0 == 2
    r = back.double() / (nx * ny * nz) - x.double()
    assert float(torch.linalg.vector_norm(r) / torch.linalg.vector_norm(x.double())) <= TOL
    e.close()
