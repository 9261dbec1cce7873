"""GPU: row layouts of the passes (gbfft_engine_set_layout).

Padded work-area rows (every r2c / c2r pass but the last writes rows that
start on 64-byte boundaries) and flat z passes (the lines of each (x, y)
plane taken in one run) change where the intermediates live and how lines
are grouped into tiles, never the result: r2c / c2r in both formats, FP32
and FP64, odd and even row lengths, skip flags, OVERWRITE engines (no work
area), c2c, and the persistent batch kernel, against the FP64 oracle."""
import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {"s": 2e-6, "d": 1e-12}
LAYOUTS = [(True, True), (False, True), (True, False), (False, False), (2, True), (2, False)]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def prec_of(p):
    import gbfft
    return gbfft.PREC_SINGLE if p == "s" else gbfft.PREC_DOUBLE


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("prec", ["s", "d"])
@pytest.mark.parametrize("shape", [(64, 48, 20), (30, 17, 12), (33, 20, 9), (256, 128, 9), (1024, 8, 16)])
def test_layout_r2c_c2r(layout, fmt, prec, shape):
    import gbfft
    nx, ny, nz = shape
    x = np.random.default_rng(nx + ny + fmt).standard_normal((nz, ny, nx))
    e = gbfft.Engine(fmt, nx, ny, nz, prec=prec_of(prec))
    e.set_layout(*layout)
    assert e.layout() == layout
    xd = torch.from_numpy(x.astype(np.float32 if prec == "s" else np.float64)).cuda()
    x0 = xd.clone()
    s = e.empty_spectral()
    e.r2c(xd, s)
    ref = O.fft3d_r2c(x, fmt)
    assert rel(s.cpu().numpy(), ref) <= TOL[prec]
    keep = s.clone()
    y = e.empty_physical()
    e.c2r(s, y)
    torch.cuda.synchronize()
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= TOL[prec]
    assert torch.equal(s, keep)  # c2r input kept (no OVERWRITE)
    assert torch.equal(xd, x0)
    e.close()


@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("skip", [(False, True, False), (False, False, True), (True, False, False),
                                  (False, True, True), (True, True, False)])
def test_layout_with_skip_flags(fmt, skip):
    import gbfft
    nx, ny, nz = 34, 18, 10
    rng = np.random.default_rng(3)
    x = rng.standard_normal((nz, ny, nx))
    for layout in ((True, True), (False, False)):
        e = gbfft.Engine(fmt, nx, ny, nz, skip=skip, prec=gbfft.PREC_DOUBLE)
        e.set_layout(*layout)
        xd = torch.from_numpy(x).cuda()
        s = e.empty_spectral()
        e.r2c(xd, s)
        ref = O.fft3d_r2c(x, fmt, skip=skip)
        assert rel(s.cpu().numpy(), ref) <= TOL["d"], layout
        y = e.empty_physical()
        e.c2r(s, y)
        ref_b = O.fft3d_c2r(ref.copy(), nx, ny, nz, fmt, skip=skip)
        assert rel(y.cpu().numpy(), ref_b) <= TOL["d"], layout
        e.close()


@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("prec", ["s", "d"])
def test_layout_overwrite_engine(fmt, prec):
    import gbfft
    nx, ny, nz = 66, 40, 24
    x = np.random.default_rng(11).standard_normal((nz, ny, nx))
    e = gbfft.Engine(fmt, nx, ny, nz, inplace=True, prec=prec_of(prec))
    assert e.work_bytes() == 0
    for flat in (True, False):
        e.set_layout(True, flat)
        xd = torch.from_numpy(x.astype(np.float32 if prec == "s" else np.float64)).cuda()
        s = e.empty_spectral()
        e.r2c(xd, s)
        assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= TOL[prec]
        y = e.empty_physical()
        e.c2r(s, y)
        assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= TOL[prec]
    e.close()


def test_layout_values_are_validated():
    import gbfft
    e = gbfft.Engine(1, 32, 16, 8, prec=gbfft.PREC_SINGLE)
    for bad in (-1, 3):
        with pytest.raises(gbfft.GbfftError, match="pad"):
            e.set_layout(bad, True)
    e.set_layout(2, False)
    assert e.layout() == (2, False)
    e.close()


def test_work_area_has_padded_rows():
    import gbfft
    for fmt, nx, ny, nz, prec, pitch in [(1, 1024, 8, 4, 4, 520), (1, 30, 6, 5, 8, 16), (3, 24, 6, 9, 4, 24),
                                         (3, 20, 6, 9, 8, 20)]:
        e = gbfft.Engine(fmt, nx, ny, nz, prec=prec)
        nz_sp = nz if fmt == 1 else nz // 2 + 1
        assert e.work_bytes() == pitch * ny * nz_sp * 2 * prec, (fmt, nx, prec)
        e.close()


@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("prec", ["s", "d"])
@pytest.mark.parametrize("flat", [True, False])
def test_layout_c2c(fmt, prec, flat):
    import gbfft
    nx, ny, nz = 37, 24, 16
    rng = np.random.default_rng(5)
    a = rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    e = gbfft.Engine(fmt, nx, ny, nz, prec=prec_of(prec))
    e.set_layout(True, flat)
    ad = torch.from_numpy(a.astype(np.complex64 if prec == "s" else np.complex128)).cuda()
    for isign in (-1, 1):
        out = torch.empty_like(ad)
        e.c2c(ad, out, isign)
        assert rel(out.cpu().numpy(), O.fft3d_c2c(a.copy(), fmt, isign)) <= TOL[prec]
        io = ad.clone()
        e.c2c(io, io, isign)
        assert torch.equal(io, out)
    e.close()


def test_layout_in_the_batch_kernel():
    import gbfft
    shapes = [(48, 32, 64, 1), (96, 64, 32, 3), (64, 48, 32, 1), (32, 96, 64, 3)]
    engines, reals, specs, xs = [], [], [], []
    rng = np.random.default_rng(9)
    for nx, ny, nz, fmt in shapes:
        e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
        x = rng.uniform(-1, 1, (nz, ny, nx))
        xs.append(x)
        reals.append(torch.from_numpy(x.astype(np.float32)).cuda())
        specs.append(e.empty_spectral())
        engines.append(e)
    b = gbfft.Batch()
    for e, r, s in zip(engines, reals, specs):
        b.add(e, r, s)
    st = torch.cuda.Stream()
    b.run(1, st)
    st.synchronize()
    assert b.info()["persistent"]
    for (nx, ny, nz, fmt), x, s in zip(shapes, xs, specs):
        assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= TOL["s"]
    b.run(2, st)
    st.synchronize()
    for (nx, ny, nz, fmt), x, r in zip(shapes, xs, reals):
        assert rel(r.cpu().numpy() / (nx * ny * nz), x) <= TOL["s"]
    b.close()
    for e in engines:
        e.close()
