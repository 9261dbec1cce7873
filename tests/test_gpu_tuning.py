"""GPU: the tuning knobs change speed, never results.

Every choice the autotuner can make -- strided plan (16 or 32 points per
thread), tile shape per pass, pass fusion -- must give the same spectrum
(within the FP32 tolerance against the FP64 oracle), and a cache line must be
applied to the engines created after it is read."""
import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("ey,ez", [(16, 16), (32, 16), (16, 32), (32, 32)])
def test_strided_plans_give_the_same_transform(fmt, ey, ez):
    import gbfft
    nx, ny, nz = 64, 1024, 512
    x = np.random.default_rng(ey + ez + fmt).standard_normal((nz, ny, nx))
    e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    e.set_plan(1, ey)
    e.set_plan(2, ez)
    assert e.tuning()["points"][1:] == (ey, ez)
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    s = e.empty_spectral()
    e.r2c(xd, s)
    assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= 2e-6
    y = e.empty_physical()
    e.c2r(s, y)
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= 2e-6
    e.close()


@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("nx", [512, 1024])
@pytest.mark.parametrize("ex", [16, 32])
def test_contiguous_plans_give_the_same_transform(fmt, nx, ex):
    # axis 0 (contiguous lines) with 16 points a thread or 32 (one warp a
    # line): r2c / c2r along x for PHYSICAL_IN_X, c2c along x for _Z
    import gbfft
    ny, nz = 34, 20
    x = np.random.default_rng(nx + ex + fmt).standard_normal((nz, ny, nx))
    e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    e.set_plan(0, ex)
    assert e.tuning()["points"][0] == ex
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    s = e.empty_spectral()
    e.r2c(xd, s)
    assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= 2e-6
    y = e.empty_physical()
    e.c2r(s, y)
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= 2e-6
    c = x + 1j * np.random.default_rng(1).standard_normal(x.shape)
    cd = torch.from_numpy(c.astype(np.complex64)).cuda()
    o = torch.empty_like(cd)
    e.c2c(cd, o, -1)
    assert rel(o.cpu().numpy(), O.fft3d_c2c(c.copy(), fmt, -1)) <= 2e-6
    e.close()


@pytest.mark.parametrize("ex", [16, 32])
def test_contiguous_plans_double_precision(ex):
    import gbfft
    nx, ny, nz = 1024, 6, 5
    x = np.random.default_rng(ex).standard_normal((nz, ny, nx))
    e = gbfft.Engine(1, nx, ny, nz, prec=gbfft.PREC_DOUBLE)
    e.set_plan(0, ex)
    xd = torch.from_numpy(x).cuda()
    s = e.empty_spectral()
    e.r2c(xd, s)
    assert rel(s.cpu().numpy(), O.fft3d_r2c(x, 1)) <= 1e-12
    y = e.empty_physical()
    e.c2r(s, y)
    assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= 1e-12
    e.close()


BALANCED = {243: 9, 270: 30, 360: 30, 384: 24, 400: 20}


@pytest.mark.parametrize("prec", ["s", "d"])
@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("n", sorted(BALANCED))
@pytest.mark.parametrize("plan", ["balanced", "two-stage"])
def test_non_power_of_two_plans_give_the_same_transform(prec, fmt, n, plan):
    # the balanced plan (every thread busy in every stage) and the
    # two-stage plan n = R0 R1, on every axis (contiguous and strided)
    import gbfft
    shapes = [(n, 12, 10), (14, n, 6), (10, 8, n)]
    for shape in shapes:
        nx, ny, nz = shape
        x = np.random.default_rng(n + fmt).standard_normal((nz, ny, nx))
        e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE if prec == "s" else gbfft.PREC_DOUBLE)
        axis = shape.index(n)
        pts = BALANCED[n] if plan == "balanced" else 2
        e.set_plan(axis, pts)
        assert e.tuning()["points"][axis] == pts
        xd = torch.from_numpy(x.astype(np.float32 if prec == "s" else np.float64)).cuda()
        s = e.empty_spectral()
        e.r2c(xd, s)
        tol = 2e-6 if prec == "s" else 1e-12
        assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= tol, shape
        y = e.empty_physical()
        e.c2r(s, y)
        assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= tol, shape
        c = x + 1j * np.random.default_rng(2).standard_normal(x.shape)
        cd = torch.from_numpy(c.astype(np.complex64 if prec == "s" else np.complex128)).cuda()
        o = torch.empty_like(cd)
        e.c2c(cd, o, 1)
        assert rel(o.cpu().numpy(), O.fft3d_c2c(c.copy(), fmt, 1)) <= tol, shape
        e.close()


def test_tile_shapes_give_the_same_transform():
    import gbfft
    nx, ny, nz = 256, 64, 48
    x = np.random.default_rng(3).standard_normal((nz, ny, nx))
    ref = O.fft3d_r2c(x, 1)
    e = gbfft.Engine(1, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    s = e.empty_spectral()
    for kind in ("r2c", "c2c_y", "c2c_z"):
        for L in (1, 2, 4, 8, 16):
            try:
                e.set_tile(kind, L)
            except gbfft.GbfftError:
                continue
            e.r2c(xd, s)
            assert rel(s.cpu().numpy(), ref) <= 2e-6, (kind, L)
        e.set_tile(kind, 0)
    e.close()


def test_cache_line_is_applied(tmp_path):
    import gbfft
    path = tmp_path / "cache.txt"
    path.write_text("# test\n4 1 64 1024 512 fuse=0 e_y=16 e_z=32 c2c_y=4 r2c=2 pad=1 flat=0\n")
    gbfft.set_tune_cache(str(path))
    try:
        e = gbfft.Engine(1, 64, 1024, 512, prec=gbfft.PREC_SINGLE)
        t = e.tuning()
        assert t["points"][1:] == (16, 32)
        assert t["tiles"]["c2c_y"] == 4 and t["tiles"]["r2c"] == 2
        assert t["fuse"] is False
        assert e.layout() == (True, False)
        e.close()
        other = gbfft.Engine(1, 64, 1024, 256, prec=gbfft.PREC_SINGLE)
        assert other.tuning()["tiles"]["c2c_y"] == 0  # no line for this shape
        assert other.layout() == (False, True)  # the built-in layout
        other.close()
    finally:
        gbfft.set_tune_cache(None)


# short power-of-two lines: 16, 8 or 4 points a thread (8: at most 256
# points, 4: at most 128), on every axis, both precisions, r2c / c2r / c2c
SHORT = [(n, pe) for n in (16, 32, 64, 128, 256) for pe in (16, 8, 4) if pe == 16 or (pe == 8 and n <= 256)
         or (pe == 4 and n <= 128)]


@pytest.mark.parametrize("prec", ["s", "d"])
@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("n,pe", SHORT)
def test_short_line_plans_give_the_same_transform(prec, fmt, n, pe):
    import gbfft
    for shape in [(n, 12, 10), (14, n, 6), (10, 8, n)]:
        nx, ny, nz = shape
        x = np.random.default_rng(n + pe + fmt).standard_normal((nz, ny, nx))
        e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE if prec == "s" else gbfft.PREC_DOUBLE)
        axis = shape.index(n)
        e.set_plan(axis, pe)
        assert e.tuning()["points"][axis] == pe
        tol = 2e-6 if prec == "s" else 1e-12
        xd = torch.from_numpy(x.astype(np.float32 if prec == "s" else np.float64)).cuda()
        s = e.empty_spectral()
        e.r2c(xd, s)
        assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= tol, shape
        y = e.empty_physical()
        e.c2r(s, y)
        assert rel(y.cpu().numpy() / (nx * ny * nz), x) <= tol, shape
        c = x + 1j * np.random.default_rng(3).standard_normal(x.shape)
        cd = torch.from_numpy(c.astype(np.complex64 if prec == "s" else np.complex128)).cuda()
        o = torch.empty_like(cd)
        e.c2c(cd, o, -1)
        assert rel(o.cpu().numpy(), O.fft3d_c2c(c, fmt, O.FORWARD)) <= tol, shape
        e.close()


def test_small_grid_engines_choose_short_plans_and_batch_keeps_its_own():
    """A 64^3 engine picks 4 points a thread (its grid cannot fill the GPU at
    16); a batch of such engines still runs the persistent kernel, which
    needs the 16-point plan's table, and gives the oracle's spectra."""
    import gbfft
    e = gbfft.Engine(1, 64, 64, 64, prec=gbfft.PREC_SINGLE)
    assert e.tuning()["points"] == (4, 4, 4)
    e.close()
    grids = [(64, 32, 48, 1), (32, 64, 64, 3), (128, 32, 32, 1)]
    engines, xs, specs, reals = [], [], [], []
    b = gbfft.Batch()
    for nx, ny, nz, fmt in grids:
        eng = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
        x = np.random.default_rng(nx + ny).standard_normal((nz, ny, nx))
        xd = torch.from_numpy(x.astype(np.float32)).cuda()
        s = eng.empty_spectral()
        b.add(eng, xd, s)
        engines.append(eng)
        xs.append((x, fmt))
        specs.append(s)
        reals.append(xd)
    assert b.info()["persistent"]
    b.run(1)
    torch.cuda.synchronize()
    b.status()
    for (x, fmt), s in zip(xs, specs):
        assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= 2e-6
    b.close()
    for eng in engines:
        eng.close()
