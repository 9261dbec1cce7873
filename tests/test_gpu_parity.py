"""GPU parity: the CUDA path, called through the C ABI, against the oracle.

Tolerances (relative L2 over the whole array, against the FP64 oracle):
  double engines  <= 1e-12  (the oracle itself agrees with pocketfft to ~3e-14)
  single engines  <= 2e-6   (plain FP32 with exactly rounded twiddles)
Transposes are compared bit for bit.
"""
import numpy as np
import pytest

import refcases as RC
from backends import GpuBackend
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {"d": 1e-12, "s": 2e-6}


def rel(a, b):
    b = np.asarray(b)
    den = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a) - b) / (den if den > 0 else 1.0)


@pytest.fixture(scope="module")
def gpu():
    import gbfft
    gbfft.lib()
    b = {"d": GpuBackend("d"), "s": GpuBackend("s")}
    yield b
    for v in b.values():
        v.close()


SHAPES = [(17, 13, 11), (16, 12, 10), (64, 64, 64), (24, 18, 10), (1, 5, 4), (6, 1, 1), (9, 1, 7),
          (48, 40, 27), (36, 27, 21), (33, 29, 27), (128, 8, 3), (7, 49, 25), (97, 11, 2),
          (256, 3, 2), (5, 1024, 2), (3, 2, 512)]


@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
@pytest.mark.parametrize("shape", SHAPES)
def test_r2c_c2r_against_oracle(gpu, prec, fmt, shape):
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 1000 + ny * 10 + nz + fmt)
    x = rng.uniform(-1, 1, (nz, ny, nx))
    ref = O.fft3d_r2c(x, fmt)
    rt = np.float64 if prec == "d" else np.float32
    got = gpu[prec].r2c(x.astype(rt), fmt, None)
    assert got.shape == ref.shape
    assert rel(got, ref) <= TOL[prec]
    # c2r of an arbitrary (non-Hermitian) spectrum: the reference's rule
    # decides what Im(DC)/Im(Nyquist) and the redundant half mean
    s = ref + 0.3 * (rng.standard_normal(ref.shape) + 1j * rng.standard_normal(ref.shape))
    ref_b = O.fft3d_c2r(s.copy(), nx, ny, nz, fmt)
    ct = np.complex128 if prec == "d" else np.complex64
    got_b = gpu[prec].c2r(s.astype(ct), nx, ny, nz, fmt, False, None)
    assert rel(got_b, ref_b) <= TOL[prec]


@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
@pytest.mark.parametrize("isign", [O.FORWARD, O.BACKWARD])
@pytest.mark.parametrize("shape", [(17, 13, 11), (32, 16, 8), (30, 14, 45), (1, 1, 1), (121, 3, 5)])
def test_c2c_against_oracle(gpu, prec, fmt, isign, shape):
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + 7 * ny + 13 * nz)
    a = rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    ref = O.fft3d_c2c(a.copy(), fmt, isign)
    ct = np.complex128 if prec == "d" else np.complex64
    got = gpu[prec].c2c(a.astype(ct), fmt, isign, False, None)
    assert rel(got, ref) <= TOL[prec]


# Plane shapes with a fused x/y kernel (FP32, square power-of-two planes),
# fused (256- and 512-thread tiles) and unfused, against the FP64 oracle.
@pytest.mark.parametrize("fuse", [256, 512, False])
@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
@pytest.mark.parametrize("shape", [(256, 256, 6), (512, 512, 3), (1024, 1024, 2), (256, 256, 1)])
def test_fused_planes_against_oracle(fuse, fmt, shape):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + nz + fmt)
    x = rng.standard_normal((nz, ny, nx))
    e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    e.set_fusion(bool(fuse))
    if fuse:
        ty = ny // (32 if ny in (512, 1024) else 16)  # threads a y line
        e.set_tile("xy_fused", fuse // ty)
    xd = torch.from_numpy(x.astype(np.float32)).cuda()
    s = e.empty_spectral()
    e.r2c(xd, s)
    ref = O.fft3d_r2c(x, fmt)
    assert rel(s.cpu().numpy(), ref) <= TOL["s"]
    sp = ref + 0.1 * (rng.standard_normal(ref.shape) + 1j * rng.standard_normal(ref.shape))
    y = e.empty_physical()
    e.c2r(torch.from_numpy(sp.astype(np.complex64)).cuda(), y)
    assert rel(y.cpu().numpy(), O.fft3d_c2r(sp.copy(), nx, ny, nz, fmt)) <= TOL["s"]
    c = x + 1j * rng.standard_normal(x.shape)
    cd = torch.from_numpy(c.astype(np.complex64)).cuda()
    for isign in (O.FORWARD, O.BACKWARD):
        o = torch.empty_like(cd)
        e.c2c(cd, o, isign)
        assert rel(o.cpu().numpy(), O.fft3d_c2c(c.copy(), fmt, isign)) <= TOL["s"]
    e.status()  # no bounded wait of a fused pass gave up
    e.close()


SKIPS = [(True, False, True), (False, True, False), (True, True, True), (False, False, True),
         (True, False, False)]


@pytest.mark.parametrize("skip", SKIPS)
@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
def test_skip_flags_against_oracle(gpu, skip, fmt):
    nx, ny, nz = 12, 10, 9
    rng = np.random.default_rng(4)
    a = rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    for isign in (O.FORWARD, O.BACKWARD):
        ref = O.fft3d_c2c(a.copy(), fmt, isign, skip=skip)
        assert rel(gpu["d"].c2c(a, fmt, isign, False, skip), ref) <= TOL["d"]
    x = a.real.copy()
    ref = O.fft3d_r2c(x, fmt, skip=skip)
    assert rel(gpu["d"].r2c(x, fmt, skip), ref) <= TOL["d"]
    ref_b = O.fft3d_c2r(ref.copy(), nx, ny, nz, fmt, skip=skip)
    assert rel(gpu["d"].c2r(ref, nx, ny, nz, fmt, False, skip), ref_b) <= TOL["d"]


@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
def test_inplace_semantics(fmt):
    import gbfft
    nx, ny, nz = 20, 12, 6
    rng = np.random.default_rng(8)
    x = rng.uniform(-1, 1, (nz, ny, nx))
    for inplace in (False, True):
        e = gbfft.Engine(fmt, nx, ny, nz, inplace=inplace, prec=gbfft.PREC_DOUBLE)
        assert (e.work_bytes() == 0) == inplace
        xd = torch.from_numpy(x).cuda()
        s = e.empty_spectral()
        e.r2c(xd, s)
        keep = s.clone()
        y = e.empty_physical()
        e.c2r(s, y)
        torch.cuda.synchronize()
        assert np.allclose(y.cpu().numpy() / (nx * ny * nz), x, atol=1e-13)
        # c2r input is preserved unless OVERWRITE
        assert torch.equal(s, keep) != inplace
        # c2c never modifies its input; in == out is allowed
        c = torch.from_numpy(x + 1j * x).cuda()
        c0 = c.clone()
        o = torch.empty_like(c)
        e.c2c(c, o, gbfft.FORWARD)
        e.c2c(c, c, gbfft.FORWARD)
        torch.cuda.synchronize()
        assert torch.equal(o, c)
        assert not torch.equal(c, c0)
        e.close()


def test_r2c_rejects_aliasing():
    import gbfft
    e = gbfft.Engine(gbfft.PHYSICAL_IN_X, 8, 8, 8, prec=gbfft.PREC_DOUBLE)
    buf = torch.zeros(8 * 8 * 8 * 2, dtype=torch.float64, device="cuda")
    with pytest.raises(gbfft.GbfftError, match="In-place r2c"):
        e.r2c(buf, buf)
    e.close()


# ---- the reference's example programs on the GPU ----------------------
@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("fmt", [RC.PHYSICAL_IN_X, RC.PHYSICAL_IN_Z])
@pytest.mark.parametrize("skip", [None, (True, False, True)])
def test_reference_fft_c2c_on_gpu(gpu, prec, fmt, skip):
    err, thr = RC.fft_c2c(gpu[prec], 17, 13, 11, fmt, prec, skip=skip)
    assert err <= thr, (err, thr)


@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("fmt", [RC.PHYSICAL_IN_X, RC.PHYSICAL_IN_Z])
@pytest.mark.parametrize("skip", [None, (True, False, True)])
def test_reference_fft_r2c_on_gpu(gpu, prec, fmt, skip):
    err, thr = RC.fft_r2c(gpu[prec], 17, 13, 11, fmt, prec, skip=skip)
    assert err <= thr, (err, thr)


@pytest.mark.parametrize("prec", ["d", "s"])
def test_reference_multiple_grids_on_gpu(gpu, prec):
    nx, ny, nz = 17, 13, 11
    for (fmt, sx, sy, sz) in [(RC.PHYSICAL_IN_X, nx, ny, nz), (RC.PHYSICAL_IN_Z, nx, ny, nz),
                              (RC.PHYSICAL_IN_X, nx, ny + 2, nz + 16),
                              (RC.PHYSICAL_IN_Z, nx + 16, ny + 2, nz)]:
        e, t = RC.multigrid_c2c(gpu[prec], sx, sy, sz, fmt, prec)
        assert e <= t, ("c2c", fmt, e, t)
        e, t = RC.multigrid_r2c(gpu[prec], sx, sy, sz, fmt, prec)
        assert e <= t, ("r2c", fmt, e, t)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex64, np.complex128])
def test_reference_test2d_chain_on_gpu(gpu, dtype):
    assert all(RC.test2d_chain(gpu["d"], 17, 13, 11, dtype))


@pytest.mark.parametrize("dtype", [torch.float64, torch.complex128])
def test_transposes_bit_exact_256(dtype):
    # 256^3 transpose chain x->y->z->y->x, seeded uniform [-1, 1), memcmp
    import gbfft
    n = 256
    g = torch.Generator(device="cuda").manual_seed(2)
    if dtype.is_complex:
        u = torch.complex(torch.rand((n, n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1,
                          torch.rand((n, n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1)
    else:
        u = torch.rand((n, n, n), generator=g, device="cuda", dtype=dtype) * 2 - 1
    isc = dtype.is_complex
    a, b = torch.empty_like(u), torch.empty_like(u)
    gbfft.transpose(gbfft.X_TO_Y, u, a, n, n, n, isc, gbfft.PREC_DOUBLE)
    gbfft.transpose(gbfft.Y_TO_Z, a, b, n, n, n, isc, gbfft.PREC_DOUBLE)
    gbfft.transpose(gbfft.Z_TO_Y, b, a, n, n, n, isc, gbfft.PREC_DOUBLE)
    gbfft.transpose(gbfft.Y_TO_X, a, b, n, n, n, isc, gbfft.PREC_DOUBLE)
    torch.cuda.synchronize()
    assert torch.equal(u.view(torch.uint8) if not isc else torch.view_as_real(u),
                       b.view(torch.uint8) if not isc else torch.view_as_real(b))


@pytest.mark.parametrize("nbytes,off", [(1, 0), (17, 3), (4096 + 5, 8), (1 << 20, 1)])
def test_transpose_copy_odd_sizes_and_offsets(nbytes, off):
    import gbfft
    src = torch.randint(0, 255, (nbytes + 16,), dtype=torch.uint8, device="cuda")
    dst = torch.zeros_like(src)
    # single precision real elements: use byte counts that are whole floats
    n = (nbytes + 3) // 4
    s = src[off:off + 4 * n]
    d = dst[off:off + 4 * n]
    if s.numel() < 4 * n:
        pytest.skip("buffer too small")
    gbfft.check(gbfft.lib().gbfft_transpose(0, 0, 4, s.data_ptr(), d.data_ptr(), n, 1, 1, None))
    torch.cuda.synchronize()
    assert torch.equal(s, d)


# ---- the module mirror (decomp_2d_fft.h) -------------------------------
def test_module_api_single_and_multiple_grids():
    import gbfft as G
    nx, ny, nz = 17, 13, 11
    G.decomp_2d_init(nx + 1, ny + 1, nz + 1, 0, 0, G.PREC_DOUBLE)
    try:
        G.decomp_2d_fft_set_ngrid(3)
        G.decomp_2d_fft_init(G.PHYSICAL_IN_X, nx, ny, nz, 1)
        G.decomp_2d_fft_init(G.PHYSICAL_IN_Z, nx, ny, nz, 2)
        G.decomp_2d_fft_init(G.PHYSICAL_IN_X, nx, ny + 2, nz + 16, 3)
        with pytest.raises(G.GbfftError, match="only be initialised once"):
            G.decomp_2d_fft_init(G.PHYSICAL_IN_X, nx, ny, nz, 1)
        for ig, (fmt, sx, sy, sz) in enumerate([(1, nx, ny, nz), (3, nx, ny, nz), (1, nx, ny + 2, nz + 16)], 1):
            G.decomp_2d_fft_use_grid(ig)
            assert G.decomp_2d_fft_get_ph_size() == (sx, sy, sz)
            st, en, sz_ = G.decomp_2d_fft_get_size()
            assert st == (1, 1, 1)
            assert sz_ == ((sx // 2 + 1, sy, sz) if fmt == 1 else (sx, sy, sz // 2 + 1))
            x = np.random.default_rng(ig).uniform(-1, 1, (sz, sy, sx))
            xd = torch.from_numpy(x).cuda()
            s = torch.empty(G.spectral_shape(sx, sy, sz, fmt), dtype=torch.complex128, device="cuda")
            G.decomp_2d_fft_3d_r2c(xd, s)
            y = torch.empty_like(xd)
            G.decomp_2d_fft_3d_c2r(s, y)
            torch.cuda.synchronize()
            assert rel(s.cpu().numpy(), O.fft3d_r2c(x, fmt)) <= 1e-12
            assert np.allclose(y.cpu().numpy() / (sx * sy * sz), x, atol=1e-13)
        assert "gb300" in G.decomp_2d_fft_log()
        G.decomp_2d_fft_finalize()
        with pytest.raises(G.GbfftError):
            G.decomp_2d_fft_3d_r2c(xd, s)
        # one grid on the decomp_main sizes (fft_init_arg)
        G.decomp_2d_fft_init(G.PHYSICAL_IN_Z)
        assert G.decomp_2d_fft_get_ph_size() == (nx + 1, ny + 1, nz + 1)
        u = torch.rand((nz + 1, ny + 1, nx + 1), dtype=torch.float64, device="cuda")
        v = torch.empty_like(u)
        G.transpose_x_to_y(u, v)
        torch.cuda.synchronize()
        assert torch.equal(u, v)
    finally:
        G.decomp_2d_finalize()


def _batch_items(seed, count, dims, rng_fmt=True):
    import gbfft as G
    rng = np.random.default_rng(seed)
    items = []
    for _ in range(count):
        nx, ny, nz = (int(rng.choice(dims)) for _ in range(3))
        fmt = G.PHYSICAL_IN_X if (not rng_fmt or rng.random() < 0.5) else G.PHYSICAL_IN_Z
        e = G.Engine(fmt, nx, ny, nz, prec=G.PREC_SINGLE)
        x = torch.from_numpy(rng.uniform(-1, 1, (nz, ny, nx)).astype(np.float32)).cuda()
        items.append((e, x, e.empty_spectral(), fmt))
    return items


@pytest.mark.parametrize("persistent", [True, False])
def test_batch_forward_backward_and_graph(persistent):
    import gbfft as G
    items = _batch_items(6, 10, [32, 48, 64, 96, 128, 192, 256])
    batch = G.Batch()
    for e, x, s, fmt in items:
        batch.add(e, x, s)
    batch.set_persistent(persistent)
    assert batch.info()["persistent"] == persistent
    x0 = [x.clone() for _, x, _, _ in items]
    batch.run(1)  # forward only
    torch.cuda.synchronize()
    batch.status()
    for (e, x, s, fmt), xr in zip(items, x0):
        ref = O.fft3d_r2c(xr.cpu().numpy().astype(np.float64), fmt)
        assert rel(s.cpu().numpy(), ref) <= TOL["s"]
        assert torch.equal(x, xr)
    batch.run(3)  # forward then backward: real arrays become n * x0
    torch.cuda.synchronize()
    batch.status()
    for (e, x, s, fmt), xr in zip(items, x0):
        n = e.nx * e.ny * e.nz
        assert rel((x / n).cpu().numpy(), xr.cpu().numpy()) <= 1e-6
    # graph replay of forward + backward
    stream = torch.cuda.Stream()
    for (e, x, s, fmt), xr in zip(items, x0):
        x.copy_(xr)
    torch.cuda.synchronize()
    batch.graph_build(stream)
    batch.graph_launch(stream)
    stream.synchronize()
    batch.status()
    for (e, x, s, fmt), xr in zip(items, x0):
        n = e.nx * e.ny * e.nz
        assert rel((x / n).cpu().numpy(), xr.cpu().numpy()) <= 1e-6
    batch.close()


def test_batch_with_unsupported_length_falls_back_to_loop():
    import gbfft as G
    e1 = G.Engine(G.PHYSICAL_IN_X, 64, 64, 32, prec=G.PREC_SINGLE)
    e2 = G.Engine(G.PHYSICAL_IN_X, 17, 13, 11, prec=G.PREC_SINGLE)
    batch = G.Batch()
    xs = []
    for e in (e1, e2):
        x = torch.rand((e.nz, e.ny, e.nx), device="cuda")
        s = e.empty_spectral()
        batch.add(e, x, s)
        xs.append((e, x, s, x.clone()))
    assert batch.info()["persistent"] is False
    batch.run(1)
    torch.cuda.synchronize()
    for e, x, s, x0 in xs:
        ref = O.fft3d_r2c(x0.cpu().numpy().astype(np.float64), G.PHYSICAL_IN_X)
        assert rel(s.cpu().numpy(), ref) <= TOL["s"]
    batch.close()


def test_batch_and_graph_match_single_engines():
    import gbfft as G
    rng = np.random.default_rng(6)
    dims = [32, 48, 64, 96]
    items = []
    batch = G.Batch()
    stream = torch.cuda.Stream()
    for i in range(6):
        nx, ny, nz = (int(rng.choice(dims)) for _ in range(3))
        fmt = G.PHYSICAL_IN_X if rng.random() < 0.5 else G.PHYSICAL_IN_Z
        e = G.Engine(fmt, nx, ny, nz, prec=G.PREC_SINGLE)
        x = torch.from_numpy(rng.uniform(-1, 1, (nz, ny, nx)).astype(np.float32)).cuda()
        s = e.empty_spectral()
        batch.add(e, x, s)
        items.append((e, x.clone(), s, fmt))
    batch.forward()
    torch.cuda.synchronize()
    for e, x0, s, fmt in items:
        ref = O.fft3d_r2c(x0.cpu().numpy().astype(np.float64), fmt)
        assert rel(s.cpu().numpy(), ref) <= 2e-6
    batch.graph_build(stream)
    with torch.cuda.stream(stream):
        batch.graph_launch(stream)
    stream.synchronize()
    # forward then backward leaves n * x0 in each real array
    for (e, x0, s, fmt), (_, x, _) in zip(items, batch._keep):
        n = e.nx * e.ny * e.nz
        assert torch.allclose(x / n, x0, atol=2e-5)
    batch.close()


def test_misaligned_arrays_are_rejected():
    import gbfft
    e = gbfft.Engine(gbfft.PHYSICAL_IN_X, 8, 8, 8, prec=gbfft.PREC_SINGLE)
    buf = torch.zeros(4096, dtype=torch.float32, device="cuda")
    spec = torch.zeros(8 * 8 * 5 + 2, dtype=torch.complex64, device="cuda")
    base = spec.data_ptr()
    with pytest.raises(gbfft.GbfftError, match="aligned"):
        gbfft.check(gbfft.lib().gbfft_exec_r2c(e.h, buf.data_ptr(), base + 4, None))
    with pytest.raises(gbfft.GbfftError, match="aligned"):
        gbfft.check(gbfft.lib().gbfft_exec_r2c(e.h, buf.data_ptr() + 2, base, None))
    e.close()


@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
def test_real_array_at_odd_element_offset(fmt):
    # a real array starting at an odd float: the strided pair loads/stores
    # must fall back to single elements
    import gbfft
    nx, ny, nz = 16, 8, 32
    rng = np.random.default_rng(12)
    x = rng.standard_normal((nz, ny, nx)).astype(np.float32)
    e = gbfft.Engine(fmt, nx, ny, nz, prec=gbfft.PREC_SINGLE)
    raw = torch.zeros(nx * ny * nz + 1, dtype=torch.float32, device="cuda")
    xd = raw[1:]
    xd.copy_(torch.from_numpy(x.reshape(-1)))
    s = e.empty_spectral()
    gbfft.check(gbfft.lib().gbfft_exec_r2c(e.h, xd.data_ptr(), s.data_ptr(), None))
    ref = O.fft3d_r2c(x.astype(np.float64), fmt)
    assert rel(s.cpu().numpy(), ref) <= TOL["s"]
    out_raw = torch.zeros(nx * ny * nz + 1, dtype=torch.float32, device="cuda")
    gbfft.check(gbfft.lib().gbfft_exec_c2r(e.h, s.data_ptr(), out_raw[1:].data_ptr(), None))
    torch.cuda.synchronize()
    back = out_raw[1:].cpu().numpy().reshape(nz, ny, nx) / (nx * ny * nz)
    assert np.allclose(back, x, atol=1e-5)
    e.close()


# Mixed-radix lengths with compile-time kernels (48, 96, 192, 210, 243, 270,
# 360, 384, 400) on every axis, both formats, both precisions.
MIXED_SHAPES = [(384, 400, 6), (360, 270, 4), (243, 210, 5), (48, 96, 192), (192, 48, 96),
                (210, 3, 243), (400, 2, 384), (270, 360, 2)]


@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
@pytest.mark.parametrize("shape", MIXED_SHAPES)
def test_mixed_radix_against_oracle(gpu, prec, fmt, shape):
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + 3 * ny + 7 * nz + fmt)
    x = rng.uniform(-1, 1, (nz, ny, nx))
    rt = np.float64 if prec == "d" else np.float32
    ct = np.complex128 if prec == "d" else np.complex64
    ref = O.fft3d_r2c(x, fmt)
    assert rel(gpu[prec].r2c(x.astype(rt), fmt, None), ref) <= TOL[prec]
    s = ref + 0.2 * (rng.standard_normal(ref.shape) + 1j * rng.standard_normal(ref.shape))
    assert rel(gpu[prec].c2r(s.astype(ct), nx, ny, nz, fmt, False, None),
               O.fft3d_c2r(s.copy(), nx, ny, nz, fmt)) <= TOL[prec]
    c = x + 1j * rng.uniform(-1, 1, x.shape)
    for isign in (O.FORWARD, O.BACKWARD):
        assert rel(gpu[prec].c2c(c.astype(ct), fmt, isign, False, None),
                   O.fft3d_c2c(c.copy(), fmt, isign)) <= TOL[prec]


@pytest.mark.parametrize("shape", [(384, 400, 243), (360, 270, 210)])
@pytest.mark.parametrize("prec", ["d", "s"])
def test_full_size_mixed_grids(gpu, shape, prec):
    # the non-power-of-two grids at full size: forward spectrum against the
    # FP64 oracle and the r2c -> c2r round trip
    nx, ny, nz = shape
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (nz, ny, nx))
    rt = np.float64 if prec == "d" else np.float32
    s = gpu[prec].r2c(x.astype(rt), O.PHYSICAL_IN_X, None)
    ref = O.fft3d_r2c(x, O.PHYSICAL_IN_X)
    assert rel(s, ref) <= TOL[prec]
    y = gpu[prec].c2r(s, nx, ny, nz, O.PHYSICAL_IN_X, False, None) / (nx * ny * nz)
    assert rel(y, x) <= (1e-13 if prec == "d" else 1e-6)
