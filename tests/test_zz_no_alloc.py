"""GPU: the allocation-free c2r (gbfft_exec_c2r_noalloc) against the regular
c2r entry point (gbfft_exec_c2r), two calls in a row per case.

The allocation-free entry point exists for callers that may not call
cudaMalloc (code under another runtime's memory pool, callbacks, programs
that reserved all device memory up front); it keeps its tables and work area
in one static 64 MiB device array.  This file is collected last so that a
run stopping at the first failure has already run every other test; it also
passes on its own in a fresh process (the first call does the per-device
set-up).  Tolerances are those of the parity tests: relative L2 <= 1e-12 in
double, <= 2e-6 in single.
"""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {8: 1e-12, 4: 2e-6}


def _rel(a, b):
    den = torch.linalg.vector_norm(b.double())
    return float(torch.linalg.vector_norm((a - b).double()) / (den if den > 0 else 1.0))


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("shape", [(17, 13, 11), (64, 48, 30), (128, 96, 64)])
def test_noalloc_c2r_matches_regular_c2r(prec, fmt, shape):
    import gbfft
    nx, ny, nz = shape
    rdt = torch.float64 if prec == 8 else torch.float32
    eng = gbfft.Engine(fmt, nx, ny, nz, prec=prec)
    g = torch.Generator(device="cuda").manual_seed(nx + ny + nz + fmt + prec)
    x = (torch.rand((nz, ny, nx), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).to(rdt)
    spec = eng.empty_spectral()
    eng.r2c(x, spec)
    keep = spec.clone()
    ref = eng.empty_physical()
    eng.c2r(spec, ref)
    for _ in range(2):  # two calls in a row share and reuse the static array
        out = torch.full_like(ref, float("nan"))
        gbfft.c2r_noalloc(fmt, nx, ny, nz, prec, spec, out)
        torch.cuda.synchronize()
        assert torch.isfinite(out).all()
        assert _rel(out, ref) <= TOL[prec]
        assert torch.equal(spec, keep)  # the input is preserved
    eng.close()


def test_noalloc_rejects_sizes_beyond_the_static_scratch():
    import gbfft
    nx, ny, nz = 512, 256, 128  # spectral array 257*256*128*16 B = 128.5 MiB
    x = torch.zeros(8, dtype=torch.complex128, device="cuda")
    y = torch.zeros(8, dtype=torch.float64, device="cuda")
    with pytest.raises(gbfft.GbfftError, match="static scratch"):
        gbfft.c2r_noalloc(1, nx, ny, nz, 8, x, y)


def test_noalloc_rejects_misaligned_arrays_before_any_launch():
    """A byte-offset view of a complex or real array is refused with
    GBFFT_ERR_INVALID on the host (nothing is launched, so nothing faults)."""
    import ctypes

    import gbfft
    nx, ny, nz = 16, 8, 4
    spec = torch.zeros((nz, ny, nx // 2 + 1), dtype=torch.complex128, device="cuda")
    out = torch.zeros((nz, ny, nx), dtype=torch.float64, device="cuda")
    before = gbfft.launch_count()
    lib = gbfft.lib()
    for din, dout in ((spec.data_ptr() + 8, out.data_ptr()), (spec.data_ptr(), out.data_ptr() + 4)):
        rc = lib.gbfft_exec_c2r_noalloc(1, nx, ny, nz, 8, ctypes.c_void_p(din), ctypes.c_void_p(dout), None)
        assert rc == gbfft.ERR_INVALID
        assert "aligned" in gbfft.last_error()
    assert gbfft.launch_count() == before
