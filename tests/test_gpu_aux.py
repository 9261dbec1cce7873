"""GPU: failure paths and debugging aids.

  * every device allocation of engine creation (twiddle tables, work area,
    status word, fused-pass counters, long-axis scratch) and of a persistent
    batch's first run, driven one at a time into failure by
    gbfft_debug_fail_alloc: each call returns GBFFT_ERR_ALLOC and the library
    holds no more allocations than before it;
  * NVTX ranges switched on around transforms (the results unchanged);
  * the bounds-checked build (-DGB_DEBUG_BOUNDS, built here into
    lib/debug/): prime and ragged shapes through every line-kernel family
    against the oracle, in a child process loading that build, with no
    bounds check firing."""
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _count_allocs(fn):
    import gbfft
    L = gbfft.lib()
    before = L.gbfft_debug_live_allocations()
    obj = fn()
    n = L.gbfft_debug_live_allocations() - before
    return obj, n


@pytest.mark.parametrize("shape,prec", [((64, 32, 16), 4), ((17, 13, 11), 8), ((16384, 2, 2), 4)])
def test_every_engine_allocation_failure_is_clean(shape, prec):
    import gbfft
    L = gbfft.lib()
    nx, ny, nz = shape
    eng, n = _count_allocs(lambda: gbfft.Engine(gbfft.PHYSICAL_IN_X, nx, ny, nz, prec=prec))
    eng.close()
    assert n >= 4
    for k in range(n):
        base = L.gbfft_debug_live_allocations()
        gbfft.check(L.gbfft_debug_fail_alloc(k))
        try:
            with pytest.raises(gbfft.GbfftError) as ei:
                gbfft.Engine(gbfft.PHYSICAL_IN_X, nx, ny, nz, prec=prec)
            assert ei.value.status == gbfft.ERR_ALLOC
        finally:
            L.gbfft_debug_fail_alloc(-1)
        assert L.gbfft_debug_live_allocations() == base
    # and it still works afterwards
    e = gbfft.Engine(gbfft.PHYSICAL_IN_X, nx, ny, nz, prec=prec)
    e.close()


def test_batch_allocation_failure_is_clean():
    import gbfft
    L = gbfft.lib()
    e = gbfft.Engine(gbfft.PHYSICAL_IN_X, 48, 32, 64, prec=gbfft.PREC_SINGLE)
    x = torch.rand((64, 32, 48), device="cuda")
    s = e.empty_spectral()
    probe = gbfft.Batch()
    probe.add(e, x, s)
    assert probe.info()["persistent"]  # the one-launch path: its descriptors are allocated on first run
    probe.close()
    for k in range(3):
        b = gbfft.Batch()
        b.add(e, x, s)
        base = L.gbfft_debug_live_allocations()
        gbfft.check(L.gbfft_debug_fail_alloc(k))
        try:
            with pytest.raises(gbfft.GbfftError) as ei:
                b.run(1)
            assert ei.value.status == gbfft.ERR_ALLOC
        finally:
            L.gbfft_debug_fail_alloc(-1)
        assert L.gbfft_debug_live_allocations() == base
        b.run(1)  # builds its descriptors now
        torch.cuda.synchronize()
        b.close()
    e.close()


def test_nvtx_ranges_leave_results_unchanged():
    import gbfft
    L = gbfft.lib()
    nx, ny, nz = 24, 18, 10
    x = np.random.default_rng(3).uniform(-1, 1, (nz, ny, nx))
    e = gbfft.Engine(gbfft.PHYSICAL_IN_X, nx, ny, nz, prec=gbfft.PREC_DOUBLE)
    s = e.empty_spectral()
    gbfft.check(L.gbfft_set_nvtx(1))
    try:
        e.r2c(torch.from_numpy(x).cuda(), s)
        torch.cuda.synchronize()
    finally:
        L.gbfft_set_nvtx(0)
    ref = O.fft3d_r2c(x, O.PHYSICAL_IN_X)
    assert np.linalg.norm(s.cpu().numpy() - ref) / np.linalg.norm(ref) <= 1e-12
    e.close()


@pytest.fixture(scope="module")
def debug_library():
    sys.path.insert(0, os.path.join(ROOT, "2decomp-fft_gb300"))
    import importlib.util
    spec = importlib.util.spec_from_file_location("gbfft_build_dbg", os.path.join(ROOT, "2decomp-fft_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(variant="debug")


def test_bounds_checked_build_on_prime_and_ragged_shapes(debug_library):
    env = dict(os.environ, GBFFT_LIBRARY=debug_library)
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_check_run.py")], env=env, cwd=ROOT,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bounds ok" in r.stdout
