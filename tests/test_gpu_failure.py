"""GPU: failure detection without a GPU fault.

The fused x/y kernel and the batch kernel make CTAs wait for one another.
Every such wait is bounded: after its poll limit it records an error word and
returns.  Here the same wait runs on a counter nothing increments, so it must
give up, report it, and leave the GPU usable; a satisfied counter must not
report anything.  No kernel traps, faults or hangs.
"""
import time

import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _wait(counter, need, limit):
    import ctypes
    import gbfft
    out = ctypes.c_int(-1)
    gbfft.check(gbfft.lib().gbfft_selftest_bounded_wait(counter, need, limit, ctypes.byref(out)))
    return out.value


def test_bounded_wait_gives_up_and_reports():
    t0 = time.time()
    assert _wait(0, 1, 20000) == 1  # nothing ever sets the counter
    assert time.time() - t0 < 10
    # the context is still usable afterwards
    x = torch.arange(10, device="cuda", dtype=torch.float32)
    assert float(x.sum()) == 45.0


def test_bounded_wait_that_is_satisfied_reports_nothing():
    assert _wait(3, 3, 20000) == 0
    assert _wait(5, 1, 1) == 0


def test_engine_status_after_fused_transforms_is_ok():
    import gbfft
    e = gbfft.Engine(gbfft.PHYSICAL_IN_X, 256, 256, 8, prec=gbfft.PREC_SINGLE)
    e.set_fusion(True)
    x = torch.rand((8, 256, 256), device="cuda")
    s = e.empty_spectral()
    e.r2c(x, s)
    e.status()
    e.close()
