"""CPU: the allocator that fails on demand (gbfft_debug_fail_alloc).  The
first device allocation of engine creation or of gbfft_malloc fails as
armed, whether or not a GPU is present: the call returns GBFFT_ERR_ALLOC with
the out-of-memory message and holds nothing."""
import pytest

import gbfft


def test_armed_allocation_failure_is_reported_as_alloc():
    L = gbfft.lib()
    before = L.gbfft_debug_live_allocations()
    gbfft.check(L.gbfft_debug_fail_alloc(0))
    try:
        with pytest.raises(gbfft.GbfftError) as ei:
            gbfft.Engine(gbfft.PHYSICAL_IN_X, 16, 8, 4, prec=gbfft.PREC_SINGLE)
        assert ei.value.status == gbfft.ERR_ALLOC
        assert "out of memory" in ei.value.message
    finally:
        L.gbfft_debug_fail_alloc(-1)
    assert L.gbfft_debug_live_allocations() == before
    gbfft.check(L.gbfft_debug_fail_alloc(0))
    import ctypes
    p = ctypes.c_void_p()
    assert L.gbfft_malloc(ctypes.byref(p), 1024) == gbfft.ERR_ALLOC
    assert not p.value
    L.gbfft_debug_fail_alloc(-1)


def test_debug_switches_accept_and_reject():
    L = gbfft.lib()
    assert L.gbfft_debug_fail_alloc(-2) == gbfft.ERR_INVALID
    assert L.gbfft_debug_fail_alloc(-1) == gbfft.OK
    assert L.gbfft_set_nvtx(1) == gbfft.OK and L.gbfft_set_nvtx(0) == gbfft.OK
    assert L.gbfft_debug_bounds_build() == 0  # the product build
