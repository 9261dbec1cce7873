"""CPU: the C-ABI library loads, exports every declared symbol, and rejects
bad arguments on the host with the reference's messages.  No GPU calls."""
import ctypes
import os
import re

import pytest

import gbfft

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("gbfft.h", "decomp_2d_fft.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b([a-z_][a-z0-9_]*)\s*\(", src):
            name = m.group(1)
            if name.startswith(("gbfft_", "d2d_")):
                names.add(name)
    return names


def test_every_declared_symbol_is_exported():
    L = gbfft.lib()
    decl = declared_functions()
    assert len(decl) >= 40
    for name in sorted(decl):
        assert hasattr(L, name), name


def test_binding_covers_every_declaration():
    assert set(gbfft.SIGNATURES) == declared_functions()


def test_constants_match_reference():
    # src/decomp_2d_constants.f90:86-93
    assert gbfft.PHYSICAL_IN_X == 1 and gbfft.PHYSICAL_IN_Z == 3
    assert gbfft.FORWARD == -1 and gbfft.BACKWARD == 1
    assert gbfft.lib().d2d_fft_backend() == 5


@pytest.mark.parametrize("args,msg", [
    ((1, 0, 4, 4), "Invalid value for nx"),
    ((1, 4, 0, 4), "Invalid value for ny"),
    ((1, 4, 4, -1), "Invalid value for nz"),
    ((2, 4, 4, 4), "Invalid value for pencil"),
])
def test_engine_create_rejects_bad_sizes(args, msg):
    fmt, nx, ny, nz = args
    h = ctypes.c_void_p()
    rc = gbfft.lib().gbfft_engine_create(fmt, nx, ny, nz, 0, None, 8, 0, ctypes.byref(h))
    assert rc == gbfft.ERR_INVALID
    assert gbfft.last_error() == msg
    assert not h.value


def test_engine_create_rejects_bad_precision_and_form():
    h = ctypes.c_void_p()
    L = gbfft.lib()
    assert L.gbfft_engine_create(1, 4, 4, 4, 0, None, 2, 0, ctypes.byref(h)) == gbfft.ERR_INVALID
    assert L.gbfft_engine_create(1, 4, 4, 4, 0, None, 8, 7, ctypes.byref(h)) == gbfft.ERR_INVALID


def test_exec_rejects_null_engine():
    L = gbfft.lib()
    assert L.gbfft_exec_r2c(None, None, None, None) == gbfft.ERR_INVALID
    assert L.gbfft_exec_c2c(None, None, None, -1, None) == gbfft.ERR_INVALID
    assert L.gbfft_engine_destroy(None) == gbfft.OK


def test_transpose_rejects_bad_kind():
    L = gbfft.lib()
    assert L.gbfft_transpose(9, 0, 8, None, None, 1, 1, 1, None) == gbfft.ERR_INVALID
    # zero elements is a no-op, as cudaMemcpy of 0 bytes is
    assert L.gbfft_transpose(0, 0, 8, None, None, 0, 4, 4, None) == gbfft.OK


def test_module_mirror_state_errors():
    L = gbfft.lib()
    L.d2d_decomp_2d_finalize()
    # FFT calls before initialisation
    assert L.d2d_fft_3d_r2c(None, None) == gbfft.ERR_STATE
    assert "initialised first" in gbfft.last_error()
    assert L.d2d_fft_init(1, 0, 0, 0, 0, -1, -1, -1, None) == gbfft.ERR_STATE
    # decomp_2d_init: one rank only
    assert L.d2d_decomp_2d_init(8, 8, 8, 2, 1, 8) == gbfft.ERR_UNSUPPORTED
    assert L.d2d_decomp_2d_init(8, 8, 8, 1, 1, 8) == gbfft.OK
    try:
        assert L.d2d_fft_set_ngrid(0) == gbfft.ERR_INVALID
        assert gbfft.last_error() == "Invalid value for n_grid"
        assert L.d2d_fft_use_grid(0) == gbfft.ERR_STATE
        assert gbfft.last_error() == "The FFT module was not initialised"
        assert L.d2d_fft_set_ngrid(2) == gbfft.OK
        assert L.d2d_fft_get_ngrid() == 2
        assert L.d2d_fft_use_grid(3) == gbfft.ERR_INVALID
        assert gbfft.last_error() == "Invalid value for igrid"
        assert L.d2d_fft_use_grid(1) == gbfft.ERR_STATE
        assert gbfft.last_error() == "FFT engine is not ready"
        assert L.d2d_fft_init(1, 8, 8, 8, 5, -1, -1, -1, None) == gbfft.ERR_INVALID
        assert L.d2d_fft_init(1, 0, 8, 8, 1, -1, -1, -1, None) == gbfft.ERR_INVALID
        assert gbfft.last_error() == "Invalid value for nx"
        assert L.d2d_fft_init(1, 8, 8, 8, 1, -1, 1, -1, None) == gbfft.ERR_UNSUPPORTED
        assert gbfft.last_error() == "In-place r2c transform is not yet available"
        assert L.d2d_fft_init(1, 8, 8, 8, 1, -1, -1, 0, None) == gbfft.ERR_UNSUPPORTED
        assert gbfft.last_error() == "In-place c2r transform is not yet available"
        main = gbfft.decomp_main()
        assert main["xst"] == (1, 1, 1) and main["zsz"] == (8, 8, 8)
    finally:
        L.d2d_decomp_2d_finalize()


def test_missing_library_fails_loudly():
    # no silent fallback: without the built library the binding refuses to load
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, %r); import gbfft\n"
            "try:\n    gbfft.lib()\nexcept ImportError as e:\n    print('refused:', e)\n    raise SystemExit(3)\n"
            % os.path.join(ROOT, "2decomp-fft_gb300"))
    env = dict(os.environ, GBFFT_LIBRARY=os.path.join(ROOT, "no_such_dir", "libgbfft.so"))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 3 and "refused: libgbfft.so is not built" in r.stdout


@pytest.mark.skipif(__import__("torch").cuda.is_available(), reason="a GPU is present")
def test_engine_without_a_gpu_is_an_error_not_a_fallback():
    # the library has no CPU path: engine creation needs the device and
    # reports why it cannot have it
    with pytest.raises(gbfft.GbfftError) as ei:
        gbfft.Engine(1, 16, 16, 16, prec=gbfft.PREC_SINGLE)
    assert "cuda" in str(ei.value).lower()
