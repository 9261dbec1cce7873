"""Oracle wrapper (test infrastructure only).

numpy front end over ``oracle/glassman_oracle.c``, the CPU restatement of the
2DECOMP&FFT generic backend (src/glassman.f90, src/fft_generic.f90,
src/fft_common_3d.f90).  Only tests, the smoke check and the CPU-baseline leg
of the benchmark use it, as the checker; the product never does.

Array convention: the reference stores a pencil as Fortran ``a(nx, ny, nz)``
with x fastest.  Here the same bytes are a C-ordered numpy array of shape
``(nz, ny, nx)``.  The spectral array of an r2c transform is
``(nz, ny, nx//2+1)`` for PHYSICAL_IN_X and ``(nz//2+1, ny, nx)`` for
PHYSICAL_IN_Z.

Parity status: pinned against the reference's known-answer tests (round
trips of examples/fft_physical_{x,z}, examples/fft_multiple_grids, and the
exact transpose chain of examples/test2d) and cross-checked with pocketfft;
the Fortran reference itself cannot be compiled here.
"""
import ctypes

import numpy as np

from . import build as _build

PHYSICAL_IN_X = 1
PHYSICAL_IN_Z = 3
FORWARD = -1
BACKWARD = 1

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, ip = ctypes.c_void_p, ctypes.c_int
        for sfx in ("d", "s"):
            getattr(L, "oracle_fft1d_" + sfx).argtypes = [vp, ip, ip]
            getattr(L, "oracle_fft3d_c2c_" + sfx).argtypes = [vp, vp, ip, ip, ip, ip, ip, ip, vp]
            getattr(L, "oracle_fft3d_r2c_" + sfx).argtypes = [vp, vp, ip, ip, ip, ip, vp]
            getattr(L, "oracle_fft3d_c2r_" + sfx).argtypes = [vp, vp, ip, ip, ip, ip, ip, vp]
            getattr(L, "oracle_sample_" + sfx).argtypes = [ip, ip, vp, vp, ip, ip, ip, ctypes.c_long]
        L.oracle_transpose_copy.argtypes = [vp, vp, ctypes.c_size_t]
        L.oracle_pool_release.argtypes = []
        L.oracle_set_threads.argtypes = [ip]
        L.oracle_set_threads.restype = ip
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    """Set the OpenMP thread count of the line loops; returns the count in use."""
    return lib().oracle_set_threads(int(n))


def _types(prec):
    if prec in ("d", "f64", np.float64):
        return "d", np.float64, np.complex128
    if prec in ("s", "f32", np.float32):
        return "s", np.float32, np.complex64
    raise ValueError("prec must be 'd' or 's'")


def _skip_arr(skip):
    if skip is None:
        return None, None
    arr = (ctypes.c_int * 3)(*[int(bool(s)) for s in skip])
    return arr, ctypes.cast(arr, ctypes.c_void_p)


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("oracle %s failed with status %d" % (what, rc))


def fft1d(x, isign, prec="d"):
    """Unnormalised 1D DFT by SPCFFT (src/glassman.f90:29-67); returns a copy."""
    sfx, _, ct = _types(prec)
    a = np.ascontiguousarray(np.array(x, dtype=ct, copy=True))
    _check(getattr(lib(), "oracle_fft1d_" + sfx)(a.ctypes.data, a.size, int(isign)), "fft1d")
    return a


def spectral_shape(nx, ny, nz, fmt):
    if fmt == PHYSICAL_IN_X:
        return (nz, ny, nx // 2 + 1)
    if fmt == PHYSICAL_IN_Z:
        return (nz // 2 + 1, ny, nx)
    raise ValueError("invalid format %r" % (fmt,))


def fft3d_c2c(a, fmt, isign, inplace=False, skip=None, prec="d"):
    """3D c2c (src/fft_common_3d.f90:9-116).  With inplace=True the input
    array ``a`` is overwritten with intermediate data, as in the reference."""
    sfx, _, ct = _types(prec)
    if a.dtype != ct or not a.flags.c_contiguous:
        raise TypeError("a must be a C-contiguous %s array" % np.dtype(ct))
    nz, ny, nx = a.shape
    out = np.empty_like(a)
    keep, sp = _skip_arr(skip)
    rc = getattr(lib(), "oracle_fft3d_c2c_" + sfx)(
        a.ctypes.data, out.ctypes.data, nx, ny, nz, int(fmt), int(isign), int(bool(inplace)), sp)
    _check(rc, "fft3d_c2c")
    return out


def fft3d_r2c(a, fmt, skip=None, prec="d"):
    """3D r2c (src/fft_common_3d.f90:121-189); unnormalised."""
    sfx, rt, ct = _types(prec)
    a = np.ascontiguousarray(a, dtype=rt)
    nz, ny, nx = a.shape
    out = np.empty(spectral_shape(nx, ny, nz, fmt), dtype=ct)
    keep, sp = _skip_arr(skip)
    rc = getattr(lib(), "oracle_fft3d_r2c_" + sfx)(
        a.ctypes.data, out.ctypes.data, nx, ny, nz, int(fmt), sp)
    _check(rc, "fft3d_r2c")
    return out


def fft3d_c2r(c, nx, ny, nz, fmt, inplace=False, skip=None, prec="d"):
    """3D c2r (src/fft_common_3d.f90:194-296); unnormalised.  With
    inplace=True the spectral input ``c`` is overwritten."""
    sfx, rt, ct = _types(prec)
    if c.dtype != ct or not c.flags.c_contiguous:
        raise TypeError("c must be a C-contiguous %s array" % np.dtype(ct))
    if c.shape != spectral_shape(nx, ny, nz, fmt):
        raise ValueError("spectral shape mismatch")
    out = np.empty((nz, ny, nx), dtype=rt)
    keep, sp = _skip_arr(skip)
    rc = getattr(lib(), "oracle_fft3d_c2r_" + sfx)(
        c.ctypes.data, out.ctypes.data, nx, ny, nz, int(fmt), int(bool(inplace)), sp)
    _check(rc, "fft3d_c2r")
    return out


def fft3d_r2c_into(a, out, fmt, prec="d"):
    """fft3d_r2c writing into a preallocated spectral array ``out`` (for
    timing: nothing is allocated per call)."""
    sfx, rt, ct = _types(prec)
    nz, ny, nx = a.shape
    if (a.dtype != rt or out.dtype != ct or not a.flags.c_contiguous or not out.flags.c_contiguous
            or out.shape != spectral_shape(nx, ny, nz, fmt)):
        raise TypeError("r2c_into: contiguous %s input and %s spectral output required"
                        % (np.dtype(rt), np.dtype(ct)))
    _check(getattr(lib(), "oracle_fft3d_r2c_" + sfx)(a.ctypes.data, out.ctypes.data, nx, ny, nz, int(fmt),
                                                      None), "fft3d_r2c")
    return out


def fft3d_c2r_into(c, out, fmt, prec="d"):
    """fft3d_c2r (input preserved) writing into a preallocated real array."""
    sfx, rt, ct = _types(prec)
    nz, ny, nx = out.shape
    if (c.dtype != ct or out.dtype != rt or not c.flags.c_contiguous or not out.flags.c_contiguous
            or c.shape != spectral_shape(nx, ny, nz, fmt)):
        raise TypeError("c2r_into: contiguous %s spectral input and %s output required"
                        % (np.dtype(ct), np.dtype(rt)))
    _check(getattr(lib(), "oracle_fft3d_c2r_" + sfx)(c.ctypes.data, out.ctypes.data, nx, ny, nz, int(fmt), 0,
                                                      None), "fft3d_c2r")
    return out


def pool_release():
    """Free the oracle's persistent work arrays (the stand-in for the
    reference's decomp_pool)."""
    lib().oracle_pool_release()


def transpose(src):
    """transpose_* at one rank: an identity-layout copy (src/transpose_x_to_y.f90:41-50)."""
    src = np.ascontiguousarray(src)
    dst = np.empty_like(src)
    lib().oracle_transpose_copy(dst.ctypes.data, src.ctypes.data, src.nbytes)
    return dst


def sample_pass(kind, axis, a, b, n1, n2, n3, max_lines, prec="s"):
    """Run one line pass of the generic backend over its first ``max_lines``
    lines (bounded CPU timing sample).  kind: "c2c" (on complex ``a`` of
    shape n1 x n2 x n3), "r2c" (real ``a`` -> complex ``b``) or "c2r"
    (complex ``a`` -> real ``b``; n1..n3 are the real sizes)."""
    sfx, _, _ = _types(prec)
    k = {"c2c": 0, "r2c": 1, "c2r": 2}[kind]
    rc = getattr(lib(), "oracle_sample_" + sfx)(k, axis, a.ctypes.data,
                                                 b.ctypes.data if b is not None else None,
                                                 n1, n2, n3, int(max_lines))
    _check(rc, "sample_pass")
