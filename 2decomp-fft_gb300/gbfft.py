"""ctypes front end of libgbfft.so (include/gbfft.h, include/decomp_2d_fft.h).

This is a thin binding used by the tests and the benchmark: every call goes
through the C ABI, with device arrays passed as raw pointers.  torch is used
only to own device memory and streams.  There is no CPU path here: when the
library is missing the import fails loudly.

Array convention: a reference pencil ``a(nx, ny, nz)`` (x fastest) is a
C-contiguous tensor of shape ``(nz, ny, nx)``.  Spectral arrays of r2c/c2r are
``(nz, ny, nx//2+1)`` (PHYSICAL_IN_X) or ``(nz//2+1, ny, nx)``
(PHYSICAL_IN_Z), of dtype complex64 (single) or complex128 (double).
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# GBFFT_LIBRARY selects another build of the library (the bounds-checked
# lib/debug/libgbfft.so); the default is the product build
LIB_PATH = os.environ.get("GBFFT_LIBRARY") or os.path.join(HERE, "lib", "libgbfft.so")

OK = 0
ERR_INVALID = 1
ERR_ALLOC = 2
ERR_CUDA = 3
ERR_UNSUPPORTED = 4
ERR_STATE = 5
ERR_TIMEOUT = 6
ERR_BOUNDS = 7

PHYSICAL_IN_X = 1
PHYSICAL_IN_Z = 3
FORWARD = -1
BACKWARD = 1
PREC_SINGLE = 4
PREC_DOUBLE = 8
FORM_PLAIN = 0
FORM_SPLIT = 1
FORM_SPLIT_TC = 2
X_TO_Y, Y_TO_Z, Z_TO_Y, Y_TO_X = 0, 1, 2, 3
PASS_NAMES = ["r2c", "c2r", "c2c_x", "c2c_y", "c2c_z", "xy_fused"]
D2D_FFT_BACKEND = 5

# Every symbol the two public headers declare, with (restype, argtypes).
_vp, _i, _ip, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_size_t
SIGNATURES = {
    "gbfft_engine_create": (_i, [_i, _i, _i, _i, _i, _ip, _i, _i, ctypes.POINTER(_vp)]),
    "gbfft_engine_destroy": (_i, [_vp]),
    "gbfft_engine_get_sizes": (_i, [_vp, _ip, _ip]),
    "gbfft_engine_work_bytes": (_i, [_vp, ctypes.POINTER(_sz)]),
    "gbfft_exec_r2c": (_i, [_vp, _vp, _vp, _vp]),
    "gbfft_exec_c2r": (_i, [_vp, _vp, _vp, _vp]),
    "gbfft_exec_c2c": (_i, [_vp, _vp, _vp, _i, _vp]),
    "gbfft_transpose": (_i, [_i, _i, _i, _vp, _vp, _i, _i, _i, _vp]),
    "gbfft_malloc": (_i, [ctypes.POINTER(_vp), _sz]),
    "gbfft_decomp_info": (_i, [_i, _i, _i, _i, _i, _i, _vp]),
    "gbfft_decomp_distribute": (_i, [_i, _i, _ip, _ip, _ip]),
    "gbfft_decomp_counts": (_i, [_i] * 7 + [_ip] * 7),
    "gbfft_transpose_pack": (_i, [_i, _i, _i, _vp, _i, _i, _i, _i, _ip, _ip, _vp, _sz, _vp]),
    "gbfft_transpose_unpack": (_i, [_i, _i, _i, _vp, _i, _i, _i, _i, _ip, _ip, _sz, _vp, _vp]),
    "gbfft_box_copy": (_i, [_i, _i, _vp, _ip, _ip, _vp, _ip, _ip, _ip, _vp]),
    "gbfft_debug_fail_alloc": (_i, [ctypes.c_longlong]),
    "gbfft_debug_live_allocations": (ctypes.c_longlong, []),
    "gbfft_set_nvtx": (_i, [_i]),
    "gbfft_debug_bounds_build": (_i, []),
    "gbfft_free": (_i, [_vp]),
    "gbfft_last_error_string": (ctypes.c_char_p, []),
    "gbfft_warning_count": (_i, []),
    "gbfft_batch_create": (_i, [ctypes.POINTER(_vp)]),
    "gbfft_batch_add": (_i, [_vp, _vp, _vp, _vp]),
    "gbfft_batch_forward": (_i, [_vp, _vp]),
    "gbfft_batch_backward": (_i, [_vp, _vp]),
    "gbfft_batch_set_persistent": (_i, [_vp, _i]),
    "gbfft_batch_run": (_i, [_vp, _i, _vp]),
    "gbfft_batch_info": (_i, [_vp, _ip, _ip]),
    "gbfft_batch_status": (_i, [_vp]),
    "gbfft_batch_graph_build": (_i, [_vp, _vp]),
    "gbfft_batch_graph_launch": (_i, [_vp, _vp]),
    "gbfft_batch_destroy": (_i, [_vp]),
    "gbfft_engine_set_profiling": (_i, [_vp, _i]),
    "gbfft_engine_set_tile": (_i, [_vp, _i, _i]),
    "gbfft_engine_set_cluster": (_i, [_vp, _i, _i, _i]),
    "gbfft_dtt_create": (_i, [_i, _i, _i, _i, _ip, _i, _ip, _i, ctypes.POINTER(_vp)]),
    "gbfft_dtt_destroy": (_i, [_vp]),
    "gbfft_dtt_get_config": (_i, [_vp, _ip]),
    "gbfft_exec_r2r": (_i, [_vp, _vp, _vp, _i, _vp]),
    "gbfft_engine_get_cluster": (_i, [_vp, _ip, _ip]),
    "gbfft_engine_set_fusion": (_i, [_vp, _i]),
    "gbfft_engine_set_layout": (_i, [_vp, _i, _i]),
    "gbfft_plan_describe": (_i, [_i, _i, _i, _i, _i, _ip, _i, _i, _i, _i, _vp, _i, _ip]),
    "gbfft_engine_get_layout": (_i, [_vp, _ip, _ip]),
    "gbfft_engine_status": (_i, [_vp]),
    "gbfft_tune_cache_path": (_i, [ctypes.c_char_p]),
    "gbfft_engine_set_plan": (_i, [_vp, _i, _i]),
    "gbfft_engine_get_tuning": (_i, [_vp, _ip, _ip, _ip]),
    "gbfft_engine_profile_read": (_i, [_vp, _i, ctypes.POINTER(ctypes.c_longlong),
                                       ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "gbfft_exec_c2r_noalloc": (_i, [_i, _i, _i, _i, _i, _vp, _vp, _vp]),
    "gbfft_selftest_bounded_wait": (_i, [_i, _i, ctypes.c_longlong, _ip]),
    "gbfft_version": (_i, [_ip, _ip]),
    "gbfft_launch_count": (ctypes.c_longlong, []),
    "gbfft_tma_pass_count": (ctypes.c_longlong, []),
    "gbfft_tc_pass_count": (ctypes.c_longlong, []),
    "gbfft_engine_set_tma": (_i, [_vp, _i]),
    "gbfft_engine_get_tma": (_i, [_vp, _ip]),
    # decomp_2d_fft.h
    "d2d_decomp_2d_init": (_i, [_i, _i, _i, _i, _i, _i]),
    "d2d_decomp_2d_finalize": (_i, []),
    "d2d_get_decomp_main": (_i, [_ip] * 9),
    "d2d_transpose_x_to_y": (_i, [_vp, _vp, _i]),
    "d2d_transpose_y_to_z": (_i, [_vp, _vp, _i]),
    "d2d_transpose_z_to_y": (_i, [_vp, _vp, _i]),
    "d2d_transpose_y_to_x": (_i, [_vp, _vp, _i]),
    "d2d_fft_set_default_inplace": (_i, [_i]),
    "d2d_fft_init": (_i, [_i, _i, _i, _i, _i, _i, _i, _i, _ip]),
    "d2d_fft_init_dtt": (_i, [_i, _i, _i, _i, _i, _i, _i, _i, _ip, _ip, _i]),
    "d2d_dtt_3d_r2r": (_i, [_vp, _vp, _i]),
    "d2d_fft_get_dtt_input": (_i, [_ip]),
    "d2d_fft_set_ngrid": (_i, [_i]),
    "d2d_fft_get_ngrid": (_i, []),
    "d2d_fft_use_grid": (_i, [_i]),
    "d2d_fft_get_engine": (_i, [_i, ctypes.POINTER(_vp)]),
    "d2d_fft_3d_c2c": (_i, [_vp, _vp, _i]),
    "d2d_fft_3d_r2c": (_i, [_vp, _vp]),
    "d2d_fft_3d_c2r": (_i, [_vp, _vp]),
    "d2d_fft_finalize": (_i, []),
    "d2d_fft_get_size": (_i, [_ip, _ip, _ip]),
    "d2d_fft_get_ph_size": (_i, [_ip]),
    "d2d_fft_get_sp_size": (_i, [_ip]),
    "d2d_fft_get_format": (_i, []),
    "d2d_fft_get_inplace": (_i, []),
    "d2d_fft_get_inplace_r2c": (_i, []),
    "d2d_fft_get_inplace_c2r": (_i, []),
    "d2d_fft_backend": (_i, []),
    "d2d_set_stream": (_i, [_vp]),
    "d2d_fft_log": (_i, [ctypes.c_char_p, _i]),
}


class GbfftError(RuntimeError):
    """A nonzero status from the library, with its message."""

    def __init__(self, status, message):
        super().__init__("gbfft status %d: %s" % (status, message))
        self.status = status
        self.message = message


_lib = None


def lib():
    """Load libgbfft.so (built by __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libgbfft.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error():
    return lib().gbfft_last_error_string().decode()


def check(status):
    if status != OK:
        raise GbfftError(status, last_error())
    return status


def launch_count():
    return int(lib().gbfft_launch_count())


def tc_pass_count():
    """gbfft_tc_pass_count: tcgen05 split-precision passes launched so far."""
    return int(lib().gbfft_tc_pass_count())


def tma_pass_count():
    """Strided passes run so far by the bulk-tensor-copy kernel."""
    return int(lib().gbfft_tma_pass_count())


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream(stream):
    if stream is None:
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(stream.cuda_stream)


def _int3(x):
    return (ctypes.c_int * 3)(*[int(v) for v in x])


def spectral_shape(nx, ny, nz, fmt):
    if fmt == PHYSICAL_IN_X:
        return (nz, ny, nx // 2 + 1)
    return (nz // 2 + 1, ny, nx)


class Dtt:
    """Real-to-real (DCT / DST) transforms of one grid (gbfft_dtt_create):
    dtt = 3 kinds 1..8 (x, y, z) or the 12-int form with the windows."""

    def __init__(self, fmt, nx, ny, nz, dtt, skip=None, prec=PREC_DOUBLE):
        self.h = ctypes.c_void_p()
        sk = _int3([int(bool(s)) for s in skip]) if skip is not None else None
        arr = (ctypes.c_int * len(dtt))(*[int(v) for v in dtt])
        check(lib().gbfft_dtt_create(int(fmt), int(nx), int(ny), int(nz), sk, int(prec), arr, len(dtt),
                                     ctypes.byref(self.h)))
        self.fmt, self.nx, self.ny, self.nz, self.prec = fmt, nx, ny, nz, prec

    def close(self):
        if self.h:
            check(lib().gbfft_dtt_destroy(self.h))
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def config(self):
        c = (ctypes.c_int * 15)()
        check(lib().gbfft_dtt_get_config(self.h, c))
        return list(c)

    def r2r(self, x, out, isign, stream=None):
        """decomp_2d_dtt_3d_r2r: x is modified by the first pass."""
        check(lib().gbfft_exec_r2r(self.h, _ptr(x), _ptr(out), int(isign), _stream(stream)))
        return out


class Engine:
    """One FFT grid (gbfft_engine_create / destroy)."""

    def __init__(self, fmt, nx, ny, nz, inplace=False, skip=None, prec=PREC_DOUBLE,
                 form=FORM_PLAIN):
        self.h = ctypes.c_void_p()
        sk = _int3([int(bool(s)) for s in skip]) if skip is not None else None
        check(lib().gbfft_engine_create(int(fmt), int(nx), int(ny), int(nz), int(bool(inplace)),
                                        sk, int(prec), int(form), ctypes.byref(self.h)))
        self.fmt, self.nx, self.ny, self.nz = fmt, nx, ny, nz
        self.prec, self.inplace = prec, inplace

    def close(self):
        if self.h:
            check(lib().gbfft_engine_destroy(self.h))
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sizes(self):
        ph, sp = (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
        check(lib().gbfft_engine_get_sizes(self.h, ph, sp))
        return tuple(ph), tuple(sp)

    def work_bytes(self):
        b = ctypes.c_size_t()
        check(lib().gbfft_engine_work_bytes(self.h, ctypes.byref(b)))
        return b.value

    def r2c(self, x, out, stream=None):
        check(lib().gbfft_exec_r2c(self.h, _ptr(x), _ptr(out), _stream(stream)))
        return out

    def c2r(self, x, out, stream=None):
        check(lib().gbfft_exec_c2r(self.h, _ptr(x), _ptr(out), _stream(stream)))
        return out

    def c2c(self, x, out, isign, stream=None):
        check(lib().gbfft_exec_c2c(self.h, _ptr(x), _ptr(out), int(isign), _stream(stream)))
        return out

    def set_tile(self, kind, lines):
        """Lines per CTA of pass kind (index into PASS_NAMES); 0 = built-in."""
        if isinstance(kind, str):
            kind = PASS_NAMES.index(kind)
        check(lib().gbfft_engine_set_tile(self.h, int(kind), int(lines)))


    def set_cluster(self, kind, ctas, sync=True):
        """Launch a pass kind's CTAs in clusters of ctas (2, 4, 8; 0 = off),
        with a cluster barrier at the start when sync."""
        k = PASS_NAMES.index(kind) if isinstance(kind, str) else int(kind)
        check(lib().gbfft_engine_set_cluster(self.h, k, int(ctas), int(bool(sync))))

    def cluster(self):
        c, s = (ctypes.c_int * len(PASS_NAMES))(), (ctypes.c_int * len(PASS_NAMES))()
        check(lib().gbfft_engine_get_cluster(self.h, c, s))
        return {k: (c[i], s[i]) for i, k in enumerate(PASS_NAMES)}

    def set_tma(self, enable):
        """Run eligible strided passes with the bulk-tensor-copy kernel."""
        check(lib().gbfft_engine_set_tma(self.h, int(bool(enable))))

    def tma(self):
        v = ctypes.c_int(0)
        check(lib().gbfft_engine_get_tma(self.h, ctypes.byref(v)))
        return bool(v.value)

    def set_layout(self, pad=1, flat=True):
        """Padded work-area rows (aligned row segments for the strided passes):
        pad 1 (or True) for r2c and c2r, 2 for c2r only, 0 (default) none;
        flat z passes over unpadded misaligned planes (default on)."""
        check(lib().gbfft_engine_set_layout(self.h, int(pad), int(bool(flat))))

    def layout(self):
        """(pad, flat): pad 0, 1 or 2, flat a bool."""
        p, f = ctypes.c_int(), ctypes.c_int()
        check(lib().gbfft_engine_get_layout(self.h, ctypes.byref(p), ctypes.byref(f)))
        return p.value, bool(f.value)

    def set_fusion(self, enable):
        """Fuse the x and y passes of each z-plane into one kernel (default on)."""
        check(lib().gbfft_engine_set_fusion(self.h, int(bool(enable))))

    def set_plan(self, axis, points):
        """Strided axis 1/2 of 512 or 1024 points: 16 or 32 points per thread."""
        check(lib().gbfft_engine_set_plan(self.h, int(axis), int(points)))

    def tuning(self):
        f = ctypes.c_int()
        tiles = (ctypes.c_int * len(PASS_NAMES))()
        pts = (ctypes.c_int * 3)()
        check(lib().gbfft_engine_get_tuning(self.h, ctypes.byref(f), tiles, pts))
        return {"fuse": bool(f.value), "tiles": dict(zip(PASS_NAMES, tiles)), "points": tuple(pts)}

    def status(self):
        """Raise GbfftError if the last fused pass gave up on a bounded wait."""
        check(lib().gbfft_engine_status(self.h))

    def set_profiling(self, enable):
        check(lib().gbfft_engine_set_profiling(self.h, int(bool(enable))))

    def profile(self):
        """{pass name: (launches, total ms, total algorithmic bytes)}"""
        res = {}
        for k, name in enumerate(PASS_NAMES):
            n, ms, by = ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
            check(lib().gbfft_engine_profile_read(self.h, k, ctypes.byref(n), ctypes.byref(ms),
                                                  ctypes.byref(by)))
            if n.value:
                res[name] = (n.value, ms.value, by.value)
        return res

    # torch conveniences ------------------------------------------------
    def _dtypes(self):
        import torch
        return (torch.float64, torch.complex128) if self.prec == PREC_DOUBLE else (torch.float32, torch.complex64)

    def empty_spectral(self, device="cuda"):
        import torch
        return torch.empty(spectral_shape(self.nx, self.ny, self.nz, self.fmt),
                           dtype=self._dtypes()[1], device=device)

    def empty_physical(self, complex_=False, device="cuda"):
        import torch
        return torch.empty((self.nz, self.ny, self.nx), dtype=self._dtypes()[1 if complex_ else 0],
                           device=device)


NOALLOC_SCRATCH_BYTES = 64 * 1024 * 1024


def set_tune_cache(path):
    """Tuning cache for engines created from now on: a path, "" for none,
    None for the default (tune_cache.txt in the package directory)."""
    check(lib().gbfft_tune_cache_path(None if path is None else path.encode()))


def c2r_noalloc(fmt, nx, ny, nz, prec, x, out, stream=None):
    """gbfft_exec_c2r_noalloc: c2r that allocates no device memory."""
    check(lib().gbfft_exec_c2r_noalloc(int(fmt), int(nx), int(ny), int(nz), int(prec), _ptr(x),
                                       _ptr(out), _stream(stream)))
    return out


def transpose(kind, src, dst, n1, n2, n3, is_complex, prec, stream=None):
    check(lib().gbfft_transpose(int(kind), int(bool(is_complex)), int(prec), _ptr(src), _ptr(dst),
                                int(n1), int(n2), int(n3), _stream(stream)))
    return dst


class PassDesc(ctypes.Structure):
    """gbfft_pass_desc_t: one axis pass of a plan (gbfft_plan_describe)."""
    _fields_ = [("kind", ctypes.c_int), ("contiguous", ctypes.c_int), ("n", ctypes.c_int),
                ("row_w", ctypes.c_int), ("nlines", ctypes.c_longlong), ("real_lines", ctypes.c_longlong),
                ("nv", ctypes.c_longlong), ("s_src_n", ctypes.c_longlong), ("s_src_l", ctypes.c_longlong),
                ("s_src_r", ctypes.c_longlong), ("s_dst_n", ctypes.c_longlong), ("s_dst_l", ctypes.c_longlong),
                ("s_dst_r", ctypes.c_longlong), ("src", ctypes.c_int), ("dst", ctypes.c_int)]


def plan_describe(fmt, nx, ny, nz, which, inplace=False, skip=(False, False, False), prec=PREC_DOUBLE,
                  pad=-1, flat=-1):
    """The axis passes an engine would run (host only, no GPU): which 0 r2c,
    1 c2r, 2 c2c forward, 3 c2c backward; a list of dicts."""
    arr = (PassDesc * 8)()
    n = ctypes.c_int()
    sk = (ctypes.c_int * 3)(*[int(bool(v)) for v in skip])
    check(lib().gbfft_plan_describe(int(fmt), int(nx), int(ny), int(nz), int(bool(inplace)), sk, int(prec),
                                    int(pad), int(flat), int(which), ctypes.cast(arr, ctypes.c_void_p), 8,
                                    ctypes.byref(n)))
    return [{f: getattr(arr[i], f) for f, _ in PassDesc._fields_} for i in range(n.value)]


class Batch:
    """gbfft_batch_*: independent grids run as one batch / one CUDA graph."""

    def __init__(self):
        self.h = ctypes.c_void_p()
        check(lib().gbfft_batch_create(ctypes.byref(self.h)))
        self._keep = []

    def add(self, engine, real, spec):
        check(lib().gbfft_batch_add(self.h, engine.h, _ptr(real), _ptr(spec)))
        self._keep.append((engine, real, spec))

    def forward(self, stream=None):
        check(lib().gbfft_batch_forward(self.h, _stream(stream)))

    def backward(self, stream=None):
        check(lib().gbfft_batch_backward(self.h, _stream(stream)))

    def set_persistent(self, enable):
        check(lib().gbfft_batch_set_persistent(self.h, int(bool(enable))))

    def run(self, mask=3, stream=None):
        check(lib().gbfft_batch_run(self.h, int(mask), _stream(stream)))

    def info(self):
        p, n = ctypes.c_int(), ctypes.c_int()
        check(lib().gbfft_batch_info(self.h, ctypes.byref(p), ctypes.byref(n)))
        return {"persistent": bool(p.value), "launches_per_run": n.value}

    def status(self):
        check(lib().gbfft_batch_status(self.h))

    def graph_build(self, stream):
        check(lib().gbfft_batch_graph_build(self.h, _stream(stream)))

    def graph_launch(self, stream=None):
        check(lib().gbfft_batch_graph_launch(self.h, _stream(stream)))

    def close(self):
        if self.h:
            check(lib().gbfft_batch_destroy(self.h))
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Mirror of the reference module API (decomp_2d_fft.h)
# ---------------------------------------------------------------------------
def decomp_2d_init(nx, ny, nz, p_row=0, p_col=0, prec=PREC_DOUBLE):
    check(lib().d2d_decomp_2d_init(nx, ny, nz, p_row, p_col, prec))


def decomp_2d_finalize():
    check(lib().d2d_decomp_2d_finalize())


def decomp_main():
    arrs = [(ctypes.c_int * 3)() for _ in range(9)]
    check(lib().d2d_get_decomp_main(*arrs))
    keys = ["xst", "xen", "xsz", "yst", "yen", "ysz", "zst", "zen", "zsz"]
    return {k: tuple(a) for k, a in zip(keys, arrs)}


def transpose_x_to_y(src, dst, is_complex=False):
    check(lib().d2d_transpose_x_to_y(_ptr(src), _ptr(dst), int(bool(is_complex))))


def transpose_y_to_z(src, dst, is_complex=False):
    check(lib().d2d_transpose_y_to_z(_ptr(src), _ptr(dst), int(bool(is_complex))))


def transpose_z_to_y(src, dst, is_complex=False):
    check(lib().d2d_transpose_z_to_y(_ptr(src), _ptr(dst), int(bool(is_complex))))


def transpose_y_to_x(src, dst, is_complex=False):
    check(lib().d2d_transpose_y_to_x(_ptr(src), _ptr(dst), int(bool(is_complex))))


def decomp_2d_fft_init(pencil=PHYSICAL_IN_X, nx=0, ny=0, nz=0, igrid=0, opt_inplace=None,
                       opt_inplace_r2c=None, opt_inplace_c2r=None, opt_skip_XYZ_c2c=None, opt_DTT=None):
    sk = _int3([int(bool(s)) for s in opt_skip_XYZ_c2c]) if opt_skip_XYZ_c2c is not None else None
    opt = lambda v: -1 if v is None else int(bool(v))
    if opt_DTT is None:
        check(lib().d2d_fft_init(pencil, nx, ny, nz, igrid, opt(opt_inplace), opt(opt_inplace_r2c),
                                 opt(opt_inplace_c2r), sk))
    else:
        dtt = (ctypes.c_int * len(opt_DTT))(*[int(v) for v in opt_DTT])
        check(lib().d2d_fft_init_dtt(pencil, nx, ny, nz, igrid, opt(opt_inplace), opt(opt_inplace_r2c),
                                     opt(opt_inplace_c2r), sk, dtt, len(opt_DTT)))


def decomp_2d_dtt_3d_r2r(x, out, isign):
    check(lib().d2d_dtt_3d_r2r(_ptr(x), _ptr(out), int(isign)))


def decomp_2d_fft_get_dtt_input():
    k = (ctypes.c_int * 3)()
    check(lib().d2d_fft_get_dtt_input(k))
    return tuple(k)


def decomp_2d_fft_set_ngrid(n):
    check(lib().d2d_fft_set_ngrid(n))


def decomp_2d_fft_get_ngrid():
    return lib().d2d_fft_get_ngrid()


def decomp_2d_fft_use_grid(igrid=0):
    check(lib().d2d_fft_use_grid(igrid))


def decomp_2d_fft_3d_c2c(x, out, isign):
    check(lib().d2d_fft_3d_c2c(_ptr(x), _ptr(out), int(isign)))


def decomp_2d_fft_3d_r2c(x, out):
    check(lib().d2d_fft_3d_r2c(_ptr(x), _ptr(out)))


def decomp_2d_fft_3d_c2r(x, out):
    check(lib().d2d_fft_3d_c2r(_ptr(x), _ptr(out)))


def decomp_2d_fft_finalize():
    check(lib().d2d_fft_finalize())


def decomp_2d_fft_get_size():
    a, b, c = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
    check(lib().d2d_fft_get_size(a, b, c))
    return tuple(a), tuple(b), tuple(c)


def decomp_2d_fft_get_ph_size():
    a = (ctypes.c_int * 3)()
    check(lib().d2d_fft_get_ph_size(a))
    return tuple(a)


def decomp_2d_fft_get_sp_size():
    a = (ctypes.c_int * 3)()
    check(lib().d2d_fft_get_sp_size(a))
    return tuple(a)


def set_stream(stream):
    check(lib().d2d_set_stream(_stream(stream) if stream is not None else None))


def decomp_2d_fft_log():
    buf = ctypes.create_string_buffer(1024)
    check(lib().d2d_fft_log(buf, 1024))
    return buf.value.decode()


# ---------------------------------------------------------------------------
# multi-rank pencil transposes (p_row x p_col ranks)
# ---------------------------------------------------------------------------
MAX_PEERS = 1024


class PencilInfo(ctypes.Structure):
    """gbfft_pencil_info_t: a rank's sub-block of each pencil (1-based)."""
    _fields_ = [(n, ctypes.c_int * 3) for n in ("xst", "xen", "xsz", "yst", "yen", "ysz", "zst", "zen", "zsz")] + \
               [("coord", ctypes.c_int * 2)]


def decomp_distribute(n, nproc):
    """distribute: 1-based starts, ends and sizes of n points over nproc."""
    a = [(ctypes.c_int * nproc)() for _ in range(3)]
    check(lib().gbfft_decomp_distribute(int(n), int(nproc), *a))
    return tuple(list(x) for x in a)


class Decomp:
    """Decomposition of an (nx, ny, nz) grid over a p_row x p_col rank grid,
    seen from `rank` (row-major: rank = coord1 * p_col + coord2): the
    rank's pencil sub-blocks (xst/xen/xsz ... , 1-based, Fortran order) and
    the exchange counts of each transpose."""

    def __init__(self, nx, ny, nz, p_row, p_col, rank):
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.p_row, self.p_col, self.rank = int(p_row), int(p_col), int(rank)
        info = PencilInfo()
        check(lib().gbfft_decomp_info(self.nx, self.ny, self.nz, self.p_row, self.p_col, self.rank,
                                      ctypes.byref(info)))
        for name, _ in PencilInfo._fields_:
            setattr(self, name, tuple(getattr(info, name)))

    def shape(self, pencil):
        """numpy / torch view (n3, n2, n1) of the rank's `pencil` ('x', 'y' or 'z')."""
        sz = getattr(self, pencil + "sz")
        return (sz[2], sz[1], sz[0])

    def counts(self, kind):
        """dict of send_dist, send_cnts, send_disp, recv_dist, recv_cnts,
        recv_disp (lists, one entry per peer of the exchange)."""
        arrs = [(ctypes.c_int * MAX_PEERS)() for _ in range(6)]
        n = ctypes.c_int(0)
        check(lib().gbfft_decomp_counts(self.nx, self.ny, self.nz, self.p_row, self.p_col, self.rank, int(kind),
                                        *arrs, ctypes.byref(n)))
        names = ("send_dist", "send_cnts", "send_disp", "recv_dist", "recv_cnts", "recv_disp")
        return {k: list(a[: n.value]) for k, a in zip(names, arrs)}


def _elem(t):
    import torch
    cplx = t.dtype in (torch.complex64, torch.complex128)
    prec = PREC_DOUBLE if t.dtype in (torch.float64, torch.complex128) else PREC_SINGLE
    return cplx, prec


def transpose_pack(kind, src, send, dist, disp, stream=None):
    """gbfft_transpose_pack: the pencil `src` (numpy view (n3, n2, n1)) into
    the 1D buffer `send` (device tensors of the same dtype)."""
    cplx, prec = _elem(src)
    n3, n2, n1 = src.shape
    p = len(dist)
    check(lib().gbfft_transpose_pack(int(kind), int(cplx), prec, _ptr(src), n1, n2, n3, p,
                                     (ctypes.c_int * p)(*dist), (ctypes.c_int * p)(*disp), _ptr(send),
                                     send.numel(), _stream(stream)))
    return send


def transpose_unpack(kind, recv, dst, dist, disp, stream=None):
    """gbfft_transpose_unpack: the received 1D buffer into the pencil `dst`."""
    cplx, prec = _elem(dst)
    n3, n2, n1 = dst.shape
    p = len(dist)
    check(lib().gbfft_transpose_unpack(int(kind), int(cplx), prec, _ptr(recv), n1, n2, n3, p,
                                       (ctypes.c_int * p)(*dist), (ctypes.c_int * p)(*disp), recv.numel(),
                                       _ptr(dst), _stream(stream)))
    return dst


def pencil_groups(p_row, p_col):
    """The row and column process groups of this rank for a p_row x p_col
    grid (torch.distributed must be initialised; every rank creates every
    group, in the same order): ROW = the p_col ranks of one grid row (y <-> z
    exchanges), COL = the p_row ranks of one grid column (x <-> y)."""
    import torch.distributed as dist
    rank = dist.get_rank()
    row = col = None
    for c1 in range(p_row):
        g = dist.new_group([c1 * p_col + c2 for c2 in range(p_col)])
        if rank // p_col == c1:
            row = g
    for c2 in range(p_col):
        g = dist.new_group([c1 * p_col + c2 for c1 in range(p_row)])
        if rank % p_col == c2:
            col = g
    return row, col


def transpose_dist(kind, src, dst, decomp, groups, pack=None, unpack=None):
    """One transpose between pencils on a p_row x p_col rank grid:
    pack (gbfft_transpose_pack), ALLTOALLV of the row (y <-> z) or column
    (x <-> y) group (torch.distributed all_to_all_single: NCCL between GPUs),
    unpack (gbfft_transpose_unpack) -- transpose_x_to_y and siblings of
    src/transpose_x_to_y.f90:96-133 etc.  `src` and `dst` are this rank's
    pencils, `groups` = pencil_groups(p_row, p_col).  With one peer the
    exchange is a local copy."""
    import torch
    import torch.distributed as dist
    pack = pack or transpose_pack
    unpack = unpack or transpose_unpack
    c = decomp.counts(kind)
    send = torch.empty(sum(c["send_cnts"]), dtype=src.dtype, device=src.device)
    recv = torch.empty(sum(c["recv_cnts"]), dtype=dst.dtype, device=dst.device)
    pack(kind, src, send, c["send_dist"], c["send_disp"])
    if len(c["send_cnts"]) == 1:
        recv.copy_(send)
    else:
        group = groups[1] if kind in (X_TO_Y, Y_TO_X) else groups[0]
        k = 2 if send.is_complex() else 1
        sv = torch.view_as_real(send).reshape(-1) if k == 2 else send
        rv = torch.view_as_real(recv).reshape(-1) if k == 2 else recv
        dist.all_to_all_single(rv, sv, [k * v for v in c["recv_cnts"]], [k * v for v in c["send_cnts"]],
                               group=group)
    unpack(kind, recv, dst, c["recv_dist"], c["recv_disp"])
    return dst


class DistFFT:
    """3D FFT of an (nx, ny, nz) grid distributed over a p_row x p_col rank
    grid, this rank's part: decomp_2d_fft_3d at p > 1 for the given
    format (src/fft_common_3d.f90:9-296 with real transposes).

    Each axis is transformed by an engine over the rank's pencil with the
    other two axes skipped, and the pencils are exchanged by
    transpose_dist: PHYSICAL_IN_X r2c = r2c along x on the X pencil,
    x -> y, c2c along y, y -> z, c2c along z (the spectrum in Z pencils);
    c2r the reverse; PHYSICAL_IN_Z the mirror image.  c2c runs the same
    path on complex data.  Arrays are this rank's pencils (numpy view
    (n3, n2, n1) of the Fortran sub-block), device tensors.

    The *_steps methods are generators: they do the local work and yield
    every transpose as (kind, src, dst, decomp) for the caller to perform;
    r2c / c2r / c2c perform them with transpose_dist on `groups`
    (pencil_groups(p_row, p_col); not needed on a 1 x 1 grid)."""

    def __init__(self, fmt, nx, ny, nz, p_row, p_col, rank, prec=PREC_SINGLE, groups=None, device="cuda"):
        import torch
        if fmt not in (PHYSICAL_IN_X, PHYSICAL_IN_Z):
            raise GbfftError(ERR_INVALID, "Invalid value for pencil")
        self.fmt, self.prec, self.groups, self.device = fmt, prec, groups, device
        self.ph = Decomp(nx, ny, nz, p_row, p_col, rank)
        sp = (nx // 2 + 1, ny, nz) if fmt == PHYSICAL_IN_X else (nx, ny, nz // 2 + 1)
        self.sp = Decomp(*sp, p_row, p_col, rank)
        self.cdtype = torch.complex64 if prec == PREC_SINGLE else torch.complex128
        self.rdtype = torch.float32 if prec == PREC_SINGLE else torch.float64

        # one pass each, from its input to its output: no work area needed
        # (a c2r input is still preserved)
        def eng(f, sz, skip):
            return Engine(f, sz[0], sz[1], sz[2], inplace=True, skip=skip, prec=prec)
        x_only, y_only, z_only = (False, True, True), (True, False, True), (True, True, False)
        if fmt == PHYSICAL_IN_X:
            self.e_real = eng(PHYSICAL_IN_X, self.ph.xsz, x_only)  # r2c / c2r along x
            self.e_last = eng(PHYSICAL_IN_X, self.sp.zsz, z_only)
        else:
            self.e_real = eng(PHYSICAL_IN_Z, self.ph.zsz, z_only)  # r2c / c2r along z
            self.e_last = eng(PHYSICAL_IN_X, self.sp.xsz, x_only)
        self.e_y = eng(PHYSICAL_IN_X, self.sp.ysz, y_only)
        self._tmp = {}
        self._cx = None

    def _t(self, pencil, decomp=None):
        d = decomp or self.sp
        key = (pencil, id(d))
        if key not in self._tmp:
            import torch
            self._tmp[key] = torch.empty(d.shape(pencil), dtype=self.cdtype, device=self.device)
        return self._tmp[key]

    def spectral_shape(self):
        return self.sp.shape("z" if self.fmt == PHYSICAL_IN_X else "x")

    def physical_shape(self):
        return self.ph.shape("x" if self.fmt == PHYSICAL_IN_X else "z")

    def r2c_steps(self, x, out):
        first, last = ("x", "z") if self.fmt == PHYSICAL_IN_X else ("z", "x")
        k1, k2 = (X_TO_Y, Y_TO_Z) if self.fmt == PHYSICAL_IN_X else (Z_TO_Y, Y_TO_X)
        t1, ty = self._t(first), self._t("y")
        self.e_real.r2c(x, t1)
        yield (k1, t1, ty, self.sp)
        self.e_y.c2c(ty, ty, FORWARD)
        yield (k2, ty, out, self.sp)
        self.e_last.c2c(out, out, FORWARD)

    def c2r_steps(self, c, out):
        """The input spectrum is preserved."""
        first, last = ("x", "z") if self.fmt == PHYSICAL_IN_X else ("z", "x")
        k1, k2 = (Z_TO_Y, Y_TO_X) if self.fmt == PHYSICAL_IN_X else (X_TO_Y, Y_TO_Z)
        tl, ty, t1 = self._t(last), self._t("y"), self._t(first)
        self.e_last.c2c(c, tl, BACKWARD)
        yield (k1, tl, ty, self.sp)
        self.e_y.c2c(ty, ty, BACKWARD)
        yield (k2, ty, t1, self.sp)
        self.e_real.c2r(t1, out)

    def c2c_steps(self, a, out, isign):
        """Complex data on the full grid: X pencil in, Z pencil out (forward,
        PHYSICAL_IN_X) or the reverse, as src/fft_common_3d.f90:9-116."""
        if self._cx is None:
            def eng(sz, skip):
                return Engine(PHYSICAL_IN_X, sz[0], sz[1], sz[2], inplace=True, skip=skip, prec=self.prec)
            self._cx = {"x": eng(self.ph.xsz, (False, True, True)), "y": eng(self.ph.ysz, (True, False, True)),
                        "z": eng(self.ph.zsz, (True, True, False))}
        x_first = (self.fmt == PHYSICAL_IN_X) == (isign == FORWARD)
        order = ("x", "y", "z") if x_first else ("z", "y", "x")
        kinds = (X_TO_Y, Y_TO_Z) if x_first else (Z_TO_Y, Y_TO_X)
        t0, ty = self._t(order[0], self.ph), self._t("y", self.ph)
        self._cx[order[0]].c2c(a, t0, isign)
        yield (kinds[0], t0, ty, self.ph)
        self._cx["y"].c2c(ty, ty, isign)
        yield (kinds[1], ty, out, self.ph)
        self._cx[order[2]].c2c(out, out, isign)

    def _drive(self, steps):
        for kind, src, dst, decomp in steps:
            transpose_dist(kind, src, dst, decomp, self.groups)

    def r2c(self, x, out):
        self._drive(self.r2c_steps(x, out))
        return out

    def c2r(self, c, out):
        self._drive(self.c2r_steps(c, out))
        return out

    def c2c(self, a, out, isign):
        self._drive(self.c2c_steps(a, out, isign))
        return out

    def close(self):
        for e in [self.e_real, self.e_y, self.e_last] + (list(self._cx.values()) if self._cx else []):
            e.close()


# ---------------------------------------------------------------------------
# halo-cell update (src/halo.f90, src/halo_common.f90)
# ---------------------------------------------------------------------------
HALO_PHASES = {"x": (1, 2), "y": (0, 2), "z": (0, 1)}  # distributed axes, phase order


def box_copy(src, src_off, dst, dst_off, box, stream=None):
    """gbfft_box_copy: the Fortran box `box` = (w1, w2, w3) of `src` at
    src_off into `dst` at dst_off (0-based offsets; tensors viewed
    (n3, n2, n1), same dtype, on the device)."""
    cplx, prec = _elem(src)
    sd = src.shape[::-1]
    dd = dst.shape[::-1]
    check(lib().gbfft_box_copy(int(cplx), prec, _ptr(src), _int3(sd), _int3(src_off), _ptr(dst), _int3(dd),
                               _int3(dst_off), _int3(box), _stream(stream)))
    return dst


def halo_extents(pencil, sizes, level, start=None):
    """Index ranges (1-based, inclusive, Fortran order) of the halo-extended
    array of a pencil of local sizes (s1, s2, s3): init_halo_extents of
    src/halo.f90:230-309.  With `start` (the pencil's xst / yst / zst) the
    global-coordinate form (opt_global)."""
    st = list(start) if start is not None else [1, 1, 1]
    lo, hi = [], []
    for d in range(3):
        l = level if d in HALO_PHASES[pencil] else 0
        lo.append(st[d] - l)
        hi.append(st[d] + sizes[d] - 1 + l)
    return lo, hi


def _halo_neighbours(coord, dims, cdim, periodic):
    me = coord[cdim]

    def nb(shift):
        c = list(coord)
        v = me + shift
        if v < 0 or v >= dims[cdim]:
            if not periodic:
                return None
            v %= dims[cdim]
        c[cdim] = v
        return c[0] * dims[1] + c[1]
    return nb(-1), nb(+1)


def update_halo(inp, level, decomp, pencil, periodic=(False, False, False), copy=None, exchange=None):
    """update_halo (src/halo.f90:100-146 with src/halo_common.f90): a new
    array holding this rank's pencil `inp` with `level` halo cells on the
    pencil's two distributed axes, filled from the neighbouring ranks of the
    p_row x p_col grid of `decomp` (rank, coordinates, grid).  periodic =
    (periodic_x, periodic_y, periodic_z) of decomp_2d_init.

    As the reference: the halos are filled in two phases (X pencil: y then
    z, Y pencil: x then z, Z pencil: x then y), each moving slabs that span
    the whole halo-extended array in the other axes, so the corners come
    from diagonal neighbours; across a non-periodic edge a halo is left as
    allocated (unset); on a periodic dimension of one rank the rank is its
    own neighbour and, as the reference's two same-tag messages match, its
    low halo receives its own first interior planes and its high halo its
    last ones.

    Device work: one box copy into the interior, box copies packing and
    unpacking the slabs (gbfft_box_copy); the exchange: torch.distributed
    point-to-point in two batches per phase (every rank's minus-going
    messages, then its plus-going ones), so that a pair of ranks that are
    each other's two neighbours never has two messages in flight the same
    way.  `copy` / `exchange` replace the device copy and the exchange
    (tests)."""
    import torch
    copy = copy or box_copy
    sizes = list(inp.shape[::-1])
    if pencil not in HALO_PHASES:
        raise GbfftError(ERR_INVALID, "Invalid data passed to update_halo")
    for a in HALO_PHASES[pencil]:
        if level < 0 or sizes[a] < level:
            raise GbfftError(ERR_INVALID, "halo level larger than the local pencil")
    ext = list(sizes)
    for a in HALO_PHASES[pencil]:
        ext[a] += 2 * level
    out = torch.empty(ext[::-1], dtype=inp.dtype, device=inp.device)
    off = [level if d in HALO_PHASES[pencil] else 0 for d in range(3)]
    copy(inp, [0, 0, 0], out, off, sizes)
    if level == 0:
        return out
    dims = (decomp.p_row, decomp.p_col)
    for phase, axis in enumerate(HALO_PHASES[pencil]):
        minus, plus = _halo_neighbours(decomp.coord, dims, phase, periodic[axis])
        s = sizes[axis]
        box = list(ext)
        box[axis] = level

        def at(pos):
            o = [0, 0, 0]
            o[axis] = pos
            return o
        me = decomp.rank
        # the rank its own neighbour (one rank on a periodic dimension): the
        # reference's matching gives each halo the adjacent interior planes
        if minus == me and plus == me:
            copy(out, at(level), out, at(0), box)
            copy(out, at(s), out, at(s + level), box)
            continue
        def slab(pos):
            b = torch.empty(box[::-1], dtype=out.dtype, device=out.device)
            copy(out, at(pos), b, [0, 0, 0], box)
            return b
        # minus-going: own first interior planes to minus, high halo from plus
        # plus-going: own last interior planes to plus, low halo from minus
        send_lo = slab(level) if minus is not None else None
        send_hi = slab(s) if plus is not None else None
        recv_hi = torch.empty(box[::-1], dtype=out.dtype, device=out.device) if plus is not None else None
        recv_lo = torch.empty(box[::-1], dtype=out.dtype, device=out.device) if minus is not None else None
        (exchange or _p2p)([(send_lo, minus)], [(recv_hi, plus)])
        (exchange or _p2p)([(send_hi, plus)], [(recv_lo, minus)])
        if recv_hi is not None:
            copy(recv_hi, [0, 0, 0], out, at(s + level), box)
        if recv_lo is not None:
            copy(recv_lo, [0, 0, 0], out, at(0), box)
    return out


def _p2p(sends, recvs):
    """One batch of point-to-point messages (torch.distributed)."""
    import torch
    import torch.distributed as dist
    ops = []
    for t, peer in sends:
        if t is not None and peer is not None:
            ops.append(dist.P2POp(dist.isend, torch.view_as_real(t) if t.is_complex() else t, peer))
    for t, peer in recvs:
        if t is not None and peer is not None:
            ops.append(dist.P2POp(dist.irecv, torch.view_as_real(t) if t.is_complex() else t, peer))
    if ops:
        for req in dist.batch_isend_irecv(ops):
            req.wait()
