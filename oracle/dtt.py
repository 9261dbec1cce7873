"""Oracle of the real-to-real transforms (test infrastructure only).

The reference computes `decomp_2d_dtt_3d_r2r` with FFTW's r2r plans
(src/fft_fftw3_f03.f90:341-471 configuration, :1555-1656 the 1D passes,
:1959-2023 the 3D driver).  FFTW (version 3, the library the reference's
FFTW3_F03 backend links; not vendored in the reference tree) defines its
kinds as unnormalised sums; this module restates those definitions as dense
matrices in float64 (O(n^2) a line, for the small grids of the tests) and
the reference's configuration logic and pass order around them.

Kinds (the reference's numbering, 1..8):
  1 DCT-I   (REDFT00) Y_k = x_0 + (-1)^k x_{n-1} + 2 sum_{j=1}^{n-2} x_j cos(pi j k / (n-1))
  2 DCT-II  (REDFT10) Y_k = 2 sum_j x_j cos(pi (j + 1/2) k / n)
  3 DCT-III (REDFT01) Y_k = x_0 + 2 sum_{j>=1} x_j cos(pi j (k + 1/2) / n)
  4 DCT-IV  (REDFT11) Y_k = 2 sum_j x_j cos(pi (j + 1/2)(k + 1/2) / n)
  5 DST-I   (RODFT00) Y_k = 2 sum_j x_j sin(pi (j + 1)(k + 1) / (n + 1))
  6 DST-II  (RODFT10) Y_k = 2 sum_j x_j sin(pi (j + 1/2)(k + 1) / n)
  7 DST-III (RODFT01) Y_k = (-1)^k x_{n-1} + 2 sum_{j<n-1} x_j sin(pi (j + 1)(k + 1/2) / n)
  8 DST-IV  (RODFT11) Y_k = 2 sum_j x_j sin(pi (j + 1/2)(k + 1/2) / n)

Array convention as in oracle.py: a C-ordered (nz, ny, nx) array holds the
reference's Fortran a(nx, ny, nz).
"""
import numpy as np

FORWARD = -1
BACKWARD = 1
PHYSICAL_IN_X = 1
PHYSICAL_IN_Z = 3

# inverse kind (dtt_invert, src/fft_fftw3_f03.f90:431-455): DCT-II <-> DCT-III,
# DST-II <-> DST-III, the others their own inverse
INVERSE = {1: 1, 2: 3, 3: 2, 4: 4, 5: 5, 6: 7, 7: 6, 8: 8}


def dtt_matrix(kind, n):
    """Dense n x n matrix of kind 1..8 (unnormalised, FFTW's definitions)."""
    j = np.arange(n, dtype=np.float64)
    k = j[:, None]
    if kind == 1:
        if n < 2:
            raise ValueError("DCT-I needs n >= 2")
        m = 2.0 * np.cos(np.pi * j * k / (n - 1))
        m[:, 0] = 1.0
        m[:, n - 1] = (-1.0) ** np.arange(n)
        return m
    if kind == 2:
        return 2.0 * np.cos(np.pi * (j + 0.5) * k / n)
    if kind == 3:
        m = 2.0 * np.cos(np.pi * j * (k + 0.5) / n)
        m[:, 0] = 1.0
        return m
    if kind == 4:
        return 2.0 * np.cos(np.pi * (j + 0.5) * (k + 0.5) / n)
    if kind == 5:
        return 2.0 * np.sin(np.pi * (j + 1) * (k + 1) / (n + 1))
    if kind == 6:
        return 2.0 * np.sin(np.pi * (j + 0.5) * (k + 1) / n)
    if kind == 7:
        m = 2.0 * np.sin(np.pi * (j + 1) * (k + 0.5) / n)
        m[:, n - 1] = (-1.0) ** np.arange(n)
        return m
    if kind == 8:
        return 2.0 * np.sin(np.pi * (j + 0.5) * (k + 0.5) / n)
    raise ValueError("kind must be 1..8")


def config(dtt):
    """The reference's 15-entry DTT configuration (decomp_2d_fft_engine_dtt_init,
    dtt_assign_default, dtt_invert; src/fft_fftw3_f03.f90:341-455), kinds kept
    in the 1..8 numbering:
      [0:3] forward kinds, [3:6] ifirst (1-based), [6:9] ndismiss,
      [9:12] ofirst, [12:15] backward kinds."""
    dtt = [int(v) for v in dtt]
    if len(dtt) < 3:
        raise ValueError("Invalid argument")
    if min(dtt[:3]) < 1 or max(dtt[:3]) > 8:
        raise ValueError("Invalid argument")
    c = [0] * 15
    if len(dtt) == 12:
        c[:12] = dtt
        if c[3:6] != c[9:12]:
            raise ValueError("Setup is not compatible with in-place r2r transforms")
    elif len(dtt) == 3:
        c[:3] = dtt
        c[3:6] = [1, 1, 1]
        c[6:9] = [1, 1, 1]
        for k in range(3):
            if c[k] == 1:
                c[k + 6] = 0
            if c[k] == 5:
                c[k + 3] = 2
                c[k + 6] = 2
            if c[k] == 7:
                c[k + 3] = 2
        c[9:12] = c[3:6]
    else:
        raise ValueError("Invalid argument")
    c[12:15] = [INVERSE[v] for v in c[:3]]
    return c


def r2r_axis(a, axis_xyz, kind, ifirst, ndismiss):
    """In-place r2r along one axis (x = 0, y = 1, z = 2) of a (nz, ny, nx)
    array: kind on the window of n - ndismiss points starting at ifirst
    (1-based), other points unchanged (r2r_1m_*, src/fft_fftw3_f03.f90:1555-1656)."""
    ax = 2 - axis_xyz
    n = a.shape[ax] - ndismiss
    lo = ifirst - 1
    m = dtt_matrix(kind, n)
    sl = [slice(None)] * 3
    sl[ax] = slice(lo, lo + n)
    win = np.moveaxis(a[tuple(sl)], ax, -1)
    out = np.moveaxis(win @ m.T, -1, ax)
    a[tuple(sl)] = out
    return a


def dtt_3d_r2r(a, fmt, cfg, isign, skip=(False, False, False)):
    """decomp_2d_dtt_3d_r2r at one rank (src/fft_fftw3_f03.f90:1959-2023):
    returns (input after the call, output).  The first pass works in place on
    the input; the transposes are copies."""
    a = np.array(a, dtype=np.float64, copy=True)
    if isign not in (FORWARD, BACKWARD):
        raise ValueError("Invalid value")
    kinds = cfg[0:3] if isign == FORWARD else cfg[12:15]
    first = cfg[3:6] if isign == FORWARD else cfg[9:12]
    nd = cfg[6:9]
    order = [0, 1, 2] if ((fmt == PHYSICAL_IN_X) == (isign == FORWARD)) else [2, 1, 0]
    cur = a
    for i, d in enumerate(order):
        if i > 0:
            cur = cur.copy()  # transpose at one rank
        if not skip[d]:
            r2r_axis(cur, d, kinds[d], first[d], nd[d])
        if i == 0:
            a = cur
    return a, cur


def roundtrip_scale(cfg, shape_xyz):
    """The factor the reference's DTT example divides a forward + backward round
    trip by (examples/dtt/fftw_f03_dtt_x.f90:132-161)."""
    s = 1.0
    for d in range(3):
        n, kind, nd = shape_xyz[d], cfg[d], cfg[6 + d]
        if kind in (1, 4):
            s *= 2 * n - 2
        elif kind == 5:
            s *= 2 * n + 2 - 2 * nd
        else:
            s *= 2 * n - 2 * nd
    return s
