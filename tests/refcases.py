"""The reference's own FFT test programs, restated over a pluggable backend.

Each function follows one example program of the reference and keeps its
input formula, loop structure and pass threshold:

  fft_c2c      examples/fft_physical_x/fft_c2c_x.f90:64-154 (and _z, _skip)
  fft_r2c      examples/fft_physical_x/fft_r2c_x.f90:66-152 (and _z, _skip)
  multigrid    examples/fft_multiple_grids/fft_multiple_grids.f90:43-68 with
               the checks of fft_multiple_grids_utilities.f90:151-191,347-393
  test2d       examples/test2d/test2d.f90:74-199 (exact transpose chain)

A backend provides numpy-in/numpy-out c2c, r2c, c2r and transpose calls; the
oracle and the GPU library are both wrapped this way by the tests.
"""
import numpy as np

PHYSICAL_IN_X = 1
PHYSICAL_IN_Z = 3
FORWARD = -1
BACKWARD = 1


def dtypes(prec):
    return (np.float64, np.complex128) if prec == "d" else (np.float32, np.complex64)


def analytic_real(nx, ny, nz, prec):
    """real(i)/real(nx)*real(j)/real(ny)*real(k)/real(nz), 1-based, evaluated
    left to right in mytype (examples/fft_physical_x/fft_r2c_x.f90:69-70)."""
    rt, _ = dtypes(prec)
    i = np.arange(1, nx + 1, dtype=rt)[None, None, :]
    j = np.arange(1, ny + 1, dtype=rt)[None, :, None]
    k = np.arange(1, nz + 1, dtype=rt)[:, None, None]
    v = i / rt(nx)
    v = v * j
    v = v / rt(ny)
    v = v * k
    v = v / rt(nz)
    return np.ascontiguousarray(v.astype(rt))


def eps(prec):
    return float(np.finfo(np.float64 if prec == "d" else np.float32).eps)


def fft_c2c(backend, nx, ny, nz, fmt, prec, ntest=10, skip=None, inplace=False):
    """fft_c2c_{x,z}[_skip]: returns (error per mesh point, threshold)."""
    rt, ct = dtypes(prec)
    dr = analytic_real(nx, ny, nz, prec)
    a = (dr + 1j * dr).astype(ct)  # di = dr
    fwd, bwd = FORWARD, BACKWARD
    sk = skip or (False, False, False)
    ns = [nx, ny, nz]

    def normalise(x):
        # "normalisation - note 2DECOMP&FFT doesn't normalise"; only the
        # transformed axes count (fft_c2c_x_skip.f90:100-102)
        for d in range(3):
            if not sk[d]:
                x = (x / rt(ns[d])).astype(ct)
        return x

    out = backend.c2c(a.copy(), fmt, fwd, inplace, skip)
    a = backend.c2c(out, fmt, bwd, inplace, skip)
    a = normalise(a)
    for _ in range(ntest):
        out = backend.c2c(a, fmt, fwd, inplace, skip)
        a = backend.c2c(out, fmt, bwd, inplace, skip)
        a = normalise(a)
    d_r = dr - a.real
    d_i = dr - a.imag
    err = float(np.sum(np.sqrt(d_r.astype(np.float64) ** 2 + d_i.astype(np.float64) ** 2))) / (nx * ny * nz)
    return err, eps(prec) * 50 * ntest


def fft_r2c(backend, nx, ny, nz, fmt, prec, ntest=10, skip=None):
    """fft_r2c_{x,z}[_skip]: returns (error per mesh point, threshold)."""
    rt, _ = dtypes(prec)
    ref = analytic_real(nx, ny, nz, prec)
    sk = skip or (False, False, False)
    ns = [nx, ny, nz]

    def normalise(x):
        for d in range(3):
            # the real axis is always transformed (it cannot be skipped)
            real_axis = 0 if fmt == PHYSICAL_IN_X else 2
            if d == real_axis or not sk[d]:
                x = (x / rt(ns[d])).astype(rt)
        return x

    x = ref.copy()
    out = backend.r2c(x, fmt, skip)
    x = backend.c2r(out, nx, ny, nz, fmt, False, skip)
    x = normalise(x)
    for _ in range(ntest):
        out = backend.r2c(x, fmt, skip)
        x = backend.c2r(out, nx, ny, nz, fmt, False, skip)
        x = normalise(x)
    err = float(np.sum(np.abs(x.astype(np.float64) - ref.astype(np.float64)))) / (nx * ny * nz)
    return err, eps(prec) * 50 * ntest


def multigrid_c2c(backend, nx, ny, nz, fmt, prec, nt=10):
    """ntest_c2c of fft_multiple_grids: data (r, -3r), sqrt-L2 error / N <= eps*5*nt."""
    rt, ct = dtypes(prec)
    r = analytic_real(nx, ny, nz, prec)
    a = (r - 3j * r).astype(ct)
    n = rt(nx) * rt(ny) * rt(nz)
    if fmt == PHYSICAL_IN_X:
        fwd, bwd = FORWARD, BACKWARD
    else:
        fwd, bwd = FORWARD, BACKWARD
    for _ in range(nt):
        out = backend.c2c(a, fmt, fwd, False, None)
        a = backend.c2c(out, fmt, bwd, False, None)
        a = (a / n).astype(ct)
    e = np.sum((a.real.astype(np.float64) - r) ** 2 + (a.imag.astype(np.float64) + 3 * r) ** 2)
    err = float(np.sqrt(e)) / (nx * ny * nz)
    return err, eps(prec) * 5 * nt


def multigrid_r2c(backend, nx, ny, nz, fmt, prec, nt=10):
    """ntest_r2c of fft_multiple_grids: sqrt-L2 error / N <= eps*5*nt."""
    rt, _ = dtypes(prec)
    r = analytic_real(nx, ny, nz, prec)
    x = r.copy()
    n = rt(nx) * rt(ny) * rt(nz)
    for _ in range(nt):
        out = backend.r2c(x, fmt, None)
        x = backend.c2r(out, nx, ny, nz, fmt, False, None)
        x = (x / n).astype(rt)
    err = float(np.sqrt(np.sum((x.astype(np.float64) - r) ** 2))) / (nx * ny * nz)
    return err, eps(prec) * 5 * nt


def test2d_values(nx, ny, nz, dtype):
    """m = i + (j-1) nx + (k-1) nx ny (examples/test2d/test2d.f90:77)."""
    i = np.arange(1, nx + 1)[None, None, :]
    j = np.arange(1, ny + 1)[None, :, None]
    k = np.arange(1, nz + 1)[:, None, None]
    return np.ascontiguousarray((i + (j - 1) * nx + (k - 1) * nx * ny).astype(dtype))


def test2d_chain(backend, nx, ny, nz, dtype):
    """x->y->z->y->x; every stage must equal m exactly (abs(u - m) > 0 fails)."""
    m = test2d_values(nx, ny, nz, dtype)
    u2 = backend.transpose("x_to_y", m)
    ok = [np.array_equal(u2, m)]
    u3 = backend.transpose("y_to_z", u2)
    ok.append(np.array_equal(u3, m))
    u2b = backend.transpose("z_to_y", u3)
    ok.append(np.array_equal(u2b, m))
    u1 = backend.transpose("y_to_x", u2b)
    ok.append(np.array_equal(u1, m))
    return ok
