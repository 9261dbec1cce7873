"""Generate tests/golden/ramp_dft.npz: exact 1D spectra of the reference's
own test field, for pinning forward-spectrum parity.

The reference's FFT test programs (examples/fft_physical_x/fft_r2c_x.f90:65-72,
examples/fft_physical_x/fft_c2c_x.f90:64-73 and their PHYSICAL_IN_Z twins)
fill the X-pencil with

    f(i, j, k) = i/nx * j/ny * k/nz          (1-based i, j, k)

(the c2c programs use f + i f).  The field is separable, so its unnormalised
3D DFT with the forward sign is the product of three 1D spectra

    g_n(k) = sum_{m=0}^{n-1} (m+1)/n * exp(-2 pi i m k / n)
           = (n+1)/2                            k = 0
           = -1/2 + (i/2) cot(pi k / n)         k = 1 .. n-1

(from sum_m m z^m = n / (z - 1) for z^n = 1, z != 1, and
n / (exp(-i t) - 1) = -n/2 + i (n/2) cot(t/2)).  This script evaluates g_n
with mpmath at 50 significant digits, checks the closed form against the
direct sum for every n up to 64, and stores each g_n rounded once to
complex128 (key "n<length>").  Run it from the repository root:

    python tests/golden/make_ramp_golden.py
"""
import os

import mpmath
import numpy as np

# axis lengths of the shapes the golden tests use: the reference's own
# 17 x 13 x 11, the large 1024 x 1024 x 512 grid, 256^3, and the
# non-power-of-two grids 384 x 400 x 243 and 360 x 270 x 210
LENGTHS = (11, 13, 17, 64, 210, 243, 256, 270, 360, 384, 400, 512, 1024)

mpmath.mp.dps = 50


def ramp_dft(n):
    out = np.empty(n, dtype=np.complex128)
    for k in range(n):
        if k == 0:
            v = mpmath.mpc((n + 1) / mpmath.mpf(2), 0)
        else:
            v = mpmath.mpc(mpmath.mpf(-1) / 2, mpmath.cot(mpmath.pi * k / n) / 2)
        out[k] = complex(float(v.real), float(v.imag))
    return out


def direct_sum(n):
    return [mpmath.fsum((m + 1) * mpmath.expjpi(mpmath.mpf(-2) * m * k / n) for m in range(n)) / n
            for k in range(n)]


def main():
    data = {}
    for n in LENGTHS:
        g = ramp_dft(n)
        if n <= 64:
            ref = direct_sum(n)
            err = max(abs(complex(g[k]) - complex(ref[k])) for k in range(n))
            assert err < 1e-14 * n, (n, err)
        data["n%d" % n] = g
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ramp_dft.npz")
    np.savez_compressed(path, **data)
    print("wrote", path, sorted(data))


if __name__ == "__main__":
    main()
