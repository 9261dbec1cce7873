"""CPU: the real-to-real (DCT / DST) oracle, pinned.

* Each kind's matrix against scipy's DCT / DST types 1-4 (unnormalised),
  which implement the same FFTW r2r definitions.
* The reference's own DTT acceptance test (examples/dtt/fftw_f03_dtt_x.f90
  and fftw_f03_dtt_z.f90): for every combination of the 8 kinds on the three
  axes (512 cases) with the default windows, forward then backward on an
  8 x 9 x 10 grid of x/nx * y/ny * z/nz, rescaled as the example does, must
  give the input back within 100 * epsilon (max-abs over each axis's window).
* The configuration checks and defaults of decomp_2d_fft_engine_dtt_init.
"""
import itertools

import numpy as np
import pytest

from oracle import dtt as D


@pytest.mark.parametrize("kind", range(1, 9))
@pytest.mark.parametrize("n", [2, 3, 5, 8, 17, 64])
def test_kind_matrices_match_scipy(kind, n):
    sfft = pytest.importorskip("scipy.fft")
    if kind in (1,) and n < 2:
        pytest.skip("DCT-I needs n >= 2")
    x = np.random.default_rng(kind * 100 + n).standard_normal(n)
    y = D.dtt_matrix(kind, n) @ x
    typ = (kind - 1) % 4 + 1
    ref = sfft.dct(x, type=typ) if kind <= 4 else sfft.dst(x, type=typ)
    assert np.allclose(y, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def reference_example(fmt, cfg, nx=8, ny=9, nz=10):
    ii = np.arange(1, nx + 1) / nx
    jj = np.arange(1, ny + 1) / ny
    kk = np.arange(1, nz + 1) / nz
    a0 = kk[:, None, None] * jj[None, :, None] * ii[None, None, :]
    _, out = D.dtt_3d_r2r(a0, fmt, cfg, D.FORWARD)
    _, back = D.dtt_3d_r2r(out, fmt, cfg, D.BACKWARD)
    back = back / D.roundtrip_scale(cfg, (nx, ny, nz))
    sl = []
    for d, n in ((2, nz), (1, ny), (0, nx)):
        st = cfg[3 + d] - 1
        en = n - cfg[6 + d] + cfg[3 + d] - 1
        sl.append(slice(st, en))
    return np.abs(back - a0)[tuple(sl)].max()


@pytest.mark.parametrize("fmt", [D.PHYSICAL_IN_X, D.PHYSICAL_IN_Z])
def test_reference_dtt_example_all_512_combinations(fmt):
    eps = np.finfo(np.float64).eps
    worst = 0.0
    for kinds in itertools.product(range(1, 9), repeat=3):
        err = reference_example(fmt, D.config(kinds))
        worst = max(worst, err)
        assert err <= 100 * eps, kinds
    assert worst > 0.0


def test_config_defaults_and_inverse():
    c = D.config([1, 5, 7])
    assert c[0:3] == [1, 5, 7]
    assert c[3:6] == [1, 2, 2]      # ifirst: DST-I and DST-III start at 2
    assert c[6:9] == [0, 2, 1]      # ndismiss: DCT-I none, DST-I two, else one
    assert c[9:12] == c[3:6]
    assert c[12:15] == [1, 5, 6]    # inv(DST-III) = DST-II
    assert D.config([2, 3, 6])[12:15] == [3, 2, 7]


def test_config_rejects_bad_input():
    with pytest.raises(ValueError, match="Invalid argument"):
        D.config([0, 1, 1])
    with pytest.raises(ValueError, match="Invalid argument"):
        D.config([1, 9, 1])
    with pytest.raises(ValueError, match="Invalid argument"):
        D.config([1, 1, 1, 1])
    with pytest.raises(ValueError, match="in-place"):
        D.config([2, 2, 2, 1, 1, 1, 1, 1, 1, 2, 1, 1])


def test_windows_leave_other_points_alone():
    # DST-I on x (window 2..nx-1): the first and last x points pass through
    a = np.random.default_rng(1).standard_normal((4, 5, 9))
    cfg = D.config([5, 2, 2])
    inp, out = D.dtt_3d_r2r(a, D.PHYSICAL_IN_X, cfg, D.FORWARD, skip=(False, True, True))
    assert np.array_equal(out[:, :, 0], a[:, :, 0])
    assert np.array_equal(out[:, :, 8], a[:, :, 8])
    assert np.array_equal(inp, out)  # the x pass ran in place on the input
