"""GPU: real-to-real transforms (gbfft_exec_r2r, decomp_2d_dtt_3d_r2r).

* The reference's own acceptance test (examples/dtt/fftw_f03_dtt_x.f90,
  fftw_f03_dtt_z.f90): every combination of the 8 kinds on the 3 axes with
  the default windows, forward then backward on an 8 x 9 x 10 grid of
  x/nx * y/ny * z/nz, rescaled as the example does, within 100 * epsilon
  (max-abs over the windows) -- in FP64 and FP32.
* Forward transforms against the FP64 oracle (oracle/dtt.py) on random data:
  both formats, both directions, explicit windows (the 12-int form), skip
  flags, in == out, and the input left as the reference leaves it (the
  first pass runs in place on it).
"""
import itertools

import numpy as np
import pytest

from oracle import dtt as D

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {8: 1e-12, 4: 2e-6}  # rel-L2 against the FP64 oracle


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def dtype(prec):
    return torch.float64 if prec == 8 else torch.float32


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("fmt", [1, 3])
def test_reference_dtt_example_all_512_combinations(prec, fmt):
    import gbfft
    nx, ny, nz = 8, 9, 10
    ii = np.arange(1, nx + 1) / nx
    jj = np.arange(1, ny + 1) / ny
    kk = np.arange(1, nz + 1) / nz
    a0 = kk[:, None, None] * jj[None, :, None] * ii[None, None, :]
    eps = np.finfo(np.float64 if prec == 8 else np.float32).eps
    for kinds in itertools.product(range(1, 9), repeat=3):
        e = gbfft.Dtt(fmt, nx, ny, nz, list(kinds), prec=prec)
        cfg = e.config()
        assert cfg == D.config(kinds)
        x = torch.from_numpy(a0).to(dtype(prec)).cuda()
        out = torch.zeros_like(x)
        e.r2r(x, out, -1)
        e.r2r(out, x, 1)
        back = x.cpu().numpy().astype(np.float64) / D.roundtrip_scale(cfg, (nx, ny, nz))
        sl = []
        for d, n in ((2, nz), (1, ny), (0, nx)):
            sl.append(slice(cfg[3 + d] - 1, n - cfg[6 + d] + cfg[3 + d] - 1))
        err = np.abs(back - a0)[tuple(sl)].max()
        assert err <= 100 * eps, (kinds, err)
        e.close()


@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("isign", [-1, 1])
@pytest.mark.parametrize("shape", [(64, 48, 40), (33, 65, 17), (128, 8, 6)])
def test_r2r_against_oracle(prec, fmt, isign, shape):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + ny + nz + fmt + isign)
    for trial in range(3):
        kinds = [int(v) for v in rng.integers(1, 9, size=3)]
        a = rng.standard_normal((nz, ny, nx))
        cfg = D.config(kinds)
        e = gbfft.Dtt(fmt, nx, ny, nz, kinds, prec=prec)
        x = torch.from_numpy(a).to(dtype(prec)).cuda()
        out = torch.empty_like(x)
        e.r2r(x, out, isign)
        ref_in, ref_out = D.dtt_3d_r2r(a, fmt, cfg, isign)
        assert rel(out.cpu().numpy(), ref_out) <= TOL[prec], kinds
        assert rel(x.cpu().numpy(), ref_in) <= TOL[prec], kinds  # first pass in place
        e.close()


@pytest.mark.parametrize("prec", [8, 4])
def test_r2r_explicit_windows_skip_and_in_place(prec):
    import gbfft
    nx, ny, nz = 40, 36, 30
    rng = np.random.default_rng(5)
    a = rng.standard_normal((nz, ny, nx))
    # kinds, ifirst, ndismiss, ofirst
    dtt = [2, 5, 8, 3, 2, 1, 4, 3, 2, 3, 2, 1]
    cfg = D.config(dtt)
    for skip in [(False, False, False), (False, True, False), (True, False, True)]:
        e = gbfft.Dtt(1, nx, ny, nz, dtt, skip=skip, prec=prec)
        assert e.config() == cfg
        x = torch.from_numpy(a).to(dtype(prec)).cuda()
        out = torch.empty_like(x)
        e.r2r(x, out, -1)
        _, ref = D.dtt_3d_r2r(a, 1, cfg, -1, skip=skip)
        assert rel(out.cpu().numpy(), ref) <= TOL[prec], skip
        y = torch.from_numpy(a).to(dtype(prec)).cuda()
        e.r2r(y, y, -1)  # in == out
        assert rel(y.cpu().numpy(), ref) <= TOL[prec], skip
        e.close()


def test_r2r_rejects_bad_configuration():
    import gbfft
    with pytest.raises(gbfft.GbfftError, match="Invalid argument"):
        gbfft.Dtt(1, 8, 8, 8, [0, 1, 1])
    with pytest.raises(gbfft.GbfftError, match="Invalid argument"):
        gbfft.Dtt(1, 8, 8, 8, [1, 2])
    with pytest.raises(gbfft.GbfftError, match="in-place"):
        gbfft.Dtt(1, 8, 8, 8, [2, 2, 2, 1, 1, 1, 1, 1, 1, 2, 1, 1])
    with pytest.raises(gbfft.GbfftError, match="window"):
        gbfft.Dtt(1, 8, 8, 8, [2, 2, 2, 5, 1, 1, 1, 1, 1, 5, 1, 1])
    e = gbfft.Dtt(1, 8, 8, 8, [2, 2, 2])
    x = torch.zeros((8, 8, 8), dtype=torch.float64, device="cuda")
    with pytest.raises(gbfft.GbfftError, match="Invalid value"):
        e.r2r(x, x, 0)
    e.close()


def test_module_api_opt_dtt():
    # decomp_2d_fft_init(..., opt_DTT) / decomp_2d_dtt_3d_r2r /
    # decomp_2d_fft_get_dtt_input, and the reference's errors
    import gbfft as G
    nx, ny, nz = 12, 10, 9
    G.decomp_2d_init(nx, ny, nz, prec=G.PREC_DOUBLE)
    try:
        G.decomp_2d_fft_init(G.PHYSICAL_IN_X, nx, ny, nz)
        with pytest.raises(G.GbfftError, match="No DTT"):
            G.decomp_2d_fft_get_dtt_input()
        G.decomp_2d_fft_finalize()
        G.decomp_2d_fft_init(G.PHYSICAL_IN_X, nx, ny, nz, opt_DTT=[3, 6, 1])
        assert G.decomp_2d_fft_get_dtt_input() == (3, 6, 1)
        a = np.random.default_rng(2).standard_normal((nz, ny, nx))
        x = torch.from_numpy(a).cuda()
        out = torch.empty_like(x)
        G.decomp_2d_dtt_3d_r2r(x, out, -1)
        torch.cuda.synchronize()
        _, ref = D.dtt_3d_r2r(a, 1, D.config([3, 6, 1]), -1)
        assert rel(out.cpu().numpy(), ref) <= 1e-12
        G.decomp_2d_fft_finalize()
    finally:
        G.decomp_2d_finalize()


# Axes of 2^k + 1 points: every kind's default window has a power-of-two
# extension (DCT-I 2^k + 1 points -> 2^(k+1); DST-I 2^k - 1 -> 2^(k+1); the
# others 2^k -> 2^(k+1)), which runs the compile-time plan.
@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("shape", [(17, 33, 65), (129, 9, 17), (1025, 5, 3)])
def test_r2r_power_of_two_extensions_against_oracle(prec, fmt, shape):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + ny + nz + fmt)
    for k in range(1, 9):
        kinds = [k, k, k]
        a = rng.standard_normal((nz, ny, nx))
        cfg = D.config(kinds)
        e = gbfft.Dtt(fmt, nx, ny, nz, kinds, prec=prec)
        for isign in (-1, 1):
            x = torch.from_numpy(a).to(dtype(prec)).cuda()
            out = torch.empty_like(x)
            e.r2r(x, out, isign)
            _, ref = D.dtt_3d_r2r(a, fmt, cfg, isign)
            assert rel(out.cpu().numpy(), ref) <= TOL[prec], (k, isign)
        e.close()


@pytest.mark.parametrize("fmt", [1, 3])
def test_round_trip_all_512_combinations_power_of_two_extensions(fmt):
    import gbfft
    nx, ny, nz = 17, 33, 9
    ii = np.arange(1, nx + 1) / nx
    jj = np.arange(1, ny + 1) / ny
    kk = np.arange(1, nz + 1) / nz
    a0 = kk[:, None, None] * jj[None, :, None] * ii[None, None, :]
    eps = np.finfo(np.float64).eps
    for kinds in itertools.product(range(1, 9), repeat=3):
        e = gbfft.Dtt(fmt, nx, ny, nz, list(kinds), prec=8)
        cfg = e.config()
        x = torch.from_numpy(a0).cuda()
        out = torch.zeros_like(x)
        e.r2r(x, out, -1)
        e.r2r(out, x, 1)
        back = x.cpu().numpy() / D.roundtrip_scale(cfg, (nx, ny, nz))
        sl = []
        for d, n in ((2, nz), (1, ny), (0, nx)):
            sl.append(slice(cfg[3 + d] - 1, n - cfg[6 + d] + cfg[3 + d] - 1))
        assert np.abs(back - a0)[tuple(sl)].max() <= 100 * eps, kinds
        e.close()


# Axes of 64 and 256 points: every kind's default window has an extension
# of 126 = 9 * 14 or 510 = 17 * 30 points, which runs the compile-time
# two-stage plan in FP32 (and the runtime plan in FP64).
@pytest.mark.parametrize("prec", [8, 4])
@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("shape", [(256, 12, 10), (10, 256, 6), (6, 10, 256), (64, 64, 9)])
def test_r2r_two_stage_extensions_against_oracle(prec, fmt, shape):
    import gbfft
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + 2 * ny + 3 * nz + fmt)
    for k in range(1, 9):
        kinds = [k, k, k]
        a = rng.standard_normal((nz, ny, nx))
        cfg = D.config(kinds)
        e = gbfft.Dtt(fmt, nx, ny, nz, kinds, prec=prec)
        for isign in (-1, 1):
            x = torch.from_numpy(a).to(dtype(prec)).cuda()
            out = torch.empty_like(x)
            e.r2r(x, out, isign)
            _, ref = D.dtt_3d_r2r(a, fmt, cfg, isign)
            assert rel(out.cpu().numpy(), ref) <= TOL[prec], (k, isign)
        e.close()
