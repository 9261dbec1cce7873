"""Run by tests/test_gpu_aux.py in a child process with GBFFT_LIBRARY set to
the bounds-checked build: r2c, c2r and c2c on prime, ragged and mixed-radix
shapes (every line-kernel family: runtime plan, power-of-two, mixed radix,
balanced plans; contiguous and strided; both formats and precisions) against
the oracle, and no bounds check firing (gbfft_engine_status)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "2decomp-fft_gb300")):
    sys.path.insert(0, p)

import numpy as np  # noqa: E402
import torch  # noqa: E402

import gbfft  # noqa: E402
from oracle import oracle as O  # noqa: E402

assert gbfft.lib().gbfft_debug_bounds_build() == 1, "not the bounds-checked build"
SHAPES = [(17, 13, 11), (7, 5, 3), (31, 2, 29), (64, 48, 30), (243, 8, 6), (11, 256, 3), (5, 3, 1024)]
for prec, tol in ((gbfft.PREC_DOUBLE, 1e-12), (gbfft.PREC_SINGLE, 2e-6)):
    rt = np.float64 if prec == 8 else np.float32
    ct = np.complex128 if prec == 8 else np.complex64
    for fmt in (gbfft.PHYSICAL_IN_X, gbfft.PHYSICAL_IN_Z):
        for nx, ny, nz in SHAPES:
            rng = np.random.default_rng(nx + ny + nz)
            x = rng.uniform(-1, 1, (nz, ny, nx))
            e = gbfft.Engine(fmt, nx, ny, nz, prec=prec)
            s = e.empty_spectral()
            e.r2c(torch.from_numpy(x.astype(rt)).cuda(), s)
            back = e.empty_physical()
            e.c2r(s, back)
            a = (x + 1j * rng.uniform(-1, 1, x.shape)).astype(ct)
            c = torch.empty(a.shape, dtype=torch.complex128 if prec == 8 else torch.complex64, device="cuda")
            e.c2c(torch.from_numpy(a).cuda(), c, gbfft.FORWARD)
            torch.cuda.synchronize()
            e.status()  # raises GbfftError (ERR_BOUNDS) if a check fired
            ref = O.fft3d_r2c(x, fmt)
            assert np.linalg.norm(s.cpu().numpy() - ref) / np.linalg.norm(ref) <= tol, (prec, fmt, nx, ny, nz)
            assert np.abs(back.cpu().numpy() / (nx * ny * nz) - x).max() <= 10 * tol
            refc = O.fft3d_c2c(a.astype(np.complex128), fmt, O.FORWARD)
            assert np.linalg.norm(c.cpu().numpy() - refc) / np.linalg.norm(refc) <= tol
            e.close()
print("bounds ok")
