"""GPU: the distributed 3D FFT (gbfft.DistFFT) -- per-axis engines on each
rank's pencils and the multi-rank transposes between them -- against the
FP64 oracle on the global grid.

A 1 x 1 grid runs the normal driver (its exchanges are local copies).  Larger
p_row x p_col grids run every rank in this one process (one GPU, no rank
waits for another): the ranks' step generators advance in lockstep, and
each transpose they yield is done for all of them at once -- GPU pack,
exchange by slicing the send buffers, GPU unpack.  The spectrum gathered
from the ranks' pencils must match the oracle's (rel-L2 <= 1e-12 double,
<= 2e-6 single), and c2r must return the field times nx ny nz."""
import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {8: 1e-12, 4: 2e-6}


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def _slc(d, pencil):
    st, en = getattr(d, pencil + "st"), getattr(d, pencil + "en")
    return (slice(st[2] - 1, en[2]), slice(st[1] - 1, en[1]), slice(st[0] - 1, en[0]))


def _exchange(reqs, ffts):
    """One transpose for every rank at once: pack, slice, unpack."""
    import gbfft
    sends = []
    for (kind, src, dst, d) in reqs:
        c = d.counts(kind)
        send = torch.empty(sum(c["send_cnts"]), dtype=src.dtype, device="cuda")
        gbfft.transpose_pack(kind, src, send, c["send_dist"], c["send_disp"])
        sends.append(send)
    p_col = ffts[0].ph.p_col
    p_row = ffts[0].ph.p_row
    for r, (kind, src, dst, d) in enumerate(reqs):
        c = d.counts(kind)
        col = kind in (gbfft.X_TO_Y, gbfft.Y_TO_X)
        c1, c2 = d.coord
        peers = [q * p_col + c2 for q in range(p_row)] if col else [c1 * p_col + q for q in range(p_col)]
        me = c1 if col else c2
        recv = torch.empty(sum(c["recv_cnts"]), dtype=dst.dtype, device="cuda")
        for i, peer in enumerate(peers):
            cp = reqs[peer][3].counts(kind)
            recv[c["recv_disp"][i]: c["recv_disp"][i] + c["recv_cnts"][i]] = \
                sends[peer][cp["send_disp"][me]: cp["send_disp"][me] + cp["send_cnts"][me]]
        gbfft.transpose_unpack(kind, recv, dst, c["recv_dist"], c["recv_disp"])


def _lockstep(ffts, gens):
    pending = [next(g, None) for g in gens]
    while pending[0] is not None:
        assert all(p is not None and p[0] == pending[0][0] for p in pending)
        _exchange(pending, ffts)
        pending = [next(g, None) for g in gens]
    assert all(p is None for p in pending)


LAYOUTS = [(1, 1), (2, 2), (1, 3), (3, 1), (2, 3)]


@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("grid,prec", [((17, 13, 11), 8), ((32, 24, 16), 4)])
def test_distributed_r2c_c2r(fmt, layout, grid, prec):
    import gbfft
    nx, ny, nz = grid
    p_row, p_col = layout
    rng = np.random.default_rng(nx + ny + nz + fmt)
    g = rng.uniform(-1, 1, (nz, ny, nx))
    rt = np.float64 if prec == 8 else np.float32
    g = g.astype(rt)
    ref = O.fft3d_r2c(g.astype(np.float64), fmt)
    ranks = range(p_row * p_col)
    ffts = [gbfft.DistFFT(fmt, nx, ny, nz, p_row, p_col, r, prec=prec) for r in ranks]
    inp = "x" if fmt == O.PHYSICAL_IN_X else "z"
    outp = "z" if fmt == O.PHYSICAL_IN_X else "x"
    xs = [torch.from_numpy(np.ascontiguousarray(g[_slc(f.ph, inp)])).cuda() for f in ffts]
    specs = [torch.empty(f.spectral_shape(), dtype=f.cdtype, device="cuda") for f in ffts]
    if len(ffts) == 1:
        ffts[0].r2c(xs[0], specs[0])
    else:
        _lockstep(ffts, [f.r2c_steps(x, s) for f, x, s in zip(ffts, xs, specs)])
    torch.cuda.synchronize()
    got = np.empty(ref.shape, dtype=np.complex128)
    for f, s in zip(ffts, specs):
        got[_slc(f.sp, outp)] = s.cpu().numpy()
    assert rel(got, ref) <= TOL[prec]
    # back: c2r of each rank's spectrum (kept) gives the field times N
    keep = [s.clone() for s in specs]
    backs = [torch.empty(f.physical_shape(), dtype=f.rdtype, device="cuda") for f in ffts]
    if len(ffts) == 1:
        ffts[0].c2r(specs[0], backs[0])
    else:
        _lockstep(ffts, [f.c2r_steps(s, b) for f, s, b in zip(ffts, specs, backs)])
    torch.cuda.synchronize()
    for f, b, s, k in zip(ffts, backs, specs, keep):
        assert rel(b.cpu().numpy() / (nx * ny * nz), g[_slc(f.ph, inp)]) <= (1e-12 if prec == 8 else 2e-6)
        assert torch.equal(s, k)
    for f in ffts:
        f.close()


@pytest.mark.parametrize("fmt", [O.PHYSICAL_IN_X, O.PHYSICAL_IN_Z])
@pytest.mark.parametrize("layout", [(1, 1), (2, 2), (3, 2)])
def test_distributed_c2c(fmt, layout):
    import gbfft
    nx, ny, nz = 12, 10, 9
    p_row, p_col = layout
    rng = np.random.default_rng(5 + fmt)
    g = rng.uniform(-1, 1, (nz, ny, nx)) + 1j * rng.uniform(-1, 1, (nz, ny, nx))
    ffts = [gbfft.DistFFT(fmt, nx, ny, nz, p_row, p_col, r, prec=8) for r in range(p_row * p_col)]
    for isign in (gbfft.FORWARD, gbfft.BACKWARD):
        ref = O.fft3d_c2c(g.copy(), fmt, isign)
        x_first = (fmt == O.PHYSICAL_IN_X) == (isign == gbfft.FORWARD)
        inp, outp = ("x", "z") if x_first else ("z", "x")
        xs = [torch.from_numpy(np.ascontiguousarray(g[_slc(f.ph, inp)])).cuda() for f in ffts]
        outs = [torch.empty(f.ph.shape(outp), dtype=torch.complex128, device="cuda") for f in ffts]
        if len(ffts) == 1:
            ffts[0].c2c(xs[0], outs[0], isign)
        else:
            _lockstep(ffts, [f.c2c_steps(x, o, isign) for f, x, o in zip(ffts, xs, outs)])
        torch.cuda.synchronize()
        got = np.empty(ref.shape, dtype=np.complex128)
        for f, o in zip(ffts, outs):
            got[_slc(f.ph, outp)] = o.cpu().numpy()
        assert rel(got, ref) <= TOL[8]
    for f in ffts:
        f.close()
