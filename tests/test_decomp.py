"""CPU: the multi-rank decomposition of the C ABI (gbfft_decomp_info,
gbfft_decomp_counts, gbfft_decomp_distribute) against the numpy restatement
of the reference's arithmetic (oracle/transpose.py: distribute, partition,
get_dist, prepare_buffer), and the restated pack / unpack loops checked
against their definition: every rank of an emulated p_row x p_col grid
transposes x -> y -> z -> y -> x, the exchange done by slicing buffers, and
each rank's pencil must equal its slice of the global array, bit for bit
(the reference's test2d chain, examples/test2d/test2d.f90:77)."""
import itertools

import numpy as np
import pytest

import gbfft
from oracle import transpose as T

GRIDS = [(17, 13, 11), (8, 8, 8), (5, 7, 9), (16, 3, 12), (31, 29, 23)]
LAYOUTS = [(1, 1), (1, 2), (2, 1), (2, 2), (3, 2), (2, 3), (1, 3), (3, 1)]
KINDS = [gbfft.X_TO_Y, gbfft.Y_TO_Z, gbfft.Z_TO_Y, gbfft.Y_TO_X]


@pytest.mark.parametrize("grid", GRIDS)
@pytest.mark.parametrize("layout", LAYOUTS)
def test_info_and_counts_match_the_restatement(grid, layout):
    nx, ny, nz = grid
    p_row, p_col = layout
    if min(nx, ny) < p_row or min(ny, nz) < p_col:
        pytest.skip("grid smaller than the rank grid")
    total = {"x": 0, "y": 0, "z": 0}
    for rank in range(p_row * p_col):
        d = gbfft.Decomp(nx, ny, nz, p_row, p_col, rank)
        ref = T.pencil_info(nx, ny, nz, p_row, p_col, rank)
        assert d.coord == tuple(ref["coord"])
        for k in ("xst", "xen", "xsz", "yst", "yen", "ysz", "zst", "zen", "zsz"):
            assert list(getattr(d, k)) == list(ref[k]), k
        for p in "xyz":
            total[p] += int(np.prod(getattr(d, p + "sz")))
        for kind in KINDS:
            c = d.counts(kind)
            sd, sc, sp, rd, rc, rp = T.counts(nx, ny, nz, p_row, p_col, rank, kind)
            assert (c["send_dist"], c["send_cnts"], c["send_disp"]) == (sd, sc, sp)
            assert (c["recv_dist"], c["recv_cnts"], c["recv_disp"]) == (rd, rc, rp)
    # every pencil tiles the grid
    assert total == {"x": nx * ny * nz, "y": nx * ny * nz, "z": nx * ny * nz}


@pytest.mark.parametrize("layout", LAYOUTS)
def test_peer_counts_pair_up(layout):
    """What a rank sends to a peer is what that peer receives from it."""
    nx, ny, nz = 17, 13, 11
    p_row, p_col = layout
    for kind in KINDS:
        col = kind in (gbfft.X_TO_Y, gbfft.Y_TO_X)
        for rank in range(p_row * p_col):
            d = gbfft.Decomp(nx, ny, nz, p_row, p_col, rank)
            c = d.counts(kind)
            c1, c2 = d.coord
            peers = [q * p_col + c2 for q in range(p_row)] if col else [c1 * p_col + q for q in range(p_col)]
            me = c1 if col else c2
            for i, peer in enumerate(peers):
                cp = gbfft.Decomp(nx, ny, nz, p_row, p_col, peer).counts(kind)
                assert c["send_cnts"][i] == cp["recv_cnts"][me]


def test_distribute_matches_the_reference_example():
    # "17 meshes across 4 processor would be distibuted as (4,4,4,5)"
    # (src/decomp_2d.f90:1108-1109)
    st, en, sz = gbfft.decomp_distribute(17, 4)
    assert sz == [4, 4, 4, 5] and st == [1, 5, 9, 13] and en == [4, 8, 12, 17]
    for n, p in itertools.product(range(1, 40), range(1, 9)):
        if n >= p:
            assert list(gbfft.decomp_distribute(n, p)) == [list(v) for v in T.distribute(n, p)]


def test_invalid_grid_is_rejected_with_the_reference_message():
    with pytest.raises(gbfft.GbfftError, match="Invalid 2D processor grid"):
        gbfft.Decomp(4, 2, 8, 3, 1, 0)
    with pytest.raises(gbfft.GbfftError, match="min\\(nx,ny\\) >= p_row"):
        gbfft.Decomp(8, 8, 2, 1, 4, 0)
    with pytest.raises(gbfft.GbfftError):
        gbfft.Decomp(8, 8, 8, 2, 2, 4)  # rank outside the grid


def _slice(g, d, pencil):
    st, en = getattr(d, pencil + "st"), getattr(d, pencil + "en")
    return g[st[2] - 1:en[2], st[1] - 1:en[1], st[0] - 1:en[0]]


def emulated_chain(g, p_row, p_col, pack, unpack):
    """x -> y -> z -> y -> x on every rank of the grid, the exchange done by
    slicing each peer's send buffer; returns the pencils after each step."""
    nz, ny, nx = g.shape
    ds = [gbfft.Decomp(nx, ny, nz, p_row, p_col, r) for r in range(p_row * p_col)]
    cur = {r: np.ascontiguousarray(_slice(g, d, "x")) for r, d in enumerate(ds)}
    steps = []
    for kind, to in ((gbfft.X_TO_Y, "y"), (gbfft.Y_TO_Z, "z"), (gbfft.Z_TO_Y, "y"), (gbfft.Y_TO_X, "x")):
        col = kind in (gbfft.X_TO_Y, gbfft.Y_TO_X)
        sends = {}
        for r, d in enumerate(ds):
            c = d.counts(kind)
            sends[r] = pack(kind, cur[r], c["send_dist"], c["send_disp"], sum(c["send_cnts"]))
        nxt = {}
        for r, d in enumerate(ds):
            c = d.counts(kind)
            c1, c2 = d.coord
            peers = [q * p_col + c2 for q in range(p_row)] if col else [c1 * p_col + q for q in range(p_col)]
            me = c1 if col else c2
            recv = np.empty(sum(c["recv_cnts"]), dtype=g.dtype)
            for i, peer in enumerate(peers):
                cp = ds[peer].counts(kind)
                blk = sends[peer][cp["send_disp"][me]: cp["send_disp"][me] + cp["send_cnts"][me]]
                recv[c["recv_disp"][i]: c["recv_disp"][i] + c["recv_cnts"][i]] = blk
            nxt[r] = unpack(kind, recv, d.shape(to), c["recv_dist"], c["recv_disp"])
        cur = nxt
        steps.append((to, dict(cur), ds))
    return steps


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("dtype", [np.float64, np.complex128, np.float32, np.complex64])
def test_restated_pack_unpack_give_the_global_slices(layout, dtype):
    nx, ny, nz = 17, 13, 11
    p_row, p_col = layout
    m = np.arange(nx * ny * nz, dtype=np.float64).reshape(nz, ny, nx) + 1  # test2d.f90:77
    g = (m + 1j * m).astype(dtype) if np.iscomplexobj(np.zeros(1, dtype)) else m.astype(dtype)
    steps = emulated_chain(g, p_row, p_col,
                           lambda k, a, dist, disp, size: T.mem_split(k, a, dist, disp, size),
                           lambda k, b, shape, dist, disp: T.mem_merge(k, b, shape, dist, disp))
    for to, pencils, ds in steps:
        for r, d in enumerate(ds):
            assert np.array_equal(pencils[r], _slice(g, d, to))
