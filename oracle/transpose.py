"""Oracle (test infrastructure only) of the multi-rank pencil transposes:
numpy restatement of the reference's decomposition arithmetic and of its
pack / unpack loops.  Tests use it as the checker of the C ABI
(gbfft_decomp_*, gbfft_transpose_pack / _unpack) and as the CPU stand-in for
the GPU kernels when the exchange itself is tested on CPU ranks (gloo).

Arrays follow the numpy view of a Fortran pencil a(n1, n2, n3): C-ordered
shape (n3, n2, n1).  Indices in the returned decomposition are 1-based, as
in the reference.

Restated, with the reference lines each function follows:
  distribute      src/decomp_2d.f90:1070-1105
  pencil_info     src/decomp_2d.f90:1016-1064 (partition; pencils :411-416)
  counts          src/decomp_2d.f90:1112-1133 (get_dist), :1138-1206
                  (prepare_buffer), per transpose direction as the ALLTOALLV
                  calls use them (src/transpose_x_to_y.f90:124-126,
                  src/transpose_y_to_z.f90:144-146 and the reverse files)
  mem_split       src/transpose_x_to_y.f90:266-323 (split_xy), and
                  mem_split_yz / _zy / _yx of the sibling files
  mem_merge       src/transpose_x_to_y.f90:384-441 (merge_xy), and
                  mem_merge_yz / _zy / _yx
"""
import numpy as np

X_TO_Y, Y_TO_Z, Z_TO_Y, Y_TO_X = 0, 1, 2, 3


def distribute(n, p):
    """1-based starts, ends and sizes of n points over p ranks."""
    size1 = n // p
    nu = n - size1 * p
    nl = p - nu
    st, en, sz = [0] * p, [0] * p, [0] * p
    st[0], sz[0], en[0] = 1, size1, size1
    for i in range(1, nl):
        st[i] = st[i - 1] + size1
        sz[i] = size1
        en[i] = en[i - 1] + size1
    size1 += 1
    for i in range(nl, p):
        st[i] = en[i - 1] + 1
        sz[i] = size1
        en[i] = en[i - 1] + size1
    return st, en, sz


def _partition(n, pdim, p_row, p_col, coord):
    st, en, sz = [0] * 3, [0] * 3, [0] * 3
    for i in range(3):
        if pdim[i] == 1:
            st[i], en[i], sz[i] = 1, n[i], n[i]
        else:
            p, c = (p_row, coord[0]) if pdim[i] == 2 else (p_col, coord[1])
            s, e, z = distribute(n[i], p)
            st[i], en[i], sz[i] = s[c], e[c], z[c]
    return st, en, sz


def pencil_info(nx, ny, nz, p_row, p_col, rank):
    """xst/xen/xsz, yst/..., zst/... of `rank` (row-major on the grid)."""
    coord = (rank // p_col, rank % p_col)
    n = (nx, ny, nz)
    out = {"coord": coord}
    for name, pdim in (("x", (1, 2, 3)), ("y", (2, 1, 3)), ("z", (2, 3, 1))):
        st, en, sz = _partition(n, pdim, p_row, p_col, coord)
        out[name + "st"], out[name + "en"], out[name + "sz"] = st, en, sz
    return out


def counts(nx, ny, nz, p_row, p_col, rank, kind):
    """(send_dist, send_cnts, send_disp, recv_dist, recv_cnts, recv_disp) of
    one transpose direction, per peer of the row / column communicator."""
    info = pencil_info(nx, ny, nz, p_row, p_col, rank)
    xsz, ysz, zsz = info["xsz"], info["ysz"], info["zsz"]
    col = kind in (X_TO_Y, Y_TO_X)
    p = p_row if col else p_col
    if col:
        d1, d2 = distribute(nx, p)[2], distribute(ny, p)[2]  # x1dist, y1dist
        c1 = [d1[i] * xsz[1] * xsz[2] for i in range(p)]    # x1cnts
        c2 = [ysz[0] * d2[i] * ysz[2] for i in range(p)]    # y1cnts
    else:
        d1, d2 = distribute(ny, p)[2], distribute(nz, p)[2]  # y2dist, z2dist
        c1 = [ysz[0] * d1[i] * ysz[2] for i in range(p)]    # y2cnts
        c2 = [zsz[0] * zsz[1] * d2[i] for i in range(p)]    # z2cnts
    fwd = kind in (X_TO_Y, Y_TO_Z)
    sd, rd, sc, rc = (d1, d2, c1, c2) if fwd else (d2, d1, c2, c1)

    def disp(c):
        return [int(v) for v in np.concatenate([[0], np.cumsum(c)[:-1]])]

    return sd, sc, disp(sc), rd, rc, disp(rc)


# the split axis of each pack / unpack (Fortran dimension: 0 x, 1 y, 2 z)
SPLIT = {X_TO_Y: (0, 1), Y_TO_Z: (1, 2), Z_TO_Y: (2, 1), Y_TO_X: (1, 0)}


def _block(a, d, i1, i2):
    """Sub-array i1 <= index < i2 along Fortran dimension d of the numpy
    view (n3, n2, n1)."""
    sl = [slice(None)] * 3
    sl[2 - d] = slice(i1, i2)
    return a[tuple(sl)]


def mem_split(kind, a, dist, disp, size):
    """Send buffer of `size` elements: block m (widths `dist` along the
    kind's send dimension) in Fortran order at displacement disp[m]."""
    d = SPLIT[kind][0]
    out = np.zeros(size, dtype=a.dtype)
    i1 = 0
    for m, w in enumerate(dist):
        blk = _block(a, d, i1, i1 + w)
        out[disp[m]: disp[m] + blk.size] = blk.ravel()
        i1 += w
    return out


def mem_merge(kind, buf, shape, dist, disp):
    """Destination pencil (numpy view `shape`) from the received blocks."""
    d = SPLIT[kind][1]
    out = np.empty(shape, dtype=buf.dtype)
    i1 = 0
    for m, w in enumerate(dist):
        blk = _block(out, d, i1, i1 + w)
        blk[...] = buf[disp[m]: disp[m] + blk.size].reshape(blk.shape)
        i1 += w
    return out
