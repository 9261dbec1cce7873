"""Shared pieces of the halo-update tests: the global field, each rank's
pencil, a numpy stand-in for the device box copy, and the comparison with
the oracle (oracle/halo.py) on the cells the reference defines."""
import numpy as np

from oracle import halo as H

# (grid, p_row, p_col, pencil, level, periodic)
CASES = [((9, 8, 7), 1, 1, "x", 1, (False, False, False)),
         ((9, 8, 7), 1, 1, "y", 2, (True, True, True)),
         ((9, 8, 7), 2, 1, "x", 1, (False, True, False)),
         ((9, 8, 7), 1, 2, "z", 1, (True, True, False)),
         ((10, 9, 8), 2, 2, "y", 2, (True, False, True)),
         ((10, 9, 8), 2, 2, "x", 1, (False, False, False)),
         ((10, 9, 8), 2, 2, "z", 2, (True, True, True)),
         ((12, 9, 8), 1, 4, "x", 1, (False, True, True))]


def global_field(grid, dtype=np.float64):
    nx, ny, nz = grid
    m = np.arange(nx * ny * nz, dtype=np.float64).reshape(nz, ny, nx) + 1
    return m.astype(dtype)


def piece(g, d, pencil):
    st, en = getattr(d, pencil + "st"), getattr(d, pencil + "en")
    return np.ascontiguousarray(g[st[2] - 1:en[2], st[1] - 1:en[1], st[0] - 1:en[0]])


def np_copy(src, src_off, dst, dst_off, box):
    """numpy stand-in of gbfft_box_copy on CPU tensors."""
    s, t = src.numpy(), dst.numpy()
    sv = s[src_off[2]:src_off[2] + box[2], src_off[1]:src_off[1] + box[1], src_off[0]:src_off[0] + box[0]]
    t[dst_off[2]:dst_off[2] + box[2], dst_off[1]:dst_off[1] + box[1], dst_off[0]:dst_off[0] + box[0]] = sv
    return dst


def oracle(g, grid, p_row, p_col, pencil, level, periodic):
    import gbfft
    nx, ny, nz = grid
    ds = [gbfft.Decomp(nx, ny, nz, p_row, p_col, r) for r in range(p_row * p_col)]
    arrs, masks = H.update_all([piece(g, d, pencil) for d in ds], pencil, level, p_row, p_col, periodic)
    return ds, arrs, masks
