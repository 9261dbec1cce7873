"""CPU: the halo-update oracle (oracle/halo.py, an emulation of the
reference's update_halo with its message matching) against the definition
of a halo: across interior boundaries and periodic dimensions of two or more
ranks every halo cell holds the global field at that cell's (wrapped)
global position; across non-periodic edges the halo is unset; on a periodic
dimension of one rank the reference's two same-tag messages leave the
adjacent interior planes in each halo."""
import numpy as np
import pytest

from halo_cases import CASES, global_field, oracle
from oracle import halo as H


@pytest.mark.parametrize("case", CASES)
def test_oracle_halo_cells(case):
    grid, p_row, p_col, pencil, level, periodic = case
    g = global_field(grid)
    ds, arrs, masks = oracle(g, grid, p_row, p_col, pencil, level, periodic)
    dims = {0: p_row, 1: p_col}
    axes = H.PHASES[pencil]
    for d, a, m in zip(ds, arrs, masks):
        st = getattr(d, pencil + "st")
        sz = getattr(d, pencil + "sz")
        e = a.shape[::-1]
        gpos, defined = [], np.ones(a.shape, dtype=bool)
        for ax in range(3):
            shape = [1, 1, 1]
            shape[2 - ax] = e[ax]
            idx = np.arange(e[ax]).reshape(shape)
            if ax in axes:
                p = st[ax] - 1 + idx - level  # global 0-based position
                n = grid[ax]
                out = (p < 0) | (p >= n)
                if not periodic[ax]:
                    defined &= ~np.broadcast_to(out, a.shape)
                    p = np.clip(p, 0, n - 1)
                elif dims[axes.index(ax)] == 1:
                    # one rank: the adjacent interior plane on the same side
                    p = np.where(p < 0, p + level, np.where(p >= n, p - level, p))
                else:
                    p = p % n
                gpos.append(p)
            else:
                gpos.append(idx)
        expect = g[gpos[2], gpos[1], gpos[0]]
        assert np.array_equal(m, defined)
        assert np.array_equal(a[defined], np.broadcast_to(expect, a.shape)[defined])
        assert a.shape[::-1] == tuple(sz[ax] + (2 * level if ax in axes else 0) for ax in range(3))
