"""Oracle (test infrastructure only) of the halo-cell update: a numpy
emulation of update_halo for every rank of a p_row x p_col grid
(src/halo_common.f90, src/halo.f90:230-309 halo extents,
src/halo_exchange_{x,y,z}_body.f90 the exchanges), message passing
included.

Each rank copies its pencil into an array with `level` halo cells on the
pencil's two distributed axes, then fills the halos in two phases (X pencil:
y then z; Y pencil: x then z; Z pencil: x then y), each phase exchanging
slabs of `level` planes that span the whole halo-extended array in the other
two axes with the rank's neighbours along one dimension of the Cartesian
grid.  Within a phase every rank posts, in this order: a receive from its
minus neighbour (tag = own coordinate) into its low halo, a receive from its
plus neighbour (tag = coordinate + 1, or 0 for the last rank of a periodic
dimension) into its high halo, a send of its first `level` interior planes to
the minus neighbour, a send of its last `level` interior planes to the plus
neighbour.  Neighbours across a non-periodic edge are MPI_PROC_NULL: nothing
moves and that halo stays unset.  Messages match as MPI matches them: a
receive takes the earliest unmatched send from its source with its tag --
which, on a periodic dimension of one rank (the rank its own neighbour, both
tags 0), fills the low halo with the rank's own first interior planes and the
high halo with its last ones.

Arrays follow the numpy view (n3, n2, n1) of a Fortran array.  `update_all`
returns, per rank, the halo-extended array and a boolean mask of the cells
the reference defines.
"""
import numpy as np

# pencil -> (distributed axes in phase order, Fortran dims 0 x 1 y 2 z)
PHASES = {"x": (1, 2), "y": (0, 2), "z": (0, 1)}


def _view(arr, box_off, box):
    """numpy view of the Fortran box (offsets and widths per Fortran dim)."""
    sl = [slice(None)] * 3
    for d in range(3):
        sl[2 - d] = slice(box_off[d], box_off[d] + box[d])
    return arr[tuple(sl)]


def extended_dims(pencil, sizes, level):
    e = list(sizes)
    for a in PHASES[pencil]:
        e[a] += 2 * level
    return e


def update_all(pieces, pencil, level, p_row, p_col, periodic):
    """pieces[rank]: the rank's pencil (numpy view); periodic = (px, py, pz).
    Returns (arrays, masks) per rank."""
    nranks = p_row * p_col
    dims = (p_row, p_col)
    arrs, masks = [], []
    for r in range(nranks):
        sizes = list(pieces[r].shape[::-1])
        e = extended_dims(pencil, sizes, level)
        a = np.zeros(e[::-1], dtype=pieces[r].dtype)
        m = np.zeros(e[::-1], dtype=bool)
        off = [level if d in PHASES[pencil] else 0 for d in range(3)]
        _view(a, off, sizes)[...] = pieces[r]
        _view(m, off, sizes)[...] = True
        arrs.append(a)
        masks.append(m)
    for phase, axis in enumerate(PHASES[pencil]):
        cdim = phase  # Cartesian dimension of this phase: 0 (p_row), 1 (p_col)
        per = periodic[axis]
        sends, recvs = {r: [] for r in range(nranks)}, {r: [] for r in range(nranks)}
        for r in range(nranks):
            c = [r // p_col, r % p_col]
            me = c[cdim]
            sizes = list(pieces[r].shape[::-1])
            s = sizes[axis]
            e = list(arrs[r].shape[::-1])

            def nb(shift):
                cc = list(c)
                v = me + shift
                if v < 0 or v >= dims[cdim]:
                    if not per:
                        return None
                    v %= dims[cdim]
                cc[cdim] = v
                return cc[0] * p_col + cc[1]

            minus, plus = nb(-1), nb(+1)
            tag_minus = me
            tag_plus = 0 if (me == dims[cdim] - 1 and per) else me + 1

            def box_at(pos):
                o = [0, 0, 0]
                w = list(e)
                o[axis] = pos
                w[axis] = level
                return o, w

            # posting order of the reference: recv minus, recv plus, send minus, send plus
            if minus is not None:
                recvs[r].append((minus, tag_minus, box_at(0)))
            if plus is not None:
                recvs[r].append((plus, tag_plus, box_at(s + level)))
            if minus is not None:
                o, w = box_at(level)
                sends[r].append([minus, tag_minus, _view(arrs[r], o, w).copy(), _view(masks[r], o, w).copy(), False])
            if plus is not None:
                o, w = box_at(s)
                sends[r].append([plus, tag_plus, _view(arrs[r], o, w).copy(), _view(masks[r], o, w).copy(), False])
        for r in range(nranks):
            for src, tag, (o, w) in recvs[r]:
                for msg in sends[src]:
                    if msg[0] == r and msg[1] == tag and not msg[4]:
                        msg[4] = True
                        _view(arrs[r], o, w)[...] = msg[2]
                        _view(masks[r], o, w)[...] = msg[3]
                        break
                else:
                    raise AssertionError("unmatched receive")
    return arrs, masks
