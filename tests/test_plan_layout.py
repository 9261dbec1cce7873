"""CPU: the engine's pass plans stay inside their arrays, for every row
layout (gbfft_plan_describe: the host half of the engine, no GPU).

For r2c, c2r and c2c in both formats, FP32 and FP64, with and without
OVERWRITE, skip flags and the padded / flat layouts, each pass's lowest and
highest element on its source and destination side must lie in the array
that side names (input, output, or the work area sized for padded rows),
the passes must chain (each reads what the previous one wrote), and the
first must read the input and the last write the output."""
import itertools

import pytest

import gbfft as G


def pitch_padded(sp0, prec):
    q = 64 // (2 * prec)
    return (sp0 + q - 1) // q * q


def flat_off(u, w, pitch):
    return (u // w) * pitch + u % w


def side_extent(p, side):
    """Highest element offset touched on one side of a pass."""
    kind, n = p["kind"], p["n"]
    real_side = (kind == 1 and side == "src") or (kind == 2 and side == "dst")
    lines = p["nlines"] if kind == 0 else p["real_lines"]
    pts = n if (kind == 0 or real_side) else n // 2 + 1
    s_n, s_l, s_r = p["s_" + side + "_n"], p["s_" + side + "_l"], p["s_" + side + "_r"]
    if p["contiguous"]:
        base = (lines - 1) * s_l
    elif p["row_w"] > 0:
        assert p["nv"] == 1
        base = flat_off(lines - 1, p["row_w"], s_r)
    else:
        base = (lines - 1) + (p["nv"] - 1) * s_l
    return base + (pts - 1) * s_n, real_side


SHAPES = [(64, 48, 20), (33, 17, 12), (30, 17, 9), (1024, 8, 16), (256, 128, 9), (24, 40, 7)]


@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("prec", [4, 8])
@pytest.mark.parametrize("shape", SHAPES)
def test_passes_stay_in_their_arrays(fmt, prec, shape):
    nx, ny, nz = shape
    sp = (nx // 2 + 1, ny, nz) if fmt == 1 else (nx, ny, nz // 2 + 1)
    real = nx * ny * nz
    spec = sp[0] * sp[1] * sp[2]
    work = pitch_padded(sp[0], prec) * sp[1] * sp[2]
    full = nx * ny * nz
    for which, inplace, pad, flat in itertools.product(range(4), (False, True), (0, 1, 2), (0, 1)):
        for skip in [(False, False, False), (False, True, False), (True, False, True), (False, False, True)]:
            ps = G.plan_describe(fmt, nx, ny, nz, which, inplace=inplace, skip=skip, prec=prec, pad=pad, flat=flat)
            what = (which, inplace, pad, flat, skip)
            if which >= 2 and all(skip):
                assert ps == []
                continue
            assert ps, what
            # array sizes by buffer id, in elements of the side's type
            if which == 0:
                size = {0: ("r", real), 1: ("c", spec), 2: ("c", work)}
            elif which == 1:
                size = {0: ("c", spec), 1: ("r", real), 2: ("c", work)}
            else:
                size = {0: ("c", full), 1: ("c", full)}
            assert ps[0]["src"] == 0 and ps[-1]["dst"] == 1, what
            for a, b in zip(ps, ps[1:]):
                assert b["src"] == a["dst"], what
            for p in ps:
                for side in ("src", "dst"):
                    hi, real_side = side_extent(p, side)
                    typ, n = size[p[side]]
                    assert typ == ("r" if real_side else "c"), (what, p)
                    assert 0 <= hi < n, (what, side, hi, n, p)
                if p["row_w"] > 0:
                    assert not p["contiguous"] and p["nv"] == 1, (what, p)
            if inplace:
                assert all(p["src"] != 2 and p["dst"] != 2 for p in ps), what


def test_padded_layout_pitches():
    # 1024 x 8 x 16 FP32, PHYSICAL_IN_X: rows of 513 values, padded pitch 520
    ps = G.plan_describe(1, 1024, 8, 16, 1, prec=4, pad=1, flat=1)  # c2r
    z, y, x = ps
    assert (z["dst"], y["src"], y["dst"], x["src"]) == (2, 2, 2, 2)
    assert z["s_dst_l"] == 520 and y["s_dst_n"] == 520 and x["s_src_l"] == 520
    ps = G.plan_describe(1, 1024, 8, 16, 0, prec=4, pad=0, flat=1)  # r2c, unpadded
    assert [p["dst"] for p in ps] == [1, 1, 1]
    assert ps[2]["row_w"] == 513 and ps[2]["nlines"] == 513 * 8 and ps[2]["nv"] == 1  # flat z
    ps = G.plan_describe(1, 1024, 8, 16, 0, prec=4, pad=2, flat=1)  # pad 2: r2c in its output
    assert [p["dst"] for p in ps] == [1, 1, 1]


def test_describe_checks_its_arguments():
    with pytest.raises(G.GbfftError, match="nx"):
        G.plan_describe(1, 0, 8, 8, 0)
    with pytest.raises(G.GbfftError, match="which"):
        G.plan_describe(1, 8, 8, 8, 4)
    with pytest.raises(G.GbfftError, match="pad"):
        G.plan_describe(1, 8, 8, 8, 0, pad=3)


def side_offsets(p, side):
    """Every element offset a pass touches on one side (numpy array)."""
    import numpy as np
    kind, n = p["kind"], p["n"]
    real_side = (kind == 1 and side == "src") or (kind == 2 and side == "dst")
    lines = p["nlines"] if kind == 0 else p["real_lines"]
    pts = n if (kind == 0 or real_side) else n // 2 + 1
    s_n, s_l, s_r = p["s_" + side + "_n"], p["s_" + side + "_l"], p["s_" + side + "_r"]
    u = np.arange(lines, dtype=np.int64)
    if p["contiguous"]:
        base = u * s_l
    elif p["row_w"] > 0:
        base = (u // p["row_w"]) * s_r + u % p["row_w"]
    else:
        v = np.arange(p["nv"], dtype=np.int64)
        base = (u[:, None] + v[None, :] * s_l).ravel()
    return (base[:, None] + np.arange(pts, dtype=np.int64)[None, :] * s_n).ravel()


@pytest.mark.parametrize("fmt", [1, 3])
@pytest.mark.parametrize("shape", [(34, 12, 10), (33, 17, 9), (64, 16, 8)])
@pytest.mark.parametrize("pad", [0, 1, 2])
def test_passes_cover_their_arrays_once(fmt, shape, pad):
    import numpy as np
    nx, ny, nz = shape
    sp = (nx // 2 + 1, ny, nz) if fmt == 1 else (nx, ny, nz // 2 + 1)
    for which in range(4):
        for flat in (0, 1):
            ps = G.plan_describe(fmt, nx, ny, nz, which, prec=4, pad=pad, flat=flat)
            out_size = {0: sp[0] * sp[1] * sp[2], 1: nx * ny * nz}.get(which, nx * ny * nz)
            last = side_offsets(ps[-1], "dst")
            # the last pass writes every element of the output exactly once
            assert len(last) == out_size and len(np.unique(last)) == out_size, (which, flat)
            assert last.min() == 0 and last.max() == out_size - 1, (which, flat)
            # each pass reads exactly the elements the previous one wrote
            for a, b in zip(ps, ps[1:]):
                wa = np.unique(side_offsets(a, "dst"))
                rb = np.unique(side_offsets(b, "src"))
                assert np.array_equal(wa, rb), (which, flat, a, b)
