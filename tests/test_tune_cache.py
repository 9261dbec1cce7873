"""CPU: the committed tuning cache is well formed.

Engines read 2decomp-fft_gb300/tune_cache.txt at creation and ignore keys
they do not know, so a mistyped key would silently fall back to the built-in
choice.  Every line must name a shape once, with known keys and values in
their ranges."""
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(os.path.dirname(HERE), "2decomp-fft_gb300", "tune_cache.txt")
PASSES = ("r2c", "c2r", "c2c_x", "c2c_y", "c2c_z", "xy_fused")


def allowed(key, v):
    if key == "fuse":
        return v in (0, 1)
    if key == "pad":
        return v in (0, 1, 2)
    if key in ("flat", "tma"):
        return v in (0, 1)
    if key in ("e_x", "e_y", "e_z"):
        return v in (2, 4, 8, 9, 16, 20, 24, 30, 32)
    m = re.fullmatch(r"(cl_|cls_)?(\w+)", key)
    if not m or m.group(2) not in PASSES:
        return False
    prefix = m.group(1) or ""
    if prefix == "":
        return v in (1, 2, 4, 8, 16, 32)  # lines per CTA
    if prefix == "cl_":
        return v in (2, 4, 8)
    return v in (0, 1)  # cls_


def test_cache_lines_parse_with_known_keys():
    seen = set()
    lines = [l for l in open(CACHE).read().splitlines() if l.strip() and not l.startswith("#")]
    assert lines
    for line in lines:
        parts = line.split()
        prec, fmt, nx, ny, nz = (int(v) for v in parts[:5])
        assert prec in (4, 8) and fmt in (1, 3) and min(nx, ny, nz) > 0, line
        assert (prec, fmt, nx, ny, nz) not in seen, line
        seen.add((prec, fmt, nx, ny, nz))
        for kv in parts[5:]:
            key, _, val = kv.partition("=")
            assert val.lstrip("-").isdigit(), kv
            assert allowed(key, int(val)), kv


def test_cache_covers_the_benchmark_grids():
    shapes = set()
    for l in open(CACHE).read().splitlines():
        if l.strip() and not l.startswith("#"):
            shapes.add(tuple(int(v) for v in l.split()[:5]))
    assert (4, 1, 1024, 1024, 512) in shapes and (4, 3, 1024, 1024, 512) in shapes
