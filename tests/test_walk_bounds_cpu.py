"""The compaction's column-sliver test is safe: a float32 emulation of
fill_triangle_2's edge set-up and row stepping (renderer.cpp:361-460, the
arithmetic of walk_sub in swegl_gb300/csrc/raster.cu) finds no row with a
pixel in any triangle the test removes.  The test (k_compact): with rows =
ceil(max y) - ceil(min y) and eps = (rows + 32) * 2^-23 * (max |x| + 1), a
triangle covers no pixel column when ceil(min x - eps) == ceil(max x + eps).

Triangles are built with their x range within 1e-10 .. 1e-4 (relative) of a
column boundary, 1 .. 500 rows and |x| up to 3e4; with eps = 0 the same
emulation does find rows with pixels, so the margin is what makes it safe."""
import math

import numpy as np

f = np.float32


def _ceil(x):
    return f(math.ceil(x)) if math.isfinite(x) else x


def column_sliver(xs, ys, margin=True):
    lo_y, hi_y = min(ys), max(ys)
    if math.ceil(lo_y) == math.ceil(hi_y):
        return None  # a row sliver: removed before this test
    mx = f(max(abs(x) for x in xs))
    rows = f(_ceil(hi_y) - _ceil(lo_y))
    eps = f(f(f(rows + f(32.0)) * f(2.0 ** -23)) * f(mx + f(1.0))) if margin else f(0.0)
    return _ceil(f(min(xs) - eps)) == _ceil(f(max(xs) + eps))


def walk_spans(verts, vy=-(1 << 30)):
    """[ceil(xl), ceil(xr)) of every row from row vy on (the viewport's top),
    edges displaced to the first row and stepped as fill_triangle_2 does."""
    (v0x, v0y), (v1x, v1y), (v2x, v2y) = sorted(verts, key=lambda p: p[1])
    y0, y1, y2 = math.ceil(v0y), math.ceil(v1y), math.ceil(v2y)
    out = []
    if y0 == y2:
        return out
    ys = max(y0, vy)
    lr = f(f(v2x - v0x) / f(v2y - v0y))
    lm = f(f(ys) - v0y)
    lx = f(v0x + f(lr * lm))
    if y1 >= vy:
        ur = f(f(v1x - v0x) / f(v1y - v0y))
        ux = f(v0x + f(ur * lm))
        for _ in range(ys, y1):
            out.append((math.ceil(min(lx, ux)), math.ceil(max(lx, ux))))
            lx, ux = f(lx + lr), f(ux + ur)
    y = max(y1, vy)
    dr = f(f(v2x - v1x) / f(v2y - v1y))
    dx = f(v1x + f(dr * f(f(y) - v1y)))
    for _ in range(y, y2):
        out.append((math.ceil(min(lx, dx)), math.ceil(max(lx, dx))))
        lx, dx = f(lx + lr), f(dx + dr)
    return out


def _triangles(n, seed):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        scale = 10.0 ** rng.uniform(-1, 4.5)
        col = math.floor(rng.uniform(-scale, scale))
        gap = 10.0 ** rng.uniform(-7, -1) * max(1.0, abs(col)) * 1e-3
        if rng.uniform() < 0.5:  # pushed against the boundary above
            hi = col - gap
            lo = hi - rng.uniform(0, 1 - 1e-6) * (hi - (col - 1))
        else:                     # ... or the one below
            lo = (col - 1) + gap
            hi = lo + rng.uniform(0, 1) * (col - lo)
        lo, hi = min(lo, hi), max(lo, hi)
        rows = int(10 ** rng.uniform(0, 2.7))
        y0 = rng.uniform(-50, 50)
        ys = [f(y0), f(y0 + rng.uniform(0, rows)), f(y0 + rows + rng.uniform(0, 1))]
        xs = [f(rng.uniform(lo, hi)) for _ in range(3)]
        xs[int(rng.integers(0, 3))] = f(lo if rng.uniform() < 0.5 else hi)
        yield xs, ys


def test_column_slivers_cover_no_pixel():
    removed = 0
    for xs, ys in _triangles(20000, 1):
        if column_sliver(xs, ys):
            removed += 1
            # the whole triangle, and its rows below a viewport top inside it
            top = math.ceil(min(ys)) + int((max(ys) - min(ys)) * 0.6)
            for vy in (-(1 << 30), top):
                assert all(a >= b for (a, b) in walk_spans(list(zip(xs, ys)), vy)), (xs, ys, vy)
    assert removed > 5000


def test_without_the_margin_rows_get_pixels():
    """The emulation is sharp enough to see the rounding the margin covers."""
    hits = 0
    for xs, ys in _triangles(20000, 2):
        if column_sliver(xs, ys, margin=False):
            hits += any(a < b for (a, b) in walk_spans(list(zip(xs, ys))))
    assert hits > 0
