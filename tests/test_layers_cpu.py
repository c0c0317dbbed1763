"""Transparency layers, CPU checks of the two facts the GPU resolve relies on.

1. blend (src/render/colors.cpp:39-57) computes
   (uint8)(back * ((256 - a) / 256.0) + front * (a / 256.0)); both products
   are exact multiples of 1/256 below 256, so it equals the integer
   (back * (256 - a) + front * a) >> 8 the kernels use.  Checked for every
   alpha and channel pair.
2. The per-pixel insertion of renderer.cpp:494-550, run fragment by fragment
   in draw order, ends in the state that the order-free rule of the GPU
   resolve (k_layers in raster.cu) computes from the same fragments:
   the first-drawn nearest opaque fragment wins the screen, and the layers
   hold the `layers` nearest transparent fragments strictly in front of it
   (equal depths: later drawn is nearer), farthest in layer 0.  Checked on
   random fragment sequences with many depth ties and overflowing layers."""
import numpy as np

MAX_Z = float(np.frombuffer(np.uint32(0x7F7F7F7F).tobytes(), np.float32)[0])


def test_blend_double_formula_equals_integer_formula():
    a = np.arange(1, 255, dtype=np.int64)[:, None, None]
    b = np.arange(256, dtype=np.int64)[None, :, None]
    f = np.arange(256, dtype=np.int64)[None, None, :]
    dbl = np.trunc(b * ((256 - a) / 256.0) + f * (a / 256.0)).astype(np.int64)
    assert np.array_equal(dbl, (b * (256 - a) + f * a) >> 8)


def insert_in_draw_order(frags, n):
    """renderer.cpp:494-550 for one pixel: frags = [(z, colour_id, opaque)]."""
    zb, video = MAX_Z, None
    lz, lc = [MAX_Z] * n, [None] * n
    for z, c, opaque in frags:
        if z >= zb:
            continue
        li = 0
        while li < n and not (lz[li] == MAX_Z or lz[li] < z):
            li += 1
        if opaque:
            video, zb = c, z
            kept = list(zip(lz[li:], lc[li:]))
            lz = [k[0] for k in kept] + [MAX_Z] * li
            lc = [k[1] for k in kept] + [None] * li
        elif lz[n - 1] != MAX_Z:
            while li > 0:
                li -= 1
                lz[li], z = z, lz[li]
                lc[li], c = c, lc[li]
        else:
            while li < n:
                lz[li], z = z, lz[li]
                lc[li], c = c, lc[li]
                li += 1
                if z == MAX_Z:
                    break
    return video, zb, [c for z, c in zip(lz, lc) if z != MAX_Z]


def resolve_order_free(frags, n):
    """The rule of k_layers: fragments taken in (depth, draw order)."""
    order = sorted(range(len(frags)), key=lambda i: (frags[i][0], i))
    kept = []  # (z, slot, colour), nearest first: (z asc, slot desc)
    for i in order:
        z, c, opaque = frags[i]
        if opaque:
            kept = [k for k in kept if k[0] < z]
            return c, z, [k[2] for k in reversed(kept)]
        kept.append((z, i, c))
        kept.sort(key=lambda k: (k[0], -k[1]))
        kept = kept[:n]
    return None, MAX_Z, [k[2] for k in reversed(kept)]


def test_draw_order_insertion_equals_order_free_resolve():
    rng = np.random.default_rng(17)
    for trial in range(4000):
        n = int(rng.integers(1, 6))
        m = int(rng.integers(0, 14))
        zs = rng.integers(1, 7, size=m).astype(np.float32)  # few depths: many ties
        opaque = rng.random(m) < rng.choice([0.0, 0.2, 0.5])
        frags = [(float(zs[i]), i, bool(opaque[i])) for i in range(m)]
        assert insert_in_draw_order(frags, n) == resolve_order_free(frags, n), (trial, n, frags)
