"""bench.py helpers that need no GPU: the parity summary it reports beside
the CPU baseline (depth bits and the per-pixel |dRGB| histogram)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _Frame:
    def __init__(self, pixels, zbuffer):
        self.pixels, self.zbuffer = pixels, zbuffer


def test_parity_histogram_and_depth():
    rng = np.random.default_rng(1)
    pix = rng.integers(0, 2**32, (6, 5), dtype=np.uint64).astype(np.uint32)
    z = rng.random((6, 5), dtype=np.float32)
    other = pix.copy()
    b = other.view(np.uint8).reshape(6, 5, 4)
    b[0, 0, 0] ^= 1                      # 1 LSB (low bit) in blue
    b[1, 1, 2] = (int(b[1, 1, 2]) + 2) % 256  # 2 LSB in red (or a wrap)
    p = bench.parity_of([(pix, z)], [_Frame(other, z.copy())])
    h = p["rgb_abs_diff_hist_0_1_2_3plus"]
    assert p["pixels"] == 30 and p["depth_bit_exact"]
    assert sum(h) == 30 and h[0] == 28 and h[1] == 1
    z2 = z.copy()
    z2[2, 2] = np.nextafter(z2[2, 2], np.float32(2))
    assert not bench.parity_of([(pix, z)], [_Frame(pix, z2)])["depth_bit_exact"]
