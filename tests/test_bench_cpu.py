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


def test_frame_workloads_and_roofline():
    """The frame workloads' algorithmic bytes (32 B per vertex, 4 B per index
    and texel, 8 B per pixel; 12 B more per pixel with depth of field) and the
    roofline line built from them against the measured peak."""
    from swegl_gb300 import scenes as S

    sc = S.cube_scene()
    base = 32 * len(sc.positions) + 4 * len(sc.indices) + sum(4 * int(t.size) for t in sc.textures)
    assert bench.frame_alg_bytes(sc, 640, 480) == base + 8 * 640 * 480
    assert bench.frame_alg_bytes(sc, 640, 480, dof=True) == base + 20 * 640 * 480
    assert set(bench.FRAMES) == {"frame", "dof"}
    assert bench.FRAMES["dof"][1] == (3840, 2160) and bench.FRAMES["dof"][2]
    for kind in bench.FRAMES:
        rl = bench.roofline_of({"kind": kind, "alg_bytes": 10**8, "frame_ms": 0.5})
        assert rl["bound"] == "hbm" and rl["unit"] == "GB/s"
        assert abs(rl["achieved"] - 200.0) < 1e-6  # 1e8 B in 0.5 ms
        assert abs(rl["frac"] - round(200.0 / rl["peak"], 4)) < 1e-9
        assert ("depth of field" in rl["unit_of_work"]) == (kind == "dof")
        assert rl["traffic"] and rl["traffic"] > 10**8  # from the committed ncu summary
