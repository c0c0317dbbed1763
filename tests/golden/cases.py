"""Golden cases: scenes and views whose reference outputs are committed.

Shared by make_golden.py (which renders them with the reference, compiled
headless from its own sources) and by the tests (which rebuild the same
inputs and compare the oracle restatement and the GPU path against them).
All golden scenes use the Phong exponent 32, the reference's constant.
"""
from __future__ import annotations

import functools
import math

import numpy as np

from swegl_gb300 import abi
from swegl_gb300 import scenes as S

FULL = "full"      # per-pixel arrays stored
DIGEST = "digest"  # SHA-256 of the arrays stored


@functools.lru_cache(maxsize=None)
def scene(key: str) -> S.Scene:
    if key == "cube":
        return S.cube_scene()
    if key == "mixed":
        return S.mixed_scene()
    if key == "spheres20":
        return S.spheres_scene(n_spheres=20, tex_size=256, shininess=32)
    if key == "spheres200":
        return S.spheres_scene(shininess=32)
    if key == "grid":
        return S.grid_scene()
    if key == "glass":
        return S.glass_scene()
    raise KeyError(key)


def _tangent_view(sc: S.Scene, sphere: int, w: int = 320, h: int = 240) -> S.View:
    c = np.asarray(sc.node_translation[sphere], np.float64)
    prim = [p for p in sc.primitives if p[0] == sphere][0]
    v = np.asarray(sc.positions[prim[3]], np.float64)
    r = math.sqrt(float(v[0]) ** 2 + float(v[1]) ** 2 + float(v[2]) ** 2)
    pos = c + np.array([0.0, 0.0, r * 1.02])
    m, cp = S.look_at(pos, pos + np.array([1.0, -0.3, -0.2]))
    return S.view_for(w, h, m, cp)


def _look(pos, target, w, h):
    m, cp = S.look_at(pos, target)
    return S.view_for(w, h, m, cp)


def cases() -> dict:
    """name -> dict(scene=key, views=[View], shared=(w, h) or None, kinds=(...), store=FULL|DIGEST)"""
    out = {}
    out["cube_640x480"] = dict(scene="cube", views=lambda: [S.cube_view(640, 480)], kinds=(0, 1, 2, 3, 4), store=FULL)
    out["cube_close_320x240"] = dict(scene="cube", views=lambda: [_look((0.3, 0.2, 1.2), (0, 0, 0), 320, 240)],
                                     kinds=(0, 1, 2), store=FULL)
    out["cube_inside_320x240"] = dict(scene="cube", views=lambda: [_look((0.2, 0.1, 0.9), (0, 0, 0), 320, 240)],
                                      kinds=(0, 1, 2), store=FULL)
    out["mixed_320x240"] = dict(scene="mixed", views=lambda: [_look((0.5, 0.8, 4.5), (0, 0, 0), 320, 240)],
                                kinds=(0, 1, 2, 3, 4), store=FULL)
    out["spheres20_480x270"] = dict(scene="spheres20", views=lambda: [S.spheres_view(480, 270)],
                                    kinds=(0, 1, 2, 3, 4), store=FULL)
    out["grid_clip_a_320x240"] = dict(scene="grid", views=lambda: [_look((0.1, -0.3, 0.05), (0.0, -0.45, -3.0), 320, 240)],
                                      kinds=(0, 1, 2), store=FULL)
    out["grid_clip_b_320x240"] = dict(scene="grid", views=lambda: [_look((0.13, -0.47, 0.21), (2.0, -0.5, -3.0), 320, 240)],
                                      kinds=(0, 1, 2), store=FULL)
    for sp in (0, 5, 7):
        out[f"spheres_tangent{sp}_320x240"] = dict(scene="spheres200",
                                                   views=(lambda sp=sp: [_tangent_view(scene("spheres200"), sp)]),
                                                   kinds=(0, 1, 2), store=FULL)

    def shared_views():
        vs = S.batch_views(4, seed=5, min_wh=(320, 240), max_wh=(320, 240))
        for i, v in enumerate(vs):
            v.x, v.y = (i % 2) * 320, (i // 2) * 240
        return vs

    # the other pixel shaders of the reference (SGL_SHADER_* 1..8), on the
    # mixed scene (textures, untextured, fans / strips / lists, double sided)
    # and on the cube
    def shaded(view_fn, mode):
        def views():
            vs = view_fn()
            for v in vs:
                v.shader = mode
            return vs
        return views

    for mode in range(1, 9):
        name = abi.SHADERS[mode]
        out[f"mixed_{name}_320x240"] = dict(scene="mixed", views=shaded(lambda: [_look((0.5, 0.8, 4.5), (0, 0, 0), 320, 240)], mode),
                                           kinds=(0,), store=FULL)
        out[f"cube_{name}_320x240"] = dict(scene="cube", views=shaded(lambda: [_look((0.3, 0.2, 1.2), (0, 0, 0), 320, 240)], mode),
                                          kinds=(0,), store=FULL)

    # transparency layers (viewport_t's transparency_layer_count) on the glass scene
    def glass(w=320, h=240, pos=(0.3, 0.4, 3.2), target=(0.0, 0.0, -0.5), **kw):
        def views():
            v = _look(pos, target, w, h)
            for k, x in kw.items():
                setattr(v, k, x)
            return [v]
        return views

    out["glass_320x240"] = dict(scene="glass", views=glass(), kinds=(0,), store=FULL)
    for layers, mode in ((1, 0), (2, 0), (3, 0), (8, 0), (2, 4), (3, 6), (1, 8)):
        out[f"glass_l{layers}_{abi.SHADERS[mode]}_320x240"] = dict(
            scene="glass", views=glass(layers=layers, shader=mode), kinds=(0,), store=FULL)
    out["glass_close_l4_320x240"] = dict(scene="glass", views=glass(pos=(0.1, 0.0, 0.3), target=(0.2, 0.1, -2.0),
                                                                   layers=4), kinds=(0,), store=FULL)
    # a view off the surface's corner: the layer resolve reads surface rows
    # 0..h-1 and writes rows y..y+h-1, columns 0..w-1 (viewport.cpp:53-79,
    # post_shaders.hpp:22-31)
    out["glass_offset_l3_320x240"] = dict(scene="glass", views=glass(layers=3, x=40, y=30), shared=(400, 300),
                                          kinds=(0,), store=FULL)

    def glass_pair():
        a = glass(200, 150, layers=2)()[0]
        b = glass(200, 150, pos=(-0.5, 0.2, 2.5), layers=4, x=200, y=150)()[0]
        return [a, b]

    out["glass_pair_2x200x150"] = dict(scene="glass", views=glass_pair, shared=(400, 300), kinds=(0,), store=FULL)
    out["shared_4x320x240"] = dict(scene="spheres200", views=shared_views, shared=(640, 480), kinds=(0, 1), store=FULL)
    out["spheres_1920x1080"] = dict(scene="spheres200", views=lambda: [S.spheres_view(1920, 1080)], kinds=(0, 1, 2),
                                    store=DIGEST)
    out["cube_3840x2160"] = dict(scene="cube", views=lambda: [S.cube_view(3840, 2160)], kinds=(0, 1), store=DIGEST)
    out["spheres_3840x2160"] = dict(scene="spheres200", views=lambda: [S.spheres_view(3840, 2160)], kinds=(0,),
                                    store=DIGEST)
    return out


def sha(a: np.ndarray) -> str:
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
