"""The drop-in C++ API (include/swegl_gb300/swegl.hpp): swegl code built
against it renders on the GPU with the reference's results.

CPU: the header compiles with the reference's usage.  GPU: a program that
builds scene_t / viewport_t and calls swegl::render(scene, vp0, vp1) on one
surface matches the oracle (depth bit-exact, colour within 2 LSB)."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "dropin", "dropin_render.cpp")
sys.path.insert(0, os.path.join(ROOT, "tests", "dropin"))


def compile_dropin(out_dir, syntax_only=False):
    from swegl_gb300 import build

    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC]
    if syntax_only:
        cmd.append("-fsyntax-only")
    else:
        lib = build.build()
        exe = os.path.join(out_dir, "dropin_render")
        cmd += ["-o", exe, "-L", os.path.dirname(lib), "-lsgl", "-Wl,-rpath," + os.path.dirname(lib)]
    subprocess.run(cmd, check=True)
    return None if syntax_only else exe


def test_header_compiles(tmp_path):
    compile_dropin(str(tmp_path), syntax_only=True)


@pytest.mark.gpu
@pytest.mark.parametrize("scene,layers", [("mixed", (0, 0)), ("glass", (3, 0))])
def test_dropin_render_matches_oracle(tmp_path, scene, layers):
    import cases as G
    import oracle
    from dump import write_dump

    from swegl_gb300 import scenes as S

    exe = compile_dropin(str(tmp_path))
    sc = G.scene(scene)
    views = []
    for i, pos in enumerate([(0.5, 0.8, 4.5), (-2.0, 1.0, 3.5)]):
        m, c = S.look_at(pos, (0, 0, 0))
        v = S.view_for(320, 240, m, c)
        v.x = 320 * i
        v.shader = (0, 3)[i]  # Phong + bilinear; flat light + nearest texture
        v.layers = layers[i]  # viewport_t's transparency_layer_count
        views.append(v)
    dump = os.path.join(str(tmp_path), "scene.bin")
    out = os.path.join(str(tmp_path), "out.bin")
    write_dump(dump, sc, views, (640, 240))
    subprocess.run([exe, dump, out], check=True)
    raw = np.fromfile(out, np.uint32)
    surface = raw[:640 * 240].reshape(240, 640)
    ref = oracle.render(sc, views, shared_surface=(640, 240))
    d = np.abs(surface.view(np.uint8).astype(np.int16) - ref.pixels.view(np.uint8).astype(np.int16))
    assert int(d.max()) <= 2
    zs = raw[640 * 240:].view(np.float32)
    for i, v in enumerate(views):
        z = zs[i * v.w * v.h:(i + 1) * v.w * v.h].reshape(v.h, v.w)
        assert np.array_equal(z.view(np.uint32), ref.frames[i].zbuffer.view(np.uint32))
