"""glTF scenes on the GPU: a file loaded by the library (sgl_gltf_load),
uploaded and rendered, and re-rendered after scene_t::animate
(sgl_gltf_animate + sgl_scene_set_nodes), against the oracle restatement of
the reference's loader and renderer on the same file; and the same through
the drop-in C++ API (swegl::load_scene, scene_t::animate, swegl::render).

Bar: depth bit-exact; colour within 2 LSB per channel, within 1 LSB on
>= 99.9% of pixels."""
import os
import subprocess
import sys

import numpy as np
import pytest

import gltf_files as GF
import oracle
from oracle import gltf_oracle as GO
from swegl_gb300 import scenes as S

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def colour_check(got, exp, where=""):
    d = np.abs(got.view(np.uint8).astype(np.int16) - exp.view(np.uint8).astype(np.int16))
    per_px = d.reshape(-1, 4).max(axis=1)
    assert int(d.max()) <= 2, f"{where}: max |dRGB| {int(d.max())}"
    assert float((per_px <= 1).mean()) >= 0.999, f"{where}: histogram {np.bincount(per_px)[:3].tolist()}"


def light(scene):
    scene.ambient = 0.15
    scene.sun_intensity = 0.6
    scene.sun_direction = S.normalize_f32(np.array([-0.5, -1.0, -0.7]))
    scene.point_lights = [(0.5, 1.5, 2.5, 2.0)]
    return scene


def views():
    out = []
    for i, (pos, w, h) in enumerate([((0.4, 0.6, 3.8), 320, 240), ((-2.5, 1.0, 2.0), 200, 150)]):
        m, c = S.look_at(pos, (0.0, 0.0, -0.3))
        out.append(S.view_for(w, h, m, c))
    out[1].layers = 2  # a second view with transparency layers
    return out


@pytest.fixture(scope="module")
def renderer():
    from swegl_gb300.runtime import Renderer

    r = Renderer(0)
    yield r
    r.close()


@pytest.mark.parametrize("glb", [True, False])
def test_loaded_and_animated_scene_matches_oracle(renderer, tmp_path, glb):
    from swegl_gb300.gltf import GltfScene

    path = GF.build_test_scene(str(tmp_path), glb)
    g = GltfScene(path)
    ref = GO.load_scene(path, GO.decode_image)
    light(ref.scene)
    sid = renderer.upload(light(g.scene()))
    vs = views()
    for t in (None, 0.35, 1.6):
        if t is not None:
            nodes = g.animate(t)
            assert renderer.lib.sgl_scene_set_nodes(renderer.ctx, sid, nodes, len(ref.scene.node_parent)) == 0
            GO.animate(ref, t)
        frames, _ = renderer.render(sid, vs)
        exp = oracle.render(ref.scene, vs)
        for i, (f, e) in enumerate(zip(frames, exp.frames)):
            assert np.array_equal(f.zbuffer.view(np.uint32), e.zbuffer.view(np.uint32)), (t, i)
            colour_check(f.pixels, e.pixels, f"t={t} view {i}")
        assert int((frames[0].pixels != 0).sum()) > 5000  # the scene is in view
    renderer.release(sid)
    g.close()


def test_dropin_load_scene_and_animate(tmp_path):
    sys.path.insert(0, os.path.join(ROOT, "tests", "dropin"))
    from dump import write_dump
    from test_dropin import compile_dropin

    exe = compile_dropin(str(tmp_path))
    path = GF.build_test_scene(str(tmp_path), True)
    ref = GO.load_scene(path, GO.decode_image)
    light(ref.scene)
    vs = views()
    for v in vs:
        v.layers = 0
    vs[1].x = 320
    lights_only = light(S.Scene()).finalize()
    dump = os.path.join(str(tmp_path), "lights.bin")
    out = os.path.join(str(tmp_path), "out.bin")
    write_dump(dump, lights_only, vs, (520, 240))
    subprocess.run([exe, dump, out, path, "1.1"], check=True)
    GO.animate(ref, 1.1)
    raw = np.fromfile(out, np.uint32)
    surface = raw[:520 * 240].reshape(240, 520)
    exp = oracle.render(ref.scene, vs, shared_surface=(520, 240))
    colour_check(surface, exp.pixels, "drop-in glTF")
    zs = raw[520 * 240:].view(np.float32)
    off = 0
    for i, v in enumerate(vs):
        z = zs[off:off + v.w * v.h].reshape(v.h, v.w)
        off += v.w * v.h
        assert np.array_equal(z.view(np.uint32), exp.frames[i].zbuffer.view(np.uint32)), i


def test_serving_loop_with_posed_requests(renderer, tmp_path):
    """Animated serving: requests of one resident glTF scene, each with its
    own pose (sgl_gltf_animate at the request's time, passed with the
    request), mixed with unposed requests (the scene's current nodes) and a
    layered one.  Every frame equals sgl_render of a copy of the scene set
    to that pose; the shared scene's nodes are not changed."""
    from swegl_gb300.gltf import GltfScene

    path = GF.build_test_scene(str(tmp_path), True)
    g = GltfScene(path)
    scene = light(g.scene())
    from swegl_gb300 import abi

    sid = renderer.upload(scene)     # served
    check = renderer.upload(scene)   # posed one pose at a time for the expected frames
    holder = abi.SceneDescHolder(scene)
    rest = holder.nodes              # the nodes as loaded (what unposed requests render)
    n = len(scene.node_parent)
    vs = views()
    plan = [(0.35, vs[0]), (None, vs[1]), (1.6, vs[1]), (0.9, vs[0]), (None, vs[0]), (2.4, vs[1])]
    srv = renderer.server(budget_bytes=512 << 20, max_batch=4, streams=2, copy_out=True)
    subs = []
    for t, v in plan:
        nodes = g.animate(t) if t is not None else None
        pix = np.zeros((v.h, v.w), np.uint32)
        z = np.zeros((v.h, v.w), np.float32)
        subs.append((srv.submit(sid, v, pix, z, nodes=nodes), pix, z, nodes))
    for (t, v), (ticket, pix, z, nodes) in zip(plan, subs):
        assert srv.wait(ticket)["status"] == 0
        want = nodes if nodes is not None else rest
        assert renderer.lib.sgl_scene_set_nodes(renderer.ctx, check, want, n) == 0
        frames, _ = renderer.render(check, [v])
        assert np.array_equal(pix, frames[0].pixels), t
        assert np.array_equal(z.view(np.uint32), frames[0].zbuffer.view(np.uint32)), t
    srv.close()
    # the served scene still has its own nodes
    frames_a, _ = renderer.render(sid, [vs[0]])
    assert renderer.lib.sgl_scene_set_nodes(renderer.ctx, check, rest, n) == 0
    frames_b, _ = renderer.render(check, [vs[0]])
    assert np.array_equal(frames_a[0].pixels, frames_b[0].pixels)
    renderer.release(sid)
    renderer.release(check)
    g.close()
