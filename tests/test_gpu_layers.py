"""Transparency layers on the GPU (viewport_t's transparency_layer_count,
src/render/renderer.cpp:494-550, viewport.cpp:43-86, post_shaders.hpp:22-47)
against the oracle restatement, which the golden fixtures pin to the
reference: the fragment pool growing, a surface with content before the
render, device targets, the statistics, the serving loop, and the entry
points that refuse layered views.

Bar: depth bits and winners bit-exact; colour within 2 LSB per channel
everywhere and within 1 LSB on >= 99.9% of pixels."""
import numpy as np
import pytest

import oracle
from swegl_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer():
    from swegl_gb300.runtime import Renderer

    r = Renderer(0)
    yield r
    r.close()


def colour_check(got, exp, where=""):
    d = np.abs(got.view(np.uint8).astype(np.int16) - exp.view(np.uint8).astype(np.int16))
    per_px = d.reshape(-1, 4).max(axis=1)
    assert int(d.max()) <= 2, f"{where}: max |dRGB| {int(d.max())}"
    assert float((per_px <= 1).mean()) >= 0.999, f"{where}: histogram {np.bincount(per_px)[:3].tolist()}"


def stack_scene(n_sheets: int = 12) -> S.Scene:
    """n_sheets double-sided block-alpha sheets filling the view behind one
    another, over an opaque textured cube: every pixel has n_sheets or more
    fragments."""
    s = S.Scene()
    s.textures.append(S.texture_uniform(21, 64, 64))
    s.textures.append(S.texture_block_alpha(22, 64, 64, 8))
    s.textures.append(S.texture_block_alpha(23, 32, 32, 4))
    s.materials.append((0xFFFFFFFF, 0, 0, 32))
    s.materials.append((0xFFFFFFFF, 1, 1, 32))
    s.materials.append((0xFFFFFFFF, 2, 1, 32))
    n0 = s.add_node(translation=(0.0, 0.0, -2.5), rotation=S.rot_y(0.6).astype(np.float32))
    for (p, nm, t, i) in S.cube_mesh(2.0):
        s.add_primitive(n0, S.TRIANGLE_FAN, 0, p, nm, t, i)
    q = np.array([[-3.0, -2.0, 0.0], [3.0, -2.0, 0.0], [3.0, 2.0, 0.0], [-3.0, 2.0, 0.0]], np.float32)
    nq = np.tile(np.array([0.0, 0.0, 1.0], np.float32), (4, 1))
    uq = np.array([[0.0, 0.0], [2.0, 0.0], [2.0, 1.5], [0.0, 1.5]], np.float32)
    for k in range(n_sheets):
        nk = s.add_node(translation=(0.05 * k, -0.03 * k, -2.0 + 0.25 * k),
                        rotation=S.rot_z(0.07 * k).astype(np.float32))
        s.add_primitive(nk, S.TRIANGLE_FAN, 1 + (k % 2), q, nq, uq, np.arange(4, dtype=np.uint32))
    s.point_lights = [(0.0, 1.0, 2.0, 2.0)]
    return s.finalize()


def stack_view(w, h, layers, shader=0, x=0, y=0):
    m, cp = S.look_at((0.2, 0.1, 1.6), (0.0, 0.0, -2.0))
    v = S.view_for(w, h, m, cp)
    v.layers, v.shader, v.x, v.y = layers, shader, x, y
    return v


@pytest.mark.parametrize("layers,shader", [(1, 0), (3, 0), (8, 0), (4, 5), (2, 4)])
def test_deep_stack_grows_the_pool_and_matches_oracle(renderer, layers, shader):
    sc = stack_scene()
    sid = renderer.upload(sc)
    v = stack_view(240, 180, layers, shader)
    frames, stats = renderer.render(sid, [v], stats=True)
    ref = oracle.render(sc, [v])
    assert stats["fragments"] > 4 * v.w * v.h  # beyond the first pool: rendered again after growing it
    assert stats["fragments"] == ref.stats[0][1]
    assert stats["drawn_triangles"] == ref.stats[0][0]
    assert np.array_equal(frames[0].zbuffer.view(np.uint32), ref.zbuffer.view(np.uint32))
    colour_check(frames[0].pixels, ref.pixels, f"layers {layers} shader {shader}")
    renderer.release(sid)


def test_surface_content_is_blended_and_offsets_follow_the_reference(renderer):
    """A surface holding a pattern before the render: the flatten blends onto
    the surface's row y, column x for view pixel (x, y), and the copy writes
    row y + view y, column x."""
    sc = stack_scene(6)
    sid = renderer.upload(sc)
    rng = np.random.default_rng(5)
    bg = rng.integers(0, 2 ** 32, size=(260, 330), dtype=np.uint64).astype(np.uint32)
    views = [stack_view(200, 150, 3, x=70, y=60), stack_view(120, 90, 5, x=10, y=20)]
    frames, _ = renderer.render(sid, views, shared_surface=(330, 260), background=bg)
    ref = oracle.render(sc, views, shared_surface=(330, 260), background=bg)
    for i in range(2):
        assert np.array_equal(frames[i].zbuffer.view(np.uint32), ref.frames[i].zbuffer.view(np.uint32)), i
    colour_check(frames[0].pixels, ref.frames[0].pixels, "shared surface")
    renderer.release(sid)


def test_device_targets_match_host_targets(renderer):
    torch = pytest.importorskip("torch")
    from swegl_gb300 import abi

    sc = S.glass_scene()
    sid = renderer.upload(sc)
    v = stack_view(320, 240, 4)
    m, cp = S.look_at((0.3, 0.4, 3.2), (0.0, 0.0, -0.5))
    v.view, v.camera_pos = m, cp
    host, _ = renderer.render(sid, [v])
    pix = torch.zeros((240, 320), dtype=torch.int32, device="cuda")
    z = torch.zeros((240, 320), dtype=torch.float32, device="cuda")
    import ctypes as C

    t = abi.Target()
    t.pixels, t.pitch, t.width, t.height = pix.data_ptr(), 4 * 320, 320, 240
    t.zbuffer = C.cast(C.c_void_p(z.data_ptr()), C.POINTER(C.c_float))
    renderer.render_device(sid, [v], [t])
    torch.cuda.synchronize()
    assert np.array_equal(pix.cpu().numpy().view(np.uint32), host[0].pixels)
    assert np.array_equal(z.cpu().numpy().view(np.uint32), host[0].zbuffer.view(np.uint32))
    renderer.release(sid)


def test_depth_of_field_on_layered_views_matches_oracle(renderer):
    """Depth of field on views with transparency layers: the gather runs over
    the view's rectangle after the layers are flattened and copied, with the
    view's opaque depth.  One view alone, then two offset views on a surface
    holding a pattern (the copy writes the reference's offsets, the gather
    reads the rectangle back), against the oracle; the blur radius varies
    across the sheets and the cube (focus 3, aperture 0.2, at most 12 px)."""
    sc = stack_scene(6)
    sid = renderer.upload(sc)
    dof = dict(dof_focus=3.0, dof_aperture=0.2, dof_max_radius=12.0)
    v = stack_view(240, 180, 3)
    v.dof = True
    v.dof_focus, v.dof_aperture, v.dof_max_radius = dof["dof_focus"], dof["dof_aperture"], dof["dof_max_radius"]
    frames, _ = renderer.render(sid, [v])
    ref = oracle.render(sc, [v])
    assert np.array_equal(frames[0].zbuffer.view(np.uint32), ref.zbuffer.view(np.uint32))
    colour_check(frames[0].pixels, ref.pixels, "layered view with depth of field")
    plain, _ = renderer.render(sid, [stack_view(240, 180, 3)])
    assert not np.array_equal(plain[0].pixels, frames[0].pixels)  # the gather changed the frame
    rng = np.random.default_rng(9)
    bg = rng.integers(0, 2 ** 32, size=(260, 330), dtype=np.uint64).astype(np.uint32)
    views = [stack_view(200, 150, 3, x=70, y=60), stack_view(120, 90, 2, x=10, y=20)]
    for w in views:
        w.dof = True
        w.dof_focus, w.dof_aperture, w.dof_max_radius = dof["dof_focus"], dof["dof_aperture"], dof["dof_max_radius"]
    frames, _ = renderer.render(sid, views, shared_surface=(330, 260), background=bg)
    ref = oracle.render(sc, views, shared_surface=(330, 260), background=bg)
    for i in range(2):
        assert np.array_equal(frames[i].zbuffer.view(np.uint32), ref.frames[i].zbuffer.view(np.uint32)), i
    colour_check(frames[0].pixels, ref.frames[0].pixels, "offset layered views with depth of field")
    renderer.release(sid)


def test_serving_loop_renders_layered_requests(renderer):
    """Layered requests mixed with opaque ones in the serving loop (each
    layered request runs alone, its framebuffer as the surface; the deep
    stack makes the first fragment pool overflow): every frame equals
    sgl_render's for the same view."""
    glass = S.glass_scene()
    stack = stack_scene()
    gid, kid = renderer.upload(glass), renderer.upload(stack)
    m, c = S.look_at((0.3, 0.4, 3.2), (0.0, 0.0, -0.5))
    reqs = []
    for k, (w, h, layers) in enumerate([(160, 120, 0), (200, 150, 3), (96, 64, 1), (320, 240, 8), (128, 96, 0),
                                        (64, 48, 2)]):
        v = S.view_for(w, h, m, c)
        v.layers = layers
        reqs.append((gid, v))
    big = stack_view(400, 300, 4)  # > 4 fragments per pixel: the pool grows and the request is redone
    reqs.append((kid, big))
    blur = stack_view(200, 150, 2)  # with depth of field
    blur.dof, blur.dof_focus, blur.dof_aperture, blur.dof_max_radius = True, 3.0, 0.2, 12.0
    reqs.append((kid, blur))
    srv = renderer.server(budget_bytes=512 << 20, max_batch=4, streams=2, copy_out=True)
    outs = []
    for sid, v in reqs:
        pix = np.zeros((v.h, v.w), np.uint32)
        z = np.zeros((v.h, v.w), np.float32)
        outs.append((srv.submit(sid, v, pix, z), pix, z))
    for (sid, v), (t, pix, z) in zip(reqs, outs):
        res = srv.wait(t)
        assert res["status"] == 0
        frames, _ = renderer.render(sid, [v])
        assert np.array_equal(pix, frames[0].pixels), (v.w, v.layers)
        assert np.array_equal(z.view(np.uint32), frames[0].zbuffer.view(np.uint32)), (v.w, v.layers)
    srv.close()
    renderer.release(gid)
    renderer.release(kid)


def test_batch_with_layered_items(renderer):
    """sgl_render_batch with opaque and layered items on device targets:
    every item equals its own sgl_render."""
    torch = pytest.importorskip("torch")
    import ctypes as C

    from swegl_gb300 import abi

    glass = S.glass_scene()
    gid = renderer.upload(glass)
    m, c = S.look_at((0.3, 0.4, 3.2), (0.0, 0.0, -0.5))
    items, bufs = [], []
    for (w, h, layers) in [(160, 120, 2), (200, 150, 0), (96, 64, 4), (128, 96, 0)]:
        v = S.view_for(w, h, m, c)
        v.layers = layers
        pix = torch.zeros((h, w), dtype=torch.int32, device="cuda")
        z = torch.zeros((h, w), dtype=torch.float32, device="cuda")
        t = abi.Target()
        t.pixels, t.pitch, t.width, t.height = pix.data_ptr(), 4 * w, w, h
        t.zbuffer = C.cast(C.c_void_p(z.data_ptr()), C.POINTER(C.c_float))
        items.append((gid, v, t))
        bufs.append((pix, z))
    stats = renderer.render_batch(items, stats=True)
    torch.cuda.synchronize()
    assert stats["pixels"] == sum(v.w * v.h for _, v, _ in items)
    for (_, v, _), (pix, z) in zip(items, bufs):
        frames, _ = renderer.render(gid, [v])
        assert np.array_equal(pix.cpu().numpy().view(np.uint32), frames[0].pixels), (v.w, v.layers)
        assert np.array_equal(z.cpu().numpy().view(np.uint32), frames[0].zbuffer.view(np.uint32)), (v.w, v.layers)
    renderer.release(gid)


def test_layered_views_are_refused_outside_sgl_render(renderer):
    torch = pytest.importorskip("torch")
    from swegl_gb300 import abi
    from swegl_gb300.runtime import SglError

    sc = S.glass_scene()
    sid = renderer.upload(sc)
    v = stack_view(64, 48, 2)
    pix = torch.zeros((48, 64), dtype=torch.int32, device="cuda")
    t = abi.Target()
    t.pixels, t.pitch, t.width, t.height = pix.data_ptr(), 4 * 64, 64, 48
    with pytest.raises(SglError) as e:
        renderer.autotune([(sid, v, t)])
    assert e.value.status == -8
    with pytest.raises(SglError) as e:
        renderer.render_debug(sid, v)
    assert e.value.status == -8
    v.layers = 9  # above SGL_MAX_LAYERS
    with pytest.raises(SglError) as e:
        renderer.render(sid, [v])
    assert e.value.status == -1
    renderer.release(sid)
