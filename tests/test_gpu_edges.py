"""Edge cases of the render path on the GPU against the oracle restatement
(pinned to the reference's fixtures): an empty scene, primitives that draw
nothing, degenerate and sliver triangles, triangles across the viewport
edges, one-pixel views and strips / fans with repeated indices.

Bar: depth bit-exact; colour within 2 LSB per channel (within 1 LSB on
>= 99.9 % of pixels)."""
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


def check(renderer, sc, views, shared=None):
    sid = renderer.upload(sc)
    frames, stats = renderer.render(sid, views, shared_surface=shared, stats=True)
    ref = oracle.render(sc, views, shared_surface=shared)
    for i, (f, e) in enumerate(zip(frames, ref.frames)):
        assert np.array_equal(f.zbuffer.view(np.uint32), e.zbuffer.view(np.uint32)), f"view {i}: depth"
        d = np.abs(f.pixels.view(np.uint8).astype(np.int16) - e.pixels.view(np.uint8).astype(np.int16))
        assert int(d.max()) <= 2, f"view {i}: colour differs by {int(d.max())}"
        assert float((d.reshape(-1, 4).max(axis=1) <= 1).mean()) >= 0.999
    assert stats["fragments"] == sum(s[1] for s in ref.stats)
    renderer.release(sid)
    return frames, ref


def lit(s):
    s.ambient, s.sun_intensity = 0.2, 0.6
    s.point_lights = [(0.5, 1.5, 2.5, 2.0)]
    return s


def cam(w, h, pos=(0.3, 0.4, 3.0), target=(0.0, 0.0, 0.0), **kw):
    m, c = S.look_at(pos, target)
    v = S.view_for(w, h, m, c)
    for k, x in kw.items():
        setattr(v, k, x)
    return v


def test_empty_scene_is_background(renderer):
    sc = lit(S.Scene()).finalize()
    frames, _ = check(renderer, sc, [cam(64, 48)])
    assert not frames[0].pixels.any()
    assert np.all(frames[0].zbuffer.view(np.uint32) == 0x7F7F7F7F)


def test_degenerate_sliver_and_edge_triangles(renderer):
    """Zero-area (collinear, repeated vertices), one-pixel slivers, huge
    triangles reaching far outside the view, triangles along the viewport
    border, a primitive without indices and strips / fans with repeated
    indices, mixed with a lit textured cube."""
    s = lit(S.Scene())
    s.textures.append(S.texture_uniform(5, 32, 32))
    s.materials.append((0xFFFFFFFF, 0, 1, 32))
    s.materials.append((0xFF20A040, -1, 1, 32))
    n = s.add_node()
    for (p, nm, t, i) in S.cube_mesh(1.0):
        s.add_primitive(n, S.TRIANGLE_FAN, 0, p, nm, t, i)
    pos = np.array([
        [0, 0, 0], [1, 1, 0], [2, 2, 0],                 # collinear, slanted
        [0.5, 0.5, 0.2], [0.5, 0.5, 0.2], [0.7, 0.1, 0.2],  # repeated vertex
        [-0.2, -0.5, 0.4], [-0.2 + 1e-4, 0.9, 0.4], [-0.2, 0.9, 0.4],  # sliver
        [-50, -40, -3], [60, -40, -3], [0, 70, -3],       # far outside the view
        [-1.4, -1.05, 0.6], [1.4, -1.05, 0.6], [0, -1.2, 0.6],  # along the bottom border
    ], np.float32)
    nrm = S.normalize_f32(np.tile([[0.1, 0.2, 1.0]], (len(pos), 1)))
    uv = np.random.default_rng(1).uniform(0, 1, (len(pos), 2)).astype(np.float32)
    s.add_primitive(n, S.TRIANGLES, 1, pos, nrm, uv, np.arange(len(pos), dtype=np.uint32))
    s.add_primitive(n, S.TRIANGLES, 1, pos[:6], nrm[:6], uv[:6], np.zeros(0, np.uint32))  # no indices
    strip = np.array([0, 1, 1, 2, 3, 3, 4, 5], np.uint32)  # repeated indices make zero-area steps
    sp = np.array([[-0.9, 0.2, 0.3], [-0.6, 0.6, 0.3], [-0.4, 0.1, 0.3], [-0.1, 0.7, 0.3], [0.2, 0.2, 0.3],
                   [0.4, 0.65, 0.3]], np.float32)
    s.add_primitive(n, S.TRIANGLE_STRIP, 0, sp, S.normalize_f32(np.tile([[0, 0, 1.0]], (6, 1))), uv[:6], strip)
    s.add_primitive(n, S.TRIANGLE_FAN, 1, sp, S.normalize_f32(np.tile([[0, 0, 1.0]], (6, 1))), uv[:6],
                    np.array([0, 1, 2, 2, 3, 5, 4], np.uint32))
    s.finalize()
    views = [cam(160, 120), cam(97, 61, pos=(-1.5, 0.5, 2.0)), cam(1, 1), cam(3, 200, pos=(0.0, 0.0, 2.5))]
    check(renderer, s, views)
    # and every view on one surface at offsets
    for k, (x, y) in enumerate([(0, 0), (160, 0), (0, 120), (300, 0)]):
        views[k].x, views[k].y = x, y
    check(renderer, s, views, shared=(320, 240))


def test_empty_and_degenerate_scenes_in_every_entry_point(renderer):
    """Zero-work cases through the layered path, a batch and the serving loop."""
    torch = pytest.importorskip("torch")
    import ctypes as C

    from swegl_gb300 import abi

    empty = lit(S.Scene()).finalize()
    eid = renderer.upload(empty)
    v = cam(40, 30, layers=3)
    frames, _ = renderer.render(eid, [v])
    assert not frames[0].pixels.any()
    pix = torch.ones((30, 40), dtype=torch.int32, device="cuda")
    z = torch.zeros((30, 40), dtype=torch.float32, device="cuda")
    t = abi.Target()
    t.pixels, t.pitch, t.width, t.height = pix.data_ptr(), 160, 40, 30
    t.zbuffer = C.cast(C.c_void_p(z.data_ptr()), C.POINTER(C.c_float))
    opaque = cam(40, 30)
    renderer.render_batch([(eid, opaque, t), (eid, v, t)])
    torch.cuda.synchronize()
    assert not pix.any().item()
    srv = renderer.server(budget_bytes=64 << 20, max_batch=4, streams=2, copy_out=True)
    outs = []
    for view in (opaque, v):
        hp = np.full((30, 40), 7, np.uint32)
        hz = np.zeros((30, 40), np.float32)
        outs.append((srv.submit(eid, view, hp, hz), hp, hz))
    for ticket, hp, hz in outs:
        assert srv.wait(ticket)["status"] == 0
        assert not hp.any()
        assert np.all(hz.view(np.uint32) == 0x7F7F7F7F)
    srv.close()
    renderer.release(eid)
