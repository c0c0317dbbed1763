"""The library built with device-side bounds checks (libsgl_check.so: the
kernels compiled with -DSGL_BOUNDS_CHECK; a guarded access whose index falls
outside its buffer is recorded and skipped, nothing traps) over the edge-case,
view-volume and transparency-layer scenes of the other GPU tests, then over a
full-size frame, a 3840x2160 depth-of-field frame, a near-clipped floor, a
scene whose primitives take both geometry passes, a batch of uneven views
and the serving loop.  Every guarded access stays in its
buffer (the check record stays clear), and the checked library's frames equal
the normal library's bit for bit."""
import ctypes as C

import numpy as np
import pytest

import test_gpu_edges as E
import test_gpu_frustum as FR
import test_gpu_layers as LY
from swegl_gb300 import abi
from swegl_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked():
    from swegl_gb300.runtime import Renderer

    r = Renderer(0, checked=True)
    r.check_status(reset=True)
    yield r
    r.close()


def assert_clear(r, what):
    st = r.check_status(reset=True)
    assert st["count"] == 0, f"{what}: out-of-bounds access, check code {st['code']} at index {st['index']}"


def test_normal_library_has_no_checks():
    from swegl_gb300.runtime import Renderer, SglError

    r = Renderer(0)
    with pytest.raises(SglError) as e:
        r.check_status()
    assert e.value.status == -8  # SGL_ERR_UNSUPPORTED
    r.close()


def test_edge_scenes_stay_in_bounds(checked):
    E.test_empty_scene_is_background(checked)
    E.test_degenerate_sliver_and_edge_triangles(checked)
    E.test_empty_and_degenerate_scenes_in_every_entry_point(checked)
    assert_clear(checked, "edge scenes")
    for vi in range(3):
        FR.test_view_volume_sides_match_oracle(checked, vi)
    FR.test_batched_views_of_edge_scene_match_oracle(checked)
    FR.test_interleaved_vertex_ranges_match_oracle(checked)
    assert_clear(checked, "view-volume scenes")
    LY.test_deep_stack_grows_the_pool_and_matches_oracle(checked, 8, 0)
    LY.test_batch_with_layered_items(checked)
    assert_clear(checked, "transparency layers")


def _device_frames(torch, r, sid, views):
    bufs, tgts = [], []
    for v in views:
        pix = torch.zeros((v.h, v.w), dtype=torch.int32, device="cuda")
        zb = torch.zeros((v.h, v.w), dtype=torch.float32, device="cuda")
        t = abi.Target()
        t.pixels = pix.data_ptr()
        t.pitch = 4 * v.w
        t.width, t.height = v.w, v.h
        t.zbuffer = C.cast(C.c_void_p(zb.data_ptr()), C.POINTER(C.c_float))
        bufs.append((pix, zb))
        tgts.append(t)
    return bufs, tgts


def test_full_size_frames_batch_and_serving_match_the_unchecked_library(checked):
    import torch
    from swegl_gb300.runtime import Renderer

    plain = Renderer(0)
    spheres = S.spheres_scene()
    floor = S.grid_scene()
    dof = S.spheres_view(3840, 2160)
    dof.dof = True
    m, c = S.look_at((0.3, -0.3, 2.0), (0.0, -0.5, -3.0))
    cases = [(spheres, [S.spheres_view(1920, 1080)]), (spheres, [dof]), (floor, [S.view_for(640, 480, m, c)]),
             (S.mixed_size_scene(), [S.view_for(640, 480, m, c)])]  # both geometry passes on one scene
    for sc, views in cases:
        a = plain.upload(sc)
        b = checked.upload(sc)
        fa, sa = plain.render(a, views, stats=True)
        fb, sb = checked.render(b, views, stats=True)
        for x, y in zip(fa, fb):
            assert np.array_equal(x.pixels, y.pixels) and np.array_equal(x.zbuffer.view(np.uint32),
                                                                         y.zbuffer.view(np.uint32))
        assert sa["fragments"] == sb["fragments"]
        plain.release(a)
        checked.release(b)
    assert_clear(checked, "full-size frames")
    # a batch of 24 uneven views, one graph-captured launch sequence
    a, b = plain.upload(spheres), checked.upload(spheres)
    views = S.batch_views(24, seed=41)
    ba, ta = _device_frames(torch, plain, a, views)
    bb, tb = _device_frames(torch, checked, b, views)
    plain.render_batch([(a, v, t) for v, t in zip(views, ta)])
    checked.render_batch([(b, v, t) for v, t in zip(views, tb)])
    torch.cuda.synchronize()
    for (pa, za), (pb, zb) in zip(ba, bb):
        assert torch.equal(pa, pb) and torch.equal(za.view(torch.int32), zb.view(torch.int32))
    assert_clear(checked, "batch")
    # the serving loop on a mixed stream with depth of field
    reqs = S.serving_requests(24, seed=62, max_wh=(1280, 720))
    outs = []
    srv = checked.server(budget_bytes=8 << 30, max_batch=8, streams=3, copy_out=True)
    tickets = []
    for (_, _, v) in reqs:
        pix = np.zeros((v.h, v.w), np.uint32)
        z = np.zeros((v.h, v.w), np.float32)
        outs.append((pix, z))
        tickets.append(srv.submit(b, v, pix, z))
    assert all(srv.wait(t, 120.0)["status"] == 0 for t in tickets)
    srv.close()
    for (_, _, v), (pix, z) in zip(reqs, outs):
        ref, _ = plain.render(a, [v])
        assert np.array_equal(pix, ref[0].pixels) and np.array_equal(z.view(np.uint32), ref[0].zbuffer.view(np.uint32))
    assert_clear(checked, "serving")
    plain.release(a)
    checked.release(b)
    plain.close()
