"""sgl_render_noalloc: the renderer for callers that must not allocate.

Some callers cannot let a library allocate device memory — a frame callback
with a fixed memory plan, or a host that forbids the library from growing its
footprint or from taking the device-wide synchronisation of cudaMalloc.  The
entry point renders one view with all scratch taken from a static device
array.  It runs the same kernels on the same inputs as the allocating
renderer (sgl_render), so the frames must be identical bit for bit.  This
checks, through the C ABI, on two calls in a row:

* scenes of small primitives (the fused geometry pass), with and without
  depth of field;
* a floor of one 3,200-triangle list (the general geometry pass) seen by a
  camera standing on it, so that triangles cross the near plane;
* the largest floor view the static array accepts: its long-span capacity is
  then only a few thousand records, far fewer than the view's long spans, so
  the renderer takes its span-overflow path;

and that a view too large for the static scratch is refused with a clear
error.  It is collected last so that a failure here leaves every other test
already run.
"""
import ctypes as C

import numpy as np
import pytest

from swegl_gb300 import abi
from swegl_gb300 import scenes as S

pytestmark = pytest.mark.gpu

SGL_ERR_BUDGET = -5


def _target(torch, w, h):
    pix = torch.zeros((h, w), dtype=torch.int32, device="cuda")
    zb = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    t = abi.Target()
    t.pixels = pix.data_ptr()
    t.pitch = 4 * w
    t.width, t.height = w, h
    t.zbuffer = C.cast(C.c_void_p(zb.data_ptr()), C.POINTER(C.c_float))
    return pix, zb, t


def _noalloc(r, sid, v, t):
    vd = abi.view_desc(v)
    return r.lib.sgl_render_noalloc(r.ctx, sid, C.byref(vd), C.byref(t), None)


def _check_twice(r, torch, sid, v):
    """sgl_render once, then sgl_render_noalloc twice in a row: every call's
    colour and depth equal the allocating renderer's bit for bit."""
    pix_a, z_a, t_a = _target(torch, v.w, v.h)
    r.render_device(sid, [v], [t_a])
    torch.cuda.synchronize()
    a_pix, a_z = pix_a.cpu().numpy(), z_a.cpu().numpy().view(np.uint32)
    assert int((a_pix != 0).sum()) > 0, "the view shows nothing"
    for call in range(2):  # two calls in a row share the static scratch
        pix_b, z_b, t_b = _target(torch, v.w, v.h)
        st = _noalloc(r, sid, v, t_b)
        assert st == 0, r.lib.sgl_last_error(r.ctx)
        torch.cuda.synchronize()
        assert np.array_equal(pix_b.cpu().numpy(), a_pix), f"colour differs on call {call}"
        assert np.array_equal(z_b.cpu().numpy().view(np.uint32), a_z), f"depth differs on call {call}"


def test_noalloc_matches_allocating_renderer_twice():
    import torch
    from swegl_gb300.runtime import Renderer

    r = Renderer(0)
    scene = S.spheres_scene(n_spheres=20, tex_size=256)
    sid = r.upload(scene)
    views = [S.spheres_view(640, 360), S.cube_view(320, 240)]
    views[1].dof = True
    for v in views:
        _check_twice(r, torch, sid, v)
    # a view whose scratch exceeds the static array is refused, not truncated
    big = S.spheres_view(3840, 2160)
    _, _, t_big = _target(torch, big.w, big.h)
    assert _noalloc(r, sid, big, t_big) == SGL_ERR_BUDGET
    assert b"static scratch" in r.lib.sgl_last_error(r.ctx)
    r.release(sid)
    r.close()


def test_noalloc_general_geometry_near_clip_and_span_overflow():
    import torch
    from swegl_gb300.runtime import Renderer

    r = Renderer(0)
    floor = S.grid_scene()
    fid = r.upload(floor)
    # standing on the floor: near-clipped triangles, general geometry pass
    m, c = S.look_at((0.3, -0.3, 2.0), (0.0, -0.5, -3.0))
    _check_twice(r, torch, fid, S.view_for(320, 240, m, c))
    # above the floor, looking down at it: its triangles are tens of pixels
    # wide, so most rows are long spans.  Find the tallest 1920-wide view the
    # static array accepts (refusals happen on the host, before any device
    # work): its span capacity is then within one row's scratch (24 B per
    # pixel, 32 B for views of a million pixels or more, which shade through
    # a winner list) of the minimum of 4,096 records.
    m, c = S.look_at((0.3, 3.0, 7.0), (0.0, -0.5, 0.0))
    w = 1920
    _, _, t_probe = _target(torch, w, 4096)
    lo, hi = 64, 4096  # lo is accepted, hi refused
    assert _noalloc(r, fid, S.view_for(w, lo, m, c), t_probe) == 0, r.lib.sgl_last_error(r.ctx)
    assert _noalloc(r, fid, S.view_for(w, hi, m, c), t_probe) == SGL_ERR_BUDGET
    while hi - lo > 1:
        mid = (lo + hi) // 2
        st = _noalloc(r, fid, S.view_for(w, mid, m, c), t_probe)
        assert st in (0, SGL_ERR_BUDGET), r.lib.sgl_last_error(r.ctx)
        if st == 0:
            lo = mid
        else:
            hi = mid
    torch.cuda.synchronize()
    dense = S.view_for(w, lo, m, c)
    # long spans of the view: a run of more than 16 pixels won by one
    # triangle in a row lies inside that triangle's span of the row, so each
    # (row, triangle) with such a run is a distinct long span
    _, winner, _, _ = r.render_debug(fid, dense)
    long_spans = 0
    for row in winner:
        cut = np.flatnonzero(np.diff(row.astype(np.int64))) + 1
        starts = np.concatenate(([0], cut))
        lens = np.diff(np.concatenate((starts, [row.size])))
        long_spans += len(set(row[starts[(lens > 16) & (row[starts] != 0xFFFFFFFF)]].tolist()))
    assert long_spans > 5000, long_spans  # more than the static array's span capacity here
    _check_twice(r, torch, fid, dense)
    r.release(fid)
    r.close()
