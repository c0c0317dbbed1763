"""sgl_render_noalloc: the renderer for callers that must not allocate.

Some callers cannot let a library allocate device memory — a frame callback
with a fixed memory plan, or a host that forbids the library from growing its
footprint or from taking the device-wide synchronisation of cudaMalloc.  The
entry point renders one view with all scratch taken from a static device
array.  This checks, through the C ABI, that two calls in a row give the same
frames as the allocating renderer (sgl_render), and that a view too large for
the static scratch is refused with a clear error.  It is collected last so
that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from swegl_gb300 import abi
from swegl_gb300 import scenes as S

pytestmark = pytest.mark.gpu

RGB_TOL = 2  # LSB, the renderer's colour tolerance


def _target(torch, w, h):
    pix = torch.zeros((h, w), dtype=torch.int32, device="cuda")
    zb = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    t = abi.Target()
    t.pixels = pix.data_ptr()
    t.pitch = 4 * w
    t.width, t.height = w, h
    t.zbuffer = C.cast(C.c_void_p(zb.data_ptr()), C.POINTER(C.c_float))
    return pix, zb, t


def test_noalloc_matches_allocating_renderer_twice():
    import torch
    from swegl_gb300.runtime import Renderer, SglError

    r = Renderer(0)
    scene = S.spheres_scene(n_spheres=20, tex_size=256)
    sid = r.upload(scene)
    views = [S.spheres_view(640, 360), S.cube_view(320, 240)]
    views[1].dof = True
    for v in views:
        pix_a, z_a, t_a = _target(torch, v.w, v.h)
        r.render_device(sid, [v], [t_a])
        torch.cuda.synchronize()
        for call in range(2):  # two calls in a row share the static scratch
            pix_b, z_b, t_b = _target(torch, v.w, v.h)
            vd = abi.view_desc(v)
            st = r.lib.sgl_render_noalloc(r.ctx, sid, C.byref(vd), C.byref(t_b), None)
            assert st == 0, r.lib.sgl_last_error(r.ctx)
            torch.cuda.synchronize()
            a = pix_a.cpu().numpy().view(np.uint8).astype(np.int16)
            b = pix_b.cpu().numpy().view(np.uint8).astype(np.int16)
            assert int(np.abs(a - b).max()) <= RGB_TOL, f"call {call}"
            assert np.array_equal(z_a.cpu().numpy().view(np.uint32), z_b.cpu().numpy().view(np.uint32))
    # a view whose scratch exceeds the static array is refused, not truncated
    big = S.spheres_view(3840, 2160)
    _, _, t_big = _target(torch, big.w, big.h)
    vd = abi.view_desc(big)
    st = r.lib.sgl_render_noalloc(r.ctx, sid, C.byref(vd), C.byref(t_big), None)
    assert st == -5
    assert b"static scratch" in r.lib.sgl_last_error(r.ctx)
    r.release(sid)
    r.close()
