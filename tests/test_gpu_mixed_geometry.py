"""A scene whose primitives take both geometry passes: a floor of one
3,200-triangle list (beyond the fused pass's limits of 256 vertices and 512
triangles per primitive) with cubes and a sphere standing on it (within
them).  The fused pass takes the small primitives, the general passes the
floor, each skipping the other's; the frames equal the oracle's (depth and
winners bit-exact, colour within the parity bar), from above and standing on
the floor (near-clipped triangles in both passes), in a batch with views of
other scenes, posed, and through the allocation-free entry point."""
import copy
import ctypes as C

import numpy as np
import pytest

import oracle
from swegl_gb300 import abi
from swegl_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def colour_check(got, exp, where=""):
    d = np.abs(got.view(np.uint8).astype(np.int16) - exp.view(np.uint8).astype(np.int16))
    per_px = d.reshape(-1, 4).max(axis=1)
    assert int(d.max()) <= 2, f"{where}: max |dRGB| {int(d.max())}"
    assert float((per_px <= 1).mean()) >= 0.999, f"{where}: histogram {np.bincount(per_px)[:3].tolist()}"


@pytest.fixture(scope="module")
def rig():
    import torch
    from swegl_gb300.runtime import Renderer

    r = Renderer(0)
    yield r, torch
    r.close()


def views():
    above = S.view_for(320, 240, *S.look_at((0.3, 3.0, 5.0), (0.0, -0.5, -1.5)))
    standing = S.view_for(320, 240, *S.look_at((0.3, -0.3, 2.0), (0.0, -0.5, -3.0)))
    return [above, standing]


def test_mixed_scene_matches_oracle(rig):
    r, _ = rig
    sc = S.mixed_size_scene()
    sid = r.upload(sc)
    for v in views():
        frames, stats = r.render(sid, [v], stats=True)
        ref = oracle.render(sc, [v])
        assert np.array_equal(frames[0].zbuffer.view(np.uint32), ref.zbuffer.view(np.uint32))
        colour_check(frames[0].pixels, ref.pixels, "mixed scene")
        assert stats["fragments"] == ref.stats[0][1]
        assert stats["drawn_triangles"] == ref.stats[0][0]
        frame, winner, _, _ = r.render_debug(sid, v)
        assert np.array_equal(winner, oracle.render(sc, [v], winner=True).winner)
    r.release(sid)


def test_mixed_scene_in_a_batch_posed_and_without_allocation(rig):
    r, torch = rig
    sc = S.mixed_size_scene()
    others = [S.spheres_scene(n_spheres=20, tex_size=128), S.grid_scene()]
    sid = r.upload(sc)
    oid = [r.upload(o) for o in others]
    vs = views()
    items, expect, bufs = [], [], []
    for k, v in enumerate(vs + vs):
        pix = torch.zeros((v.h, v.w), dtype=torch.int32, device="cuda")
        zb = torch.zeros((v.h, v.w), dtype=torch.float32, device="cuda")
        t = abi.Target()
        t.pixels, t.pitch, t.width, t.height = pix.data_ptr(), 4 * v.w, v.w, v.h
        t.zbuffer = C.cast(C.c_void_p(zb.data_ptr()), C.POINTER(C.c_float))
        bufs.append((pix, zb))
        if k < 2:
            items.append((sid, v, t))
            expect.append(r.render(sid, [v])[0][0])
        else:  # the other scenes' views in the same batch
            o = k - 2
            items.append((oid[o], v, t))
            expect.append(r.render(oid[o], [v])[0][0])
    # a pose of the mixed scene: every node moved
    posed = copy.deepcopy(sc)
    for i in range(len(posed.node_parent)):
        posed.node_translation[i] = np.asarray(posed.node_translation[i], np.float32) + np.float32([0.2, 0.0, -0.3])
    nodes = abi.SceneDescHolder(posed).nodes
    v = vs[0]
    pix = torch.zeros((v.h, v.w), dtype=torch.int32, device="cuda")
    zb = torch.zeros((v.h, v.w), dtype=torch.float32, device="cuda")
    t = abi.Target()
    t.pixels, t.pitch, t.width, t.height = pix.data_ptr(), 4 * v.w, v.w, v.h
    t.zbuffer = C.cast(C.c_void_p(zb.data_ptr()), C.POINTER(C.c_float))
    bufs.append((pix, zb))
    items.append((sid, v, t, nodes))
    ref_posed = oracle.render(posed, [v])
    r.render_batch(items)
    torch.cuda.synchronize()
    for k, e in enumerate(expect):
        pix, zb = bufs[k]
        assert np.array_equal(pix.cpu().numpy().view(np.uint32), e.pixels), k
        assert np.array_equal(zb.cpu().numpy().view(np.uint32), e.zbuffer.view(np.uint32)), k
    pix, zb = bufs[-1]
    assert np.array_equal(zb.cpu().numpy().view(np.uint32), ref_posed.zbuffer.view(np.uint32))
    colour_check(pix.cpu().numpy().view(np.uint32), ref_posed.pixels, "posed mixed scene")
    # the allocation-free entry point
    for v in vs:
        pix = torch.zeros((v.h, v.w), dtype=torch.int32, device="cuda")
        zb = torch.zeros((v.h, v.w), dtype=torch.float32, device="cuda")
        t = abi.Target()
        t.pixels, t.pitch, t.width, t.height = pix.data_ptr(), 4 * v.w, v.w, v.h
        t.zbuffer = C.cast(C.c_void_p(zb.data_ptr()), C.POINTER(C.c_float))
        vd = abi.view_desc(v)
        assert r.lib.sgl_render_noalloc(r.ctx, sid, C.byref(vd), C.byref(t), None) == 0
        torch.cuda.synchronize()
        e = r.render(sid, [v])[0][0]
        assert np.array_equal(pix.cpu().numpy().view(np.uint32), e.pixels)
        assert np.array_equal(zb.cpu().numpy().view(np.uint32), e.zbuffer.view(np.uint32))
    r.release(sid)
    for o in oid:
        r.release(o)
