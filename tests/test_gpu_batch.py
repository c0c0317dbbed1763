"""The batched renderer (one launch sequence / one CUDA graph for many views of
uneven size, over several resident scenes) produces exactly the frames of the
plain one-frame-per-launch renderer, for every tile and span-bin choice."""
import copy
import ctypes as C

import numpy as np
import pytest

import cases as G
import oracle
from swegl_gb300 import abi
from swegl_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rig():
    import torch
    from swegl_gb300.runtime import Renderer

    r = Renderer(0)
    yield r, torch
    r.close()


def device_targets(torch, views):
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


def frames_of(bufs):
    return [(p.cpu().numpy().view(np.uint32), z.cpu().numpy()) for p, z in bufs]


def test_batch_equals_single_frames(rig):
    r, torch = rig
    scenes = [G.scene("spheres200"), G.scene("cube"), G.scene("mixed")]
    sids = [r.upload(sc) for sc in scenes]
    views = S.batch_views(12, seed=21, max_wh=(640, 480))
    owner = [i % 3 for i in range(len(views))]
    for i, v in enumerate(views):  # the cube and the mixed scene want closer cameras
        if owner[i] == 1:
            m, c = S.look_at(np.asarray(v.camera_pos, np.float64) / 7.0, (0, 0, 0))
            views[i] = S.view_for(v.w, v.h, m, c)
        elif owner[i] == 2:
            m, c = S.look_at(np.asarray(v.camera_pos, np.float64) / 6.0, (0, 0, 0))
            views[i] = S.view_for(v.w, v.h, m, c)
    bufs, tgts = device_targets(torch, views)
    for tile in (8, 16, 32):
        for span_bin in (8, 16, 32):
            for b in bufs:
                b[0].fill_(0x11)
            st = r.render_batch([(sids[owner[i]], v, t) for i, (v, t) in enumerate(zip(views, tgts))],
                                tile=tile, span_bin=span_bin, use_graph=True, stats=True)
            torch.cuda.synchronize()
            got = frames_of(bufs)
            for i, v in enumerate(views):
                ref = oracle.render(scenes[owner[i]], [v])
                assert np.array_equal(got[i][1].view(np.uint32), ref.zbuffer.view(np.uint32)), (tile, span_bin, i)
                d = np.abs(got[i][0].view(np.uint8).astype(np.int16) - ref.pixels.view(np.uint8).astype(np.int16))
                assert int(d.max()) <= 2, (tile, span_bin, i)
            assert st["fragments"] > 0


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_mixing_both_geometry_paths(rig, use_graph):
    """Scenes whose primitives fit the fused geometry pass (spheres, cube) and
    a scene that does not (the grid floor: one 3,200-triangle list) in one
    batch, in both orders: every view matches the oracle, and the triangle
    counts of both paths add up."""
    r, torch = rig
    scenes = [G.scene("grid"), G.scene("spheres200"), G.scene("cube")]
    sids = [r.upload(sc) for sc in scenes]
    views, owner = [], []
    for i, (pos, w, h) in enumerate([((0.5, 0.3, 3.0), 320, 240), ((3.0, 8.0, 30.0), 400, 300),
                                     ((1.5, 1.2, 3.5), 200, 160), ((-4.0, 1.0, 2.0), 256, 200),
                                     ((-20.0, 10.0, 25.0), 300, 200), ((2.0, -1.5, 3.0), 180, 140)]):
        k = [0, 1, 2, 0, 1, 2][i]
        target = (0.0, -0.4, 0.0) if k == 0 else (0.0, 0.0, 0.0)
        m, c = S.look_at(pos, target)
        views.append(S.view_for(w, h, m, c))
        owner.append(k)
    for order in (list(range(6)), list(reversed(range(6)))):
        vs = [views[i] for i in order]
        ow = [owner[i] for i in order]
        bufs, tgts = device_targets(torch, vs)
        st = r.render_batch([(sids[ow[i]], v, t) for i, (v, t) in enumerate(zip(vs, tgts))], use_graph=use_graph,
                            stats=True)
        torch.cuda.synchronize()
        got = frames_of(bufs)
        drawn = 0
        for i, v in enumerate(vs):
            ref = oracle.render(scenes[ow[i]], [v])
            assert np.array_equal(got[i][1].view(np.uint32), ref.zbuffer.view(np.uint32)), (order, i)
            d = np.abs(got[i][0].view(np.uint8).astype(np.int16) - ref.pixels.view(np.uint8).astype(np.int16))
            assert int(d.max()) <= 2, (order, i)
            drawn += ref.stats[0][0]
        assert st["drawn_triangles"] == drawn
    for sid in sids:
        r.release(sid)


def test_64_viewports_full_size(rig):
    """The batched configuration at full size: 64 seeded cameras on a sphere
    of radius 35 around the 200-sphere scene, viewports log-uniform from
    128x128 to 1920x1080, rendered in one graph-captured launch sequence
    with the tile and span bin the autotuner picks.  Every viewport equals
    the one-frame-per-launch render of it (bit for bit) and the oracle
    (depth bit-exact, colour within 2 LSB and within 1 LSB on >= 99.9 % of
    pixels)."""
    import os

    r, torch = rig
    sc = G.scene("spheres200")
    sid = r.upload(sc)
    views = S.batch_views(64)
    bufs, tgts = device_targets(torch, views)
    items = [(sid, v, t) for v, t in zip(views, tgts)]
    chosen = r.autotune(items)
    r.render_batch(items, tile=chosen["tile"], span_bin=chosen["span_bin"], use_graph=True)
    torch.cuda.synchronize()
    got = frames_of(bufs)
    exp = oracle.render_parallel(sc, views, max(1, min(16, os.cpu_count() or 1)))
    within1 = total = 0
    for i, v in enumerate(views):
        alone, _ = r.render(sid, [v])
        assert np.array_equal(got[i][0], alone[0].pixels), i
        assert np.array_equal(got[i][1].view(np.uint32), alone[0].zbuffer.view(np.uint32)), i
        assert np.array_equal(got[i][1].view(np.uint32), exp[i].zbuffer.view(np.uint32)), i
        d = np.abs(got[i][0].view(np.uint8).astype(np.int16) - exp[i].pixels.view(np.uint8).astype(np.int16))
        assert int(d.max()) <= 2, i
        per_px = d.reshape(-1, 4).max(axis=1)
        within1 += int((per_px <= 1).sum())
        total += per_px.size
    assert within1 >= 0.999 * total
    r.release(sid)


def test_64_viewports_of_the_cube(rig):
    """The batched configuration on the literal textured-cube scene (the
    640x480 configuration's cube): 64 seeded cameras on a sphere of radius
    35 around it, viewports log-uniform from 128x128 to 1920x1080, one
    graph-captured launch sequence with the autotuner's tile and span bin.
    Every viewport equals its one-frame-per-launch render bit for bit and the
    oracle (depth bit-exact, colour within 2 LSB, within 1 LSB on >= 99.9 %
    of pixels)."""
    import os

    r, torch = rig
    sc = G.scene("cube")
    sid = r.upload(sc)
    views = S.batch_views(64, seed=31)
    bufs, tgts = device_targets(torch, views)
    items = [(sid, v, t) for v, t in zip(views, tgts)]
    chosen = r.autotune(items)
    st = r.render_batch(items, tile=chosen["tile"], span_bin=chosen["span_bin"], use_graph=True, stats=True)
    torch.cuda.synchronize()
    assert st["fragments"] > 0
    got = frames_of(bufs)
    exp = oracle.render_parallel(sc, views, max(1, min(16, os.cpu_count() or 1)))
    within1 = total = covered = 0
    for i, v in enumerate(views):
        alone, _ = r.render(sid, [v])
        assert np.array_equal(got[i][0], alone[0].pixels), i
        assert np.array_equal(got[i][1].view(np.uint32), alone[0].zbuffer.view(np.uint32)), i
        assert np.array_equal(got[i][1].view(np.uint32), exp[i].zbuffer.view(np.uint32)), i
        d = np.abs(got[i][0].view(np.uint8).astype(np.int16) - exp[i].pixels.view(np.uint8).astype(np.int16))
        assert int(d.max()) <= 2, i
        per_px = d.reshape(-1, 4).max(axis=1)
        within1 += int((per_px <= 1).sum())
        total += per_px.size
        covered += int((got[i][1].view(np.uint32) != 0x7F7F7F7F).sum())
    assert within1 >= 0.999 * total
    assert covered > 1000  # the cube is seen
    r.release(sid)


def test_graph_replay_and_autotune(rig):
    r, torch = rig
    sc = G.scene("spheres200")
    sid = r.upload(sc)
    views = S.batch_views(8, seed=22, max_wh=(480, 320))
    bufs, tgts = device_targets(torch, views)
    items = [(sid, v, t) for v, t in zip(views, tgts)]
    chosen = r.autotune(items)
    assert chosen["tile"] in (8, 16, 32) and chosen["span_bin"] in (8, 16, 32)
    outs = []
    for rep in range(3):  # the same captured graph, replayed
        r.render_batch(items, tile=chosen["tile"], span_bin=chosen["span_bin"], use_graph=True)
        torch.cuda.synchronize()
        outs.append(frames_of(bufs))
    for rep in (1, 2):
        for a, b in zip(outs[0], outs[rep]):
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
    # a different batch through the same graphs
    views2 = S.batch_views(8, seed=23, max_wh=(480, 320))
    bufs2, tgts2 = device_targets(torch, views2)
    r.render_batch([(sid, v, t) for v, t in zip(views2, tgts2)], tile=chosen["tile"], span_bin=chosen["span_bin"])
    torch.cuda.synchronize()
    got = frames_of(bufs2)
    ref = oracle.render(sc, views2)
    for i in range(len(views2)):
        assert np.array_equal(got[i][1].view(np.uint32), ref.frames[i].zbuffer.view(np.uint32))


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_of_every_pixel_shader(rig, use_graph):
    """One batch with a view per pixel shader (SGL_SHADER_*): the frames of the
    default shader and of the other shaders come from different kernel
    instantiations of the same sequence; each matches the oracle."""
    r, torch = rig
    sc = G.scene("mixed")
    sid = r.upload(sc)
    views = []
    for mode in range(len(abi.SHADERS)):
        m, c = S.look_at((0.5 + 0.2 * mode, 0.8, 4.5), (0, 0, 0))
        v = S.view_for(160 + 8 * mode, 120, m, c)
        v.shader = mode
        views.append(v)
    bufs, tgts = device_targets(torch, views)
    r.render_batch([(sid, v, t) for v, t in zip(views, tgts)], use_graph=use_graph)
    torch.cuda.synchronize()
    for mode, ((pix, z), v) in enumerate(zip(frames_of(bufs), views)):
        ref = oracle.render(sc, [v])
        assert np.array_equal(z.view(np.uint32), ref.zbuffer.view(np.uint32)), abi.SHADERS[mode]
        if mode in (7, 8):
            # the light shaders write the int light value: compare it as an int
            dl = np.abs(pix.astype(np.int64) - ref.pixels.astype(np.int64))
            assert int(dl.max()) <= 2, (abi.SHADERS[mode], int(dl.max()))
        else:
            d = np.abs(pix.view(np.uint8).astype(np.int16) - ref.pixels.view(np.uint8).astype(np.int16))
            assert int(d.max()) <= 2, (abi.SHADERS[mode], int(d.max()))
    r.release(sid)


@pytest.mark.parametrize("make", ["spheres", "grid"])
def test_posed_items_equal_the_scene_set_to_each_pose(rig, make):
    """sgl_batch_item.nodes: several poses of one resident scene in one batch
    (each item's own node transforms), mixed with items that render the
    scene's current nodes.  Every item equals sgl_render of a second copy of
    the scene set to that item's pose (sgl_scene_set_nodes), bit for bit;
    the batched scene's own nodes are unchanged.  The spheres scene (200
    nodes) takes the fused geometry pass, where items are grouped by the
    vertex data they read; the floor takes the general one."""
    r, torch = rig
    rng = np.random.default_rng(23)
    if make == "spheres":
        base = S.spheres_scene(n_spheres=60, tex_size=128)
        views = [S.spheres_view(480, 270) for _ in range(6)]
    else:
        base = S.grid_scene()
        m, c = S.look_at((0.3, 3.0, 7.0), (0.0, -0.5, 0.0))
        views = [S.view_for(400, 300, m, c) for _ in range(6)]
    n = len(base.node_parent)
    sid, check = r.upload(base), r.upload(base)
    rest = abi.SceneDescHolder(base).nodes
    poses = []
    for k in range(4):
        sc = copy.deepcopy(base)
        for i in range(n):
            sc.node_translation[i] = (np.asarray(sc.node_translation[i], np.float32)
                                      + rng.uniform(-0.6, 0.6, 3).astype(np.float32))
        poses.append(abi.SceneDescHolder(sc).nodes)
    plan = [poses[0], None, poses[1], poses[2], None, poses[3]]
    bufs, tgts = device_targets(torch, views)
    r.render_batch([(sid, v, t, p) for v, t, p in zip(views, tgts, plan)])
    torch.cuda.synchronize()
    got = frames_of(bufs)
    for i, (v, p) in enumerate(zip(views, plan)):
        assert r.lib.sgl_scene_set_nodes(r.ctx, check, p if p is not None else rest, n) == 0
        exp, _ = r.render(check, [v])
        assert np.array_equal(got[i][0], exp[0].pixels), f"item {i}: colour"
        assert np.array_equal(got[i][1].view(np.uint32), exp[0].zbuffer.view(np.uint32)), f"item {i}: depth"
        if p is not None:
            assert not np.array_equal(got[i][1], got[1][1]), f"item {i}: the pose changed nothing"
    # the batched scene still renders its own nodes
    a, _ = r.render(sid, [views[1]])
    assert np.array_equal(a[0].pixels, got[1][0])
    # a pose must give every node of the scene
    short = (abi.NodeDesc * max(1, n - 1))()
    from swegl_gb300.runtime import SglError
    with pytest.raises(SglError) as e:
        r.render_batch([(sid, views[0], tgts[0], short)])
    assert e.value.status == -1
    r.release(sid)
    r.release(check)


def test_poses_that_bring_culled_primitives_into_view(rig):
    """The fused geometry pass skips a primitive for a view when the box of
    its world positions lies beyond one of the view's side planes; a posed
    item must use the boxes of its own pose.  The scene's own nodes put every
    sphere far to the side of the cameras (each primitive out of view), the
    poses put them back in view: each posed item matches the oracle's render
    of the scene under that pose (depth bit-exact, colour within 2 LSB,
    drawn triangles equal), and the items without a pose draw nothing."""
    r, torch = rig
    posed = S.spheres_scene(n_spheres=40, tex_size=64)
    away = copy.deepcopy(posed)
    n = len(posed.node_parent)
    for i in range(n):
        away.node_translation[i] = np.asarray(posed.node_translation[i], np.float32) + np.float32([400.0, 0.0, 0.0])
    sid = r.upload(away)
    views = []
    for k, (pos, w, h) in enumerate([((0.0, 0.0, 35.0), 320, 180), ((30.0, 5.0, 20.0), 96, 240),
                                     ((-10.0, 25.0, 20.0), 256, 64), ((0.0, 0.0, 35.0), 200, 200)]):
        m, c = S.look_at(pos, (0.0, 0.0, 0.0))
        views.append(S.view_for(w, h, m, c))
    pose = abi.SceneDescHolder(posed).nodes
    plan = [pose, None, pose, pose]
    bufs, tgts = device_targets(torch, views)
    st = r.render_batch([(sid, v, t, p) for v, t, p in zip(views, tgts, plan)], stats=True)
    torch.cuda.synchronize()
    got = frames_of(bufs)
    drawn = 0
    for i, (v, p) in enumerate(zip(views, plan)):
        ref = oracle.render(posed if p is not None else away, [v])
        assert np.array_equal(got[i][1].view(np.uint32), ref.zbuffer.view(np.uint32)), f"item {i}: depth"
        d = np.abs(got[i][0].view(np.uint8).astype(np.int16) - ref.pixels.view(np.uint8).astype(np.int16))
        assert int(d.max()) <= 2, f"item {i}: colour"
        drawn += ref.stats[0][0]
        if p is None:
            assert ref.stats[0][0] == 0
        else:
            assert ref.stats[0][0] > 0
    assert st["drawn_triangles"] == drawn
    r.release(sid)


def test_winner_list_shade_equals_tiled_shade(rig):
    """A batch of one view of a million pixels or more shades through a winner
    list (k_classify, then k_shade_wins); other batches shade in tiles
    (k_shade).  The same 1920x1080 view, with and without depth of field, as
    a batch of one (winner list) and as two items of one batch (tiled): the
    frames are equal bit for bit, and equal to the plain renderer's."""
    r, torch = rig
    sc = S.spheres_scene()
    sid = r.upload(sc)
    for dof in (False, True):
        v = S.spheres_view(1920, 1080)
        v.dof = dof
        one_bufs, one_tgts = device_targets(torch, [v])
        r.render_batch([(sid, v, one_tgts[0])])
        two_bufs, two_tgts = device_targets(torch, [v, v])
        r.render_batch([(sid, v, t) for t in two_tgts])
        torch.cuda.synchronize()
        one, two = frames_of(one_bufs), frames_of(two_bufs)
        plain, _ = r.render(sid, [v])
        for got in (one[0], two[0], two[1]):
            assert np.array_equal(got[0], plain[0].pixels), dof
            assert np.array_equal(got[1].view(np.uint32), plain[0].zbuffer.view(np.uint32)), dof
        assert int((one[0][1] < 1e30).sum()) > 100000  # the view shows the scene
    r.release(sid)
