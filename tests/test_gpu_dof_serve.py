"""Depth of field and the serving loop on the GPU.

* The gather kernel is bit-exact against the oracle's gather on the same
  input (integer sums of exact float tap offsets).
* A rendered frame with depth of field matches the oracle within the colour
  tolerance of the renderer (its input colour is within 1-2 LSB).
* The serving loop returns, for every request of a mixed stream, exactly the
  frame the plain one-frame-per-launch renderer makes for it alone; requests
  larger than the budget are refused."""
import numpy as np
import pytest

import cases as G
import oracle
from swegl_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def renderer():
    from swegl_gb300.runtime import Renderer

    r = Renderer(0)
    yield r
    r.close()


def test_dof_kernel_bit_exact(renderer):
    sc = G.scene("spheres200")
    v = S.spheres_view(480, 270)
    v.dof = True
    ref = oracle.render(sc, [S.spheres_view(480, 270)])
    got = renderer.dof(v, ref.pixels, ref.zbuffer)
    exp = oracle.dof(v, ref.pixels, ref.zbuffer)
    assert np.array_equal(got, exp)
    assert int((got != ref.pixels).sum()) > 1000  # the gather did blur


@pytest.mark.parametrize("max_radius,w,h", [(16.0, 480, 270), (5.5, 97, 61), (40.0, 300, 200), (0.0, 64, 48)])
def test_dof_kernel_radius_and_edges(renderer, max_radius, w, h):
    """Reaches staged in shared memory (<= 32 px, with tiles cut by the view
    edge) and larger ones read from memory give the oracle's bits."""
    sc = G.scene("spheres200")
    v = S.spheres_view(w, h)
    v.dof = True
    v.dof_max_radius = max_radius
    v.dof_aperture = 0.2
    ref = oracle.render(sc, [S.spheres_view(w, h)])
    got = renderer.dof(v, ref.pixels, ref.zbuffer)
    exp = oracle.dof(v, ref.pixels, ref.zbuffer)
    assert np.array_equal(got, exp)


def test_render_with_dof_matches_oracle(renderer):
    sc = G.scene("spheres200")
    sid = renderer.upload(sc)
    v = S.spheres_view(640, 360)
    v.dof = True
    frames, _ = renderer.render(sid, [v])
    ref = oracle.render(sc, [v])
    assert np.array_equal(frames[0].zbuffer.view(np.uint32), ref.zbuffer.view(np.uint32))
    d = np.abs(frames[0].pixels.view(np.uint8).astype(np.int16) - ref.pixels.view(np.uint8).astype(np.int16))
    assert int(d.max()) <= 2
    renderer.release(sid)


def test_4k_dof_frame_matches_oracle(renderer):
    """The depth-of-field configuration at full size: the 200-sphere scene at
    3840x2160 with the gather (focus 20, aperture 0.05, at most 16 px, 32
    taps).  Depth bit-exact; colour within 2 LSB, within 1 LSB on >= 99.9% of
    pixels."""
    sc = G.scene("spheres200")
    sid = renderer.upload(sc)
    v = S.spheres_view(3840, 2160)
    v.dof = True
    frames, _ = renderer.render(sid, [v])
    ref = oracle.render(sc, [v])
    assert np.array_equal(frames[0].zbuffer.view(np.uint32), ref.zbuffer.view(np.uint32))
    d = np.abs(frames[0].pixels.view(np.uint8).astype(np.int16) - ref.pixels.view(np.uint8).astype(np.int16))
    per_px = d.reshape(-1, 4).max(axis=1)
    assert int(d.max()) <= 2
    assert float((per_px <= 1).mean()) >= 0.999
    renderer.release(sid)


def test_serving_same_alone_and_in_the_mix(renderer):
    scenes = [S.spheres_scene(n_spheres=k, seed=40 + k, tex_size=128) for k in (3, 13, 25)]
    sids = [renderer.upload(sc) for sc in scenes]
    rng = S.Rng(77)
    reqs = []
    for i in range(40):
        sid_i = int(rng.integers(0, len(sids) - 1, 1)[0])
        w = S.log_uniform_int(rng, 64, 640)
        h = S.log_uniform_int(rng, 64, 480)
        m, c = S.camera_on_sphere(rng, 35.0)
        v = S.view_for(w, h, m, c)
        v.dof = bool(rng.integers(0, 1, 1)[0])
        reqs.append((sid_i, v))
    srv = renderer.server(budget_bytes=256 << 20, max_batch=8, streams=3, copy_out=True)
    outs = []
    tickets = []
    for sid_i, v in reqs:
        pix = np.zeros((v.h, v.w), np.uint32)
        z = np.zeros((v.h, v.w), np.float32)
        outs.append((pix, z))
        tickets.append(srv.submit(sids[sid_i], v, pix, z))
    results = [srv.wait(t, 60.0) for t in tickets]
    srv.close()
    assert all(r["status"] == 0 for r in results)
    for (sid_i, v), (pix, z), res in zip(reqs, outs, results):
        alone, st = renderer.render(sids[sid_i], [v], stats=True)
        assert np.array_equal(pix, alone[0].pixels), "frame differs in the mix"
        assert np.array_equal(z.view(np.uint32), alone[0].zbuffer.view(np.uint32))
        assert res["fragments"] == st["fragments"]
        assert res["submit_s"] <= res["start_s"] <= res["done_s"]
    for sid in sids:
        renderer.release(sid)


def test_serving_full_size_scenes_alone_and_in_the_mix(renderer):
    """The serving configuration's own inputs at a bounded request count: the
    8 resident scenes of 10k ... 2M triangles, and the first 32 requests of
    its seeded stream (viewports log-uniform 64x64 ... 3840x2160, depth of
    field on half of them), submitted at once to the continuous-batching loop
    under the 40 GB budget.  Each frame equals the one-frame-per-launch
    render of the same request alone (bit for bit) and the oracle (depth
    bit-exact, colour within 2 LSB and within 1 LSB on >= 99.9 % of
    pixels)."""
    import os

    scenes = S.serving_scenes()
    sids = [renderer.upload(sc) for sc in scenes]
    reqs = S.serving_requests(32, seed=61)
    assert any(v.dof for (_, _, v) in reqs) and any(not v.dof for (_, _, v) in reqs)
    assert max(v.w * v.h for (_, _, v) in reqs) > 1_000_000
    srv = renderer.server(budget_bytes=40 << 30, max_batch=16, streams=3, copy_out=True)
    outs, tickets = [], []
    for (_, k, v) in reqs:
        pix = np.zeros((v.h, v.w), np.uint32)
        z = np.zeros((v.h, v.w), np.float32)
        outs.append((pix, z))
        tickets.append(srv.submit(sids[k], v, pix, z))
    results = [srv.wait(t, 300.0) for t in tickets]
    srv.close()
    assert all(r["status"] == 0 for r in results)
    threads = max(1, min(16, os.cpu_count() or 1))
    by_scene = {}
    for j, (_, k, v) in enumerate(reqs):
        by_scene.setdefault(k, []).append(j)
    within1 = total = 0
    for k, js in by_scene.items():
        exp = oracle.render_parallel(scenes[k], [reqs[j][2] for j in js], threads)
        for j, e in zip(js, exp):
            v = reqs[j][2]
            pix, z = outs[j]
            alone, st = renderer.render(sids[k], [v], stats=True)
            assert np.array_equal(pix, alone[0].pixels), ("frame differs in the mix", j)
            assert np.array_equal(z.view(np.uint32), alone[0].zbuffer.view(np.uint32)), j
            assert results[j]["fragments"] == st["fragments"], j
            assert np.array_equal(z.view(np.uint32), e.zbuffer.view(np.uint32)), ("depth differs from the oracle", j)
            d = np.abs(pix.view(np.uint8).astype(np.int16) - e.pixels.view(np.uint8).astype(np.int16))
            assert int(d.max()) <= 2, j
            per_px = d.reshape(-1, 4).max(axis=1)
            within1 += int((per_px <= 1).sum())
            total += per_px.size
    assert within1 >= 0.999 * total
    for sid in sids:
        renderer.release(sid)


def test_serving_batch_submit_and_wait(renderer):
    """sgl_server_submit_batch / sgl_server_wait_batch: one call queues a
    list of requests (into host buffers) and one call collects them; each
    frame equals the one-frame-per-launch render; a request the budget can
    never hold stops the batch there, with the ones before it queued."""
    from swegl_gb300.runtime import Server, SglError

    sc = S.spheres_scene(n_spheres=9, seed=71, tex_size=128)
    sid = renderer.upload(sc)
    rng = S.Rng(93)
    items, views = [], []
    for i in range(20):
        m, c = S.camera_on_sphere(rng, 35.0)
        v = S.view_for(S.log_uniform_int(rng, 64, 500), S.log_uniform_int(rng, 64, 400), m, c)
        v.dof = i % 3 == 0
        pix = np.zeros((v.h, v.w), np.uint32)
        z = np.zeros((v.h, v.w), np.float32)
        items.append((sid, v, pix, z))
        views.append(v)
    srv = renderer.server(budget_bytes=256 << 20, max_batch=8, streams=2, copy_out=True)
    tickets = srv.submit_many(Server.requests(items))
    assert len(set(tickets.tolist())) == len(items)
    res = srv.wait_many(tickets, 60.0)
    assert all(x.status == 0 for x in res)
    for (_, v, pix, z), x in zip(items, res):
        alone, st = renderer.render(sid, [v], stats=True)
        assert np.array_equal(pix, alone[0].pixels)
        assert np.array_equal(z.view(np.uint32), alone[0].zbuffer.view(np.uint32))
        assert x.fragments == st["fragments"] and x.submit_s <= x.start_s <= x.rendered_s <= x.done_s
    # the third request cannot fit the budget: the first two are queued
    big = S.cube_view(3840, 2160)
    reqs = Server.requests([(sid, views[0]), (sid, views[1]), (sid, big), (sid, views[2])])
    with pytest.raises(SglError) as e:
        srv.submit_many(reqs)
    assert e.value.status == -5 and "queued 2 of 4" in str(e.value)
    srv.drain(60.0)
    srv.close()
    renderer.release(sid)


def test_serving_budget_and_poll(renderer):
    from swegl_gb300.runtime import SglError

    sc = S.cube_scene()
    sid = renderer.upload(sc)
    srv = renderer.server(budget_bytes=32 << 20, max_batch=4, streams=2, copy_out=False)
    with pytest.raises(SglError) as e:
        srv.submit(sid, S.cube_view(3840, 2160))  # colour + depth + scratch of 8.3 Mpx > 32 MiB
    assert e.value.status == -5
    t = srv.submit(sid, S.cube_view(320, 240))
    res = srv.wait(t, 30.0)
    assert res["status"] == 0 and res["fragments"] > 0
    with pytest.raises(SglError) as e:
        srv.poll(t + 1000)  # never issued
    assert e.value.status == -4
    srv.drain(10.0)
    srv.close()
    renderer.release(sid)


@pytest.mark.parametrize("pool_kind", ["pageable", "write_combined", "page_locked"])
def test_serving_copy_out_into_one_pool(renderer, pool_kind):
    """Host buffers carved from one pool in framebuffer order (colour, depth,
    next request): the loop merges the copies of a batch into one; every
    request still receives exactly its own frame — into pageable memory and
    into page-locked memory from sgl_host_alloc, write-combined or not."""
    from swegl_gb300.runtime import host_buffer

    scenes = [S.spheres_scene(n_spheres=k, seed=60 + k, tex_size=128) for k in (4, 9)]
    sids = [renderer.upload(sc) for sc in scenes]
    rng = S.Rng(91)
    reqs = []
    for i in range(24):
        w = S.log_uniform_int(rng, 64, 400)
        h = S.log_uniform_int(rng, 64, 300)
        m, c = S.camera_on_sphere(rng, 35.0)
        reqs.append((i % 2, S.view_for(w, h, m, c)))
    words = sum(2 * v.w * v.h for (_, v) in reqs)
    if pool_kind == "pageable":
        pool = np.zeros(words, np.uint32)
    else:
        pool = host_buffer(words, write_combined=pool_kind == "write_combined")
        pool[:] = 0
    srv = renderer.server(budget_bytes=256 << 20, max_batch=8, streams=2, copy_out=True)
    outs, tickets, off = [], [], 0
    for k, v in reqs:
        px = v.w * v.h
        pix = pool[off:off + px].reshape(v.h, v.w)
        z = pool[off + px:off + 2 * px].view(np.float32).reshape(v.h, v.w)
        off += 2 * px
        outs.append((pix, z))
        tickets.append(srv.submit(sids[k], v, pix, z))
    results = [srv.wait(t, 60.0) for t in tickets]
    srv.close()
    assert all(r["status"] == 0 for r in results)
    for (k, v), (pix, z) in zip(reqs, outs):
        alone, _ = renderer.render(sids[k], [v])
        assert np.array_equal(pix, alone[0].pixels)
        assert np.array_equal(z.view(np.uint32), alone[0].zbuffer.view(np.uint32))
    for sid in sids:
        renderer.release(sid)
