"""Geometry at the edges of the view volume.  Scenes put many spheres just
inside, just outside and across each side of the view volume (NDC x or y
= +-1, where inside_camera_frustum switches) and its near plane (z' = 0.001,
where triangles go to the clip path), and behind the camera; they must
render exactly as the oracle, one view at a time and batched.  Draw order
unlike vertex order, and primitives sharing vertices (refused), are covered
too.

Bar: depth, per-pixel winners, drawn triangles and fragments bit-exact;
colour within 2 LSB per channel, within 1 LSB on >= 99.9% of pixels."""
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


def _world_of(view, q):
    """World point of view-space point q (the view matrix is a rigid motion)."""
    m = view.view.astype(np.float64)
    return np.linalg.solve(m[:3, :3], np.asarray(q, np.float64) - m[:3, 3])


def edge_scene(view, n: int = 96, seed: int = 11) -> S.Scene:
    """Spheres centred on the view volume's sides (NDC x or y = +-1, that is
    x' = +-z'), on its near plane (z' = 0.001) and behind the camera, each
    moved by up to 1.5 radii, so that their triangles fall on both sides of
    every frustum test."""
    rng = np.random.default_rng(seed)
    p = view.proj.astype(np.float64)
    s = S.Scene()
    s.textures.append(S.texture_uniform(seed, 64, 64))
    s.materials.append((0xFFFFFFFF, 0, 0, 16))
    s.materials.append((0xFF80C0FF, -1, 1, 8))  # double sided
    meshes = {}
    for i in range(n):
        kind = i % 6
        depth = rng.uniform(1.0, 12.0)
        rz = p[2, 2] * depth + p[2, 3]
        a, b = rng.uniform(-1.0, 1.0, 2)
        if kind < 2:      # x' = +-z'
            q = [(1 if kind else -1) * rz / p[0, 0], b * rz / p[1, 1], depth]
        elif kind < 4:    # y' = +-z'
            q = [a * rz / p[0, 0], (1 if kind == 3 else -1) * rz / p[1, 1], depth]
        elif kind == 4:   # z' = 0.001
            near = (0.001 - p[2, 3]) / p[2, 2]
            q = [a * 0.001, b * 0.001, near]
        else:             # behind the camera
            q = [a * 2.0, b * 2.0, -depth]
        r = float(rng.uniform(0.02, 0.3)) if kind != 4 else float(rng.uniform(0.0005, 0.005))
        c = _world_of(view, q) + rng.uniform(-1.5 * r, 1.5 * r, 3)
        node = s.add_node(translation=c.astype(np.float32))
        key = round(r, 4)
        if key not in meshes:
            meshes[key] = S.uv_sphere_mesh(64, 32, key)
        for (pp, nn, tt, idx) in meshes[key]:
            s.add_primitive(node, S.TRIANGLE_STRIP, i % 2, pp, nn, tt, idx)
    s.point_lights = [(0.0, 2.0, 2.0, 4.0)]
    return s.finalize()


def views():
    m, c = S.look_at((0.3, 0.2, 6.0), (0.0, 0.0, 0.0))
    return [S.view_for(320, 240, m, c), S.view_for(64, 300, m, c), S.view_for(500, 40, m, c)]


@pytest.mark.parametrize("vi", [0, 1, 2])
def test_view_volume_sides_match_oracle(renderer, vi):
    v = views()[vi]
    sc = edge_scene(v, seed=11 + vi)
    sid = renderer.upload(sc)
    frame, winner, flags, stats = renderer.render_debug(sid, v)
    ref = oracle.render(sc, [v], winner=True)
    assert np.array_equal(winner, ref.winner), "winner slots differ"
    assert stats["drawn_triangles"] == ref.stats[0][0]
    assert stats["fragments"] == ref.stats[0][1]
    assert np.array_equal(frame.zbuffer.view(np.uint32), ref.zbuffer.view(np.uint32))
    colour_check(frame.pixels, ref.pixels, f"edge view {vi}")
    assert stats["fragments"] > 1000  # part of the scene is in view
    renderer.release(sid)


def test_batched_views_of_edge_scene_match_oracle(renderer):
    """All three views in one batch: each item tests against its own camera."""
    vs = views()
    sc = edge_scene(vs[0], seed=21)
    sid = renderer.upload(sc)
    frames, _ = renderer.render(sid, vs)
    exp = oracle.render(sc, vs)
    for i, (f, e) in enumerate(zip(frames, exp.frames)):
        assert np.array_equal(f.zbuffer.view(np.uint32), e.zbuffer.view(np.uint32)), i
        colour_check(f.pixels, e.pixels, f"batched edge view {i}")
    renderer.release(sid)


def _flat(n):
    return np.tile(np.float32([0.0, 0.0, 1.0]), (n, 1)), np.zeros((n, 2), np.float32)


def interleaved_scene(view) -> S.Scene:
    """Vertex ranges in one order, draw order in another: P0 and P2 (node 0,
    in view) have their vertex ranges around that of P1 (node 1, wholly left
    of the view); a floor of 1152 triangles (node 1) and P3 (node 1, left of
    the view) follow.  Each triangle uses only its primitive's vertices."""
    p = view.proj.astype(np.float64)
    depth = 4.0
    rz = p[2, 2] * depth + p[2, 3]
    xl = -rz / p[0, 0]  # view-space x of the left side at this depth
    s = S.Scene()
    s.materials.append((0xFFC08040, -1, 1, 8))
    s.add_node()
    s.add_node()

    def tri(node, pts):
        pos = np.array([_world_of(view, (x, y, depth)) for (x, y) in pts], np.float32)
        n, uv = _flat(len(pos))
        s.add_primitive(node, S.TRIANGLES, 0, pos, n, uv, list(range(len(pts))))

    tri(0, [(xl + 0.2, -0.3), (xl + 0.9, 0.2), (xl + 0.5, 0.6)])             # P0
    tri(1, [(xl - 0.3, 0.0), (xl - 0.2, 0.25), (xl - 0.25, -0.2)])            # P1
    tri(0, [(xl + 1.0, -0.5), (xl + 1.6, -0.1), (xl + 1.2, 0.4)])             # P2
    n = 24  # the floor: 24 x 24 quads at depth 8
    g = np.stack(np.meshgrid(np.linspace(-3.0, 3.0, n + 1), np.linspace(-2.0, 2.0, n + 1)), -1).reshape(-1, 2)
    fpos = np.array([_world_of(view, (x, y, 8.0)) for (x, y) in g], np.float32)
    fidx = []
    for r in range(n):
        for c in range(n):
            k = r * (n + 1) + c
            fidx += [k, k + 1, k + n + 1, k + 1, k + n + 2, k + n + 1]
    fn, fuv = _flat(len(fpos))
    s.add_primitive(1, S.TRIANGLES, 0, fpos, fn, fuv, fidx)
    tri(1, [(xl - 0.6, 0.0), (xl - 0.4, 0.3), (xl - 0.5, -0.3)])              # P3
    return s.finalize()


def test_interleaved_vertex_ranges_match_oracle(renderer):
    v = views()[0]
    sc = interleaved_scene(v)
    sid = renderer.upload(sc)
    frame, winner, flags, stats = renderer.render_debug(sid, v)
    ref = oracle.render(sc, [v], winner=True)
    assert np.array_equal(winner, ref.winner)
    assert stats["drawn_triangles"] == ref.stats[0][0]
    assert stats["fragments"] == ref.stats[0][1] > 0
    colour_check(frame.pixels, ref.pixels, "interleaved ranges")
    renderer.release(sid)


def test_shared_vertex_ranges_are_rejected(renderer):
    """Each primitive owns its vertices: a second primitive over the first
    one's vertex range is refused at upload."""
    from swegl_gb300.runtime import SglError

    v = views()[0]
    sc = interleaved_scene(v)
    first = sc.primitives[0]
    sc.indices = np.concatenate([sc.indices, np.array([0, 1, 2], np.uint32)])
    sc.primitives.append((1, S.TRIANGLES, 0, first[3] + 1, 2, len(sc.indices) - 3, 0))
    with pytest.raises(SglError, match="share vertices"):
        renderer.upload(sc)
