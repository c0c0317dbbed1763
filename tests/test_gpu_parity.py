"""GPU parity: the CUDA path against the reference's golden fixtures and the
oracle restatement, through the C ABI.

Bar (per pixel): depth bits, span coverage and the depth-test winner are
bit-exact; colour is within 1 LSB per channel on >= 99.9% of pixels and within
2 LSB everywhere (the specular power is evaluated in float-float arithmetic
instead of the reference's double pow)."""
import json
import os

import numpy as np
import pytest

import cases as G
import oracle
from swegl_gb300 import scenes as S

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MAX_Z = 0x7F7F7F7F
RGB_TOL = 2          # LSB, everywhere
RGB_FRAC_1LSB = 0.999


@pytest.fixture(scope="module")
def renderer():
    from swegl_gb300.runtime import Renderer

    r = Renderer(0)
    yield r
    r.close()


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden.json")) as fh:
        meta = json.load(fh)
    return meta, np.load(os.path.join(HERE, "golden.npz"))


_scene_ids = {}


def scene_id(renderer, key):
    if key not in _scene_ids:
        _scene_ids[key] = renderer.upload(G.scene(key))
    return _scene_ids[key]


def colour_check(got, exp, where=""):
    d = np.abs(got.view(np.uint8).astype(np.int16) - exp.view(np.uint8).astype(np.int16))
    worst = int(d.max()) if d.size else 0
    per_px = d.reshape(-1, 4).max(axis=1)
    frac = float((per_px <= 1).mean()) if per_px.size else 1.0
    hist = np.bincount(per_px, minlength=3)[:3].tolist()
    assert worst <= RGB_TOL, f"{where}: max |dRGB| {worst}, histogram {hist}"
    assert frac >= RGB_FRAC_1LSB, f"{where}: only {frac:.5f} of pixels within 1 LSB, histogram {hist}"
    return hist


CASES = G.cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_reference_golden(renderer, golden, name):
    meta, arrays = golden
    case = CASES[name]
    entry = meta[name]
    sc = G.scene(case["scene"])
    assert sc.digest() == entry["scene_digest"]
    views = case["views"]()
    frames, stats = renderer.render(scene_id(renderer, case["scene"]), views, shared_surface=case.get("shared"))
    k0 = entry["kinds"]["0"]
    for vi, f in enumerate(frames):
        # depth: bit-exact against the reference itself
        assert G.sha(f.zbuffer) == k0[f"z{vi}"], f"view {vi}: depth differs from the reference"
    if entry["store"] == G.FULL:
        shown = [frames[0]] if case.get("shared") else frames
        for vi, f in enumerate(shown):
            exp = arrays[f"{name}/k0/pixels{vi}"]
            if views[vi].shader in (7, 8):
                # the light shaders write the int light value 65536 * L as the colour
                dl = np.abs(f.pixels.astype(np.int64) - exp.astype(np.int64))
                assert int(dl.max()) <= RGB_TOL, f"{name} view {vi}: light differs by {int(dl.max())}"
            else:
                colour_check(f.pixels, exp, f"{name} view {vi}")
    else:
        ref = oracle.render(sc, views, 0)
        assert G.sha(ref.pixels) == k0["pixels0"]
        colour_check(frames[0].pixels, ref.pixels, name)


@pytest.mark.parametrize("name", [n for n in sorted(CASES) if not CASES[n].get("shared") and 1 in CASES[n]["kinds"]])
def test_gpu_winners_and_coverage_match(renderer, golden, name):
    """Per-pixel depth-test winner (draw slot) and span coverage are bit-exact;
    the winner's draw ordinal equals the reference's ID-shader output."""
    meta, arrays = golden
    case = CASES[name]
    sc = G.scene(case["scene"])
    view = case["views"]()[0]
    frame, winner, flags, stats = renderer.render_debug(scene_id(renderer, case["scene"]), view)
    ref = oracle.render(sc, [view], winner=True)
    assert np.array_equal(winner, ref.winner), "winner slots differ"
    assert stats["fragments"] == ref.stats[0][1], "span coverage differs"
    assert stats["drawn_triangles"] == ref.stats[0][0]
    # map slots to the reference's fill_triangle_2 ordinals
    ordinal = np.cumsum(flags.astype(np.int64)) - 1
    covered = winner != 0xFFFFFFFF
    got = np.zeros_like(winner)
    got[covered] = ordinal[winner[covered]].astype(np.uint32)
    if meta[name]["store"] == G.FULL:
        exp = arrays[f"{name}/k1/pixels0"]
        assert np.array_equal(got[covered], exp[covered])
    else:
        assert int(flags.sum()) == meta[name]["kinds"]["0"]["calls"][0]


def test_heavy_scene_varied_shininess_matches_oracle(renderer):
    """The 1080p heavy scene with per-sphere shininess in [8, 128] (the
    reference's constant exponent 32 generalised).  Restatement-only: the
    reference hard-codes the exponent 32 (pixel_shaders.cpp:192), so no
    reference fixture exists for other exponents and this case is checked
    against the C restatement alone; at 32 the restatement equals the
    reference's fixtures bit for bit."""
    sc = S.spheres_scene()
    sid = renderer.upload(sc)
    view = S.spheres_view(1920, 1080)
    frames, stats = renderer.render(sid, [view], stats=True)
    ref = oracle.render(sc, [view])
    assert np.array_equal(frames[0].zbuffer.view(np.uint32), ref.zbuffer.view(np.uint32))
    hist = colour_check(frames[0].pixels, ref.pixels, "spheres varied shininess")
    assert stats["fragments"] == ref.stats[0][1]
    renderer.release(sid)
    print("histogram |dRGB| 0/1/2:", hist)


def test_batch_cameras_match_oracle(renderer):
    """Seeded cameras on a sphere of radius 35 at uneven sizes."""
    sc = G.scene("spheres200")
    sid = scene_id(renderer, "spheres200")
    views = S.batch_views(6, seed=11, max_wh=(640, 480))
    frames, _ = renderer.render(sid, views)
    ref = oracle.render(sc, views)
    for i, (f, r) in enumerate(zip(frames, ref.frames)):
        assert np.array_equal(f.zbuffer.view(np.uint32), r.zbuffer.view(np.uint32)), f"view {i}"
        colour_check(f.pixels, r.pixels, f"view {i}")


def test_node_update_and_lights(renderer):
    """sgl_scene_set_nodes / set_lights reproduce a freshly uploaded scene."""
    from swegl_gb300 import abi
    import ctypes as C

    sc = S.mixed_scene()
    sid = renderer.upload(sc)
    view = S.view_for(320, 240, *S.look_at((0.5, 0.8, 4.5), (0, 0, 0)))
    sc2 = S.mixed_scene()
    sc2.node_translation[0] = np.array([-1.0, 0.5, 0.2], np.float32)
    holder = abi.SceneDescHolder(sc2)
    st = renderer.lib.sgl_scene_set_nodes(renderer.ctx, sid, holder.nodes, len(sc2.node_parent))
    assert st == 0
    frames, _ = renderer.render(sid, [view])
    ref = oracle.render(sc2, [view])
    assert np.array_equal(frames[0].zbuffer.view(np.uint32), ref.zbuffer.view(np.uint32))
    colour_check(frames[0].pixels, ref.pixels, "after set_nodes")
    renderer.release(sid)


def test_invalid_inputs_return_errors(renderer):
    from swegl_gb300.runtime import SglError

    sc = S.cube_scene()
    sid = renderer.upload(sc)
    bad = S.cube_view(640, 480)
    bad.x = 100  # does not fit the 640-wide surface
    with pytest.raises(SglError) as e:
        renderer.render(sid, [bad], shared_surface=(640, 480))
    assert e.value.status == -1
    with pytest.raises(SglError) as e:
        renderer.render(12345, [S.cube_view()])
    assert e.value.status == -4
    broken = S.cube_scene()
    broken.indices = broken.indices.copy()
    broken.indices[2] = 99  # outside its primitive
    with pytest.raises(SglError):
        renderer.upload(broken)
    renderer.release(sid)
