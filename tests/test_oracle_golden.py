"""The oracle restatement (oracle/sgl_oracle.c) reproduces the reference's
own outputs bit for bit on every golden case: colour, depth, the ordinal of
the winning triangle, per-pixel progress, the Phong light value and the
bilinear texel (tests/golden, generated from the reference itself)."""
import json
import os

import numpy as np
import pytest

import cases as G
import oracle

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden.json")) as fh:
        meta = json.load(fh)
    arrays = np.load(os.path.join(HERE, "golden.npz"))
    return meta, arrays


CASES = G.cases()


def test_every_case_has_a_fixture(golden):
    meta, _ = golden
    assert set(meta) == set(CASES)


@pytest.mark.parametrize("name", sorted(CASES))
def test_restatement_matches_reference(golden, name):
    meta, arrays = golden
    case = CASES[name]
    entry = meta[name]
    sc = G.scene(case["scene"])
    assert sc.digest() == entry["scene_digest"], "scene builder is not reproducible on this host"
    views = case["views"]()
    for kind in case["kinds"]:
        r = oracle.render(sc, views, kind, "restatement", shared_surface=case.get("shared"))
        k = entry["kinds"][str(kind)]
        if kind in (0, 1):
            assert [s[0] for s in r.stats] == k["calls"]
        frames = [r.frames[0]] if case.get("shared") else r.frames
        for vi, f in enumerate(frames):
            if entry["store"] == G.FULL:
                exp = arrays[f"{name}/k{kind}/pixels{vi}"]
                diff = int((f.pixels != exp).sum())
                assert diff == 0, f"kind {kind} view {vi}: {diff} pixels differ"
            assert G.sha(f.pixels) == k[f"pixels{vi}"]
        if kind == 0:
            for vi, f in enumerate(r.frames):
                if entry["store"] == G.FULL:
                    exp = arrays[f"{name}/k0/z{vi}"]
                    assert int((f.zbuffer.view(np.uint32) != exp.view(np.uint32)).sum()) == 0
                assert G.sha(f.zbuffer) == k[f"z{vi}"]


def test_clip_branches_are_exercised():
    """Both near-plane clip branches of fill_triangle run in the golden set."""
    one = two = 0
    for name in ("cube_close_320x240", "cube_inside_320x240", "grid_clip_a_320x240", "grid_clip_b_320x240"):
        case = CASES[name]
        r = oracle.render(G.scene(case["scene"]), case["views"](), 0)
        one += r.stats[0][2]
        two += r.stats[0][3]
    assert one > 0 and two > 0


def test_reference_still_matches_fixtures_when_built():
    """Where the reference sources exist, regenerate one case and compare."""
    if not oracle.reference_available():
        pytest.skip("reference not built on this host")
    case = CASES["mixed_320x240"]
    with open(os.path.join(HERE, "golden.json")) as fh:
        meta = json.load(fh)
    r = oracle.render(G.scene("mixed"), case["views"](), 0, "reference")
    assert G.sha(r.pixels) == meta["mixed_320x240"]["kinds"]["0"]["pixels0"]
