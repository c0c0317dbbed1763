"""Generate the golden fixtures from the reference itself.

Renders every case of cases.py with gbizzotto/swegl's own render path
(compiled headless by oracle/ref into oracle/_ref/libswegl_ref.so) and
writes tests/golden/golden.npz (per-pixel arrays) and
tests/golden/golden.json (scene input digests, call counts, output digests).

Run from the repository root where the reference sources exist:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import oracle  # noqa: E402
import cases as G  # noqa: E402


def main() -> None:
    oracle.build(reference=True)
    arrays = {}
    meta = {}
    for name, case in G.cases().items():
        sc = G.scene(case["scene"])
        views = case["views"]()
        shared = case.get("shared")
        entry = {"scene": case["scene"], "scene_digest": sc.digest(), "kinds": {}, "store": case["store"],
                 "views": len(views)}
        for kind in case["kinds"]:
            r = oracle.render(sc, views, kind, "reference", shared_surface=shared)
            k = {"calls": [s[0] for s in r.stats]}
            frames = [r.frames[0]] if shared else r.frames
            for vi, f in enumerate(frames):
                k[f"pixels{vi}"] = G.sha(f.pixels)
                if case["store"] == G.FULL:
                    arrays[f"{name}/k{kind}/pixels{vi}"] = f.pixels
            for vi, f in enumerate(r.frames):
                if kind == 0:
                    k[f"z{vi}"] = G.sha(f.zbuffer)
                    if case["store"] == G.FULL:
                        arrays[f"{name}/k0/z{vi}"] = f.zbuffer
            entry["kinds"][str(kind)] = k
            print(name, kind, k["calls"], flush=True)
        meta[name] = entry
    here = os.path.dirname(os.path.abspath(__file__))
    np.savez_compressed(os.path.join(here, "golden.npz"), **arrays)
    with open(os.path.join(here, "golden.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
