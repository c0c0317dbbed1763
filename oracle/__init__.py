"""The oracle: CPU renderers that the GPU path is checked against.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg may import this package; the product never does.

Two renderers share one calling convention:
  * `restatement` — oracle/sgl_oracle.c, a C restatement of gbizzotto/swegl's
    render path (builds anywhere with gcc from its source);
  * `reference`   — the reference's own sources compiled headless by
    oracle/ref (only where the reference sources exist).  Its outputs are
    committed as golden fixtures under tests/golden.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from swegl_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libsgl_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libswegl_ref.so")
# where the reference sources lie (a build-container checkout; absent elsewhere)
REFERENCE_SRC = os.environ.get("SWEGL_REFERENCE", "/root/reference")

KIND_FULL, KIND_ORDINAL, KIND_PROGRESS, KIND_PHONG, KIND_TEXTURE = 0, 1, 2, 3, 4

_libs: dict[str, C.CDLL] = {}


def build(reference: bool | None = None) -> None:
    """Compile the restatement, and the reference too when its sources exist."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if reference is None:
        reference = os.path.isdir(os.path.join(REFERENCE_SRC, "src", "render"))
    if reference:
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "-j8", "REF=" + REFERENCE_SRC], check=True)


def restatement() -> C.CDLL:
    if "orc" not in _libs:
        if not os.path.exists(ORACLE_SO):
            build(reference=False)
        lib = C.CDLL(ORACLE_SO)
        lib.orc_render.restype = C.c_int
        lib.orc_render_parallel.restype = C.c_int
        lib.orc_triangle_count.restype = C.c_uint64
        lib.orc_dof.restype = C.c_int
        _libs["orc"] = lib
    return _libs["orc"]


def reference_available() -> bool:
    return os.path.exists(REF_SO)


def reference() -> C.CDLL:
    if "ref" not in _libs:
        lib = C.CDLL(REF_SO)
        lib.ref_render.restype = C.c_int
        _libs["ref"] = lib
    return _libs["ref"]


class Result:
    def __init__(self, frames, stats, winner):
        self.frames = frames          # list of abi.HostFrame
        self.stats = stats            # per view: (drawn, fragments, clip_one, clip_two); reference: (drawn, None)
        self.winner = winner          # winner slots of view 0 or None

    @property
    def pixels(self):
        return self.frames[0].pixels

    @property
    def zbuffer(self):
        return self.frames[0].zbuffer


def render(scene, views, kind: int = KIND_FULL, which: str = "restatement", winner: bool = False,
           shared_surface: tuple[int, int] | None = None, background: np.ndarray | None = None) -> Result:
    """Render `views` in order (swegl::render(scene, vp0, vp1, ...)).

    Each view gets its own surface of the view's size unless `shared_surface`
    = (width, height) asks for one surface shared by all views; `background`
    (shared surfaces only) is the surface's content before the render."""
    holder = abi.SceneDescHolder(scene)
    if shared_surface:
        surf = abi.HostFrame(*shared_surface)
        if background is not None:
            surf.pixels[...] = background
        frames = []
        for v in views:
            f = abi.HostFrame(*shared_surface, zw=v.w, zh=v.h)
            f.pixels = surf.pixels
            frames.append(f)
    else:
        frames = [abi.HostFrame(v.w, v.h) for v in views]
    vd = (abi.ViewDesc * len(views))(*[abi.view_desc(v) for v in views])
    td = (abi.Target * len(views))(*[f.target() for f in frames])
    win = np.full((views[0].h, views[0].w), 0xFFFFFFFF, np.uint32) if winner else None
    if which == "reference":
        calls = (C.c_uint64 * len(views))()
        rc = reference().ref_render(holder.ref(), vd, td, len(views), kind, calls)
        stats = [(int(calls[i]), None) for i in range(len(views))]
    else:
        st = (C.c_uint64 * (4 * len(views)))()
        wp = win.ctypes.data_as(C.POINTER(C.c_uint32)) if winner else None
        rc = restatement().orc_render(holder.ref(), vd, td, len(views), kind, wp, st)
        stats = [tuple(int(st[4 * i + k]) for k in range(4)) for i in range(len(views))]
    if rc != 0:
        raise RuntimeError(f"{which} render failed ({rc})")
    return Result(frames, stats, win)


def render_parallel(scene, views, threads: int) -> list:
    """Independent views rendered on `threads` host threads (CPU baseline)."""
    holder = abi.SceneDescHolder(scene)
    frames = [abi.HostFrame(v.w, v.h) for v in views]
    vd = (abi.ViewDesc * len(views))(*[abi.view_desc(v) for v in views])
    td = (abi.Target * len(views))(*[f.target() for f in frames])
    rc = restatement().orc_render_parallel(holder.ref(), vd, td, len(views), threads)
    if rc != 0:
        raise RuntimeError(f"parallel oracle render failed ({rc})")
    return frames


def dof(view, pixels: np.ndarray, zbuffer: np.ndarray) -> np.ndarray:
    """The depth-of-field gather on a (h, w) uint32 frame and its z-buffer."""
    h, w = pixels.shape
    src = np.ascontiguousarray(pixels, np.uint32)
    z = np.ascontiguousarray(zbuffer, np.float32)
    out = np.zeros_like(src)
    vd = abi.view_desc(view)
    vd.x = vd.y = 0
    t_in = abi.Target(src.ctypes.data, 4 * w, w, h, z.ctypes.data_as(C.POINTER(C.c_float)))
    t_out = abi.Target(out.ctypes.data, 4 * w, w, h, None)
    rc = restatement().orc_dof(C.byref(vd), C.byref(t_in), C.byref(t_out))
    if rc != 0:
        raise RuntimeError("oracle dof failed")
    return out


# ------------------------------------------------------------------ glTF --
class RefGltf:
    """The scene_t the reference's own glTF loader (src/data/gltf.cpp, built
    by oracle/ref with its nlohmann/json include resolved to a stand-in)
    builds, as written by ref_gltf_dump (oracle/ref/ref_gltf.cpp)."""

    def __init__(self):
        self.images = 0
        self.materials = []   # (colour uint32, metallic, roughness, texture, double sided)
        self.nodes = []       # dicts: scale, translation, rotation, root, children, primitives
        self.roots = []
        self.animations = []  # (end, [(node, path, [(t, (x, y, z, w))])])


def reference_gltf(path: str) -> RefGltf:
    """Load `path` with the compiled reference loader."""
    import tempfile

    lib = reference()
    lib.ref_gltf_dump.restype = C.c_int
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "dump.txt")
        if lib.ref_gltf_dump(path.encode(), out.encode()) != 0:
            raise RuntimeError("reference glTF dump failed")
        tok = open(out).read().split()
    at = 0

    def word():
        nonlocal at
        at += 1
        return tok[at - 1]

    def num():
        return int(word())

    def f32():
        return np.float32(float.fromhex(word()))

    r = RefGltf()
    assert word() == "images"
    r.images = num()
    assert word() == "materials"
    for _ in range(num()):
        r.materials.append((num() & 0xFFFFFFFF, f32(), f32(), num(), num()))
    assert word() == "nodes"
    for _ in range(num()):
        n = {"scale": np.array([f32() for _ in range(3)], np.float32),
             "translation": np.array([f32() for _ in range(3)], np.float32),
             "rotation": np.array([f32() for _ in range(16)], np.float32).reshape(4, 4)}
        n["root"] = num()
        n["children"] = [num() for _ in range(num())]
        prims = []
        for _ in range(num()):
            mode, mat, nv, ni = num(), num(), num(), num()
            v = np.array([f32() for _ in range(8 * nv)], np.float32).reshape(nv, 8)
            idx = np.array([num() for _ in range(ni)], np.uint32)
            prims.append({"mode": mode, "material": mat, "vertices": v, "indices": idx})
        n["primitives"] = prims
        r.nodes.append(n)
    assert word() == "roots"
    r.roots = [num() for _ in range(num())]
    assert word() == "animations"
    for _ in range(num()):
        end = f32()
        chans = []
        for _ in range(num()):
            node, pth, ns = num(), num(), num()
            steps = [(f32(), (f32(), f32(), f32(), f32())) for _ in range(ns)]
            chans.append((node, pth, steps))
        r.animations.append((end, chans))
    return r
