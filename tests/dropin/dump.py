"""Scene dump for tests/dropin/dropin_render.cpp (little-endian binary)."""
import struct

import numpy as np


def write_dump(path, scene, views, surface_wh):
    scene.finalize()
    out = bytearray()
    i32 = lambda v: out.extend(struct.pack("<i", int(v)))
    f32 = lambda arr: out.extend(np.asarray(arr, np.float32).astype("<f4").tobytes())
    i32(len(scene.node_parent))
    for k in range(len(scene.node_parent)):
        f32(scene.node_scale[k])
        f32(np.asarray(scene.node_rotation[k], np.float32).reshape(-1))
        f32(scene.node_translation[k])
        i32(scene.node_parent[k])
    i32(len(scene.primitives))
    for (node, mode, mat, vo, vc, io, ic) in scene.primitives:
        for v in (node, mode, mat, vc, ic):
            i32(v)
        vtx = np.concatenate([scene.positions[vo:vo + vc], scene.normals[vo:vo + vc], scene.uvs[vo:vo + vc]], 1)
        f32(vtx.reshape(-1))
        out.extend(np.asarray(scene.indices[io:io + ic], "<u4").tobytes())
    i32(len(scene.materials))
    for (color, tex, ds, shin) in scene.materials:
        out.extend(struct.pack("<Iiii", int(color) & 0xFFFFFFFF, tex, ds, shin))
    i32(len(scene.textures))
    for t in scene.textures:
        i32(t.shape[1])
        i32(t.shape[0])
        out.extend(np.asarray(t, "<u4").tobytes())
    i32(len(scene.point_lights))
    for l in scene.point_lights:
        f32(l)
    f32([scene.ambient])
    f32(scene.sun_direction)
    f32([scene.sun_intensity])
    i32(len(views))
    i32(surface_wh[0])
    i32(surface_wh[1])
    for v in views:
        for a in (v.x, v.y, v.w, v.h):
            i32(a)
        f32(np.asarray(v.view, np.float32).reshape(-1))
        f32(np.asarray(v.proj, np.float32).reshape(-1))
        f32(v.camera_pos)
        i32(int(getattr(v, "shader", 0)))
        i32(int(getattr(v, "layers", 0)))
    with open(path, "wb") as fh:
        fh.write(out)
