"""glTF scenes and image files through the library's host loaders.

`GltfScene(path)` is swegl::load_scene (src/data/gltf.cpp:455-464): the file
is read by `sgl_gltf_load` (include/sgl.h) and exposed as a `scenes.Scene`
(for `Renderer.upload`) whose nodes follow `animate(seconds)`
(scene_t::animate, swegl/data/model.hpp:146-177).  `load_image(path)` is
read_image_file (src/misc/image.cpp:20-27) for BMP, PNG and JPEG files.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from . import scenes as S
from .runtime import SglError, library


class GltfScene:
    def __init__(self, path: str):
        self.lib = library()
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        st = self.lib.sgl_gltf_load(path.encode(), C.byref(h), err, len(err))
        if st != 0:
            raise SglError(st, err.value.decode(errors="replace"))
        self.h = h

    @property
    def animation_count(self) -> int:
        return int(self.lib.sgl_gltf_animation_count(self.h))

    def scene(self) -> S.Scene:
        """A copy of the loaded scene description (no lights, as loaded)."""
        d = self.lib.sgl_gltf_scene(self.h).contents
        s = S.Scene()
        for i in range(d.n_nodes):
            nd = d.nodes[i]
            s.node_scale.append(np.array(nd.scale[:], np.float32))
            s.node_rotation.append(np.array(nd.rotation[:], np.float32).reshape(4, 4))
            s.node_translation.append(np.array(nd.translation[:], np.float32))
            s.node_parent.append(int(nd.parent))
        for i in range(d.n_primitives):
            p = d.primitives[i]
            s.primitives.append((p.node, p.mode, p.material, p.vertex_offset, p.vertex_count, p.index_offset,
                                 p.index_count))
        nv, ni = int(d.n_vertices), int(d.n_indices)
        s.positions = np.ctypeslib.as_array(d.positions, (nv * 3,)).reshape(nv, 3).copy() if nv else np.zeros((0, 3), np.float32)
        s.normals = np.ctypeslib.as_array(d.normals, (nv * 3,)).reshape(nv, 3).copy() if nv else np.zeros((0, 3), np.float32)
        s.uvs = np.ctypeslib.as_array(d.uvs, (nv * 2,)).reshape(nv, 2).copy() if nv else np.zeros((0, 2), np.float32)
        s.indices = np.ctypeslib.as_array(d.indices, (ni,)).copy() if ni else np.zeros((0,), np.uint32)
        for i in range(d.n_materials):
            m = d.materials[i]
            s.materials.append((int(m.color), int(m.texture), int(m.double_sided), int(m.shininess)))
        for i in range(d.n_textures):
            t = d.textures[i]
            s.textures.append(np.ctypeslib.as_array(t.texels, (t.height * t.width,)).reshape(t.height, t.width).copy())
        s.ambient = float(d.ambient)
        s.sun_direction = np.array(d.sun_direction[:], np.float32)
        s.sun_intensity = float(d.sun_intensity)
        return s.finalize()

    def animate(self, seconds: float):
        """Advance the animations to `seconds`; returns the node descriptions
        (abi.NodeDesc array) for sgl_scene_set_nodes."""
        d = self.lib.sgl_gltf_scene(self.h).contents
        nodes = (abi.NodeDesc * max(1, d.n_nodes))()
        st = self.lib.sgl_gltf_animate(self.h, C.c_float(seconds), nodes)
        if st != 0:
            raise SglError(st, "sgl_gltf_animate")
        return nodes

    def close(self):
        if self.h:
            self.lib.sgl_gltf_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_image(path: str) -> np.ndarray:
    """0xAARRGGBB texels (height, width) of a BMP, PNG or JPEG file."""
    lib = library()
    t = C.POINTER(C.c_uint32)()
    w, h = C.c_int(), C.c_int()
    err = C.create_string_buffer(512)
    st = lib.sgl_image_load(path.encode(), C.byref(t), C.byref(w), C.byref(h), err, len(err))
    if st != 0:
        raise SglError(st, err.value.decode(errors="replace"))
    try:
        return np.ctypeslib.as_array(t, (h.value * w.value,)).reshape(h.value, w.value).copy()
    finally:
        lib.sgl_image_free(t)
