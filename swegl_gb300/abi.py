"""ctypes mirror of include/sgl.h plus helpers that turn a `scenes.Scene` /
`scenes.View` into the flat C structures.

The structures must stay field-for-field identical to include/sgl.h.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

SGL_OK = 0
STATUS_NAMES = {
    0: "SGL_OK", -1: "SGL_ERR_INVALID", -2: "SGL_ERR_OOM", -3: "SGL_ERR_CUDA", -4: "SGL_ERR_NOT_FOUND",
    -5: "SGL_ERR_BUDGET", -6: "SGL_ERR_TIMEOUT", -7: "SGL_ERR_NO_DEVICE", -8: "SGL_ERR_UNSUPPORTED",
    -9: "SGL_ERR_BUSY",
}

F16 = C.c_float * 16
F3 = C.c_float * 3


class NodeDesc(C.Structure):
    _fields_ = [("scale", F3), ("rotation", F16), ("translation", F3), ("parent", C.c_int)]


class PrimitiveDesc(C.Structure):
    _fields_ = [("node", C.c_int), ("mode", C.c_int), ("material", C.c_int),
                ("vertex_offset", C.c_uint32), ("vertex_count", C.c_uint32),
                ("index_offset", C.c_uint32), ("index_count", C.c_uint32)]


class MaterialDesc(C.Structure):
    _fields_ = [("color", C.c_uint32), ("texture", C.c_int), ("double_sided", C.c_int), ("shininess", C.c_int)]


class TextureDesc(C.Structure):
    _fields_ = [("texels", C.POINTER(C.c_uint32)), ("width", C.c_int), ("height", C.c_int)]


class PointLight(C.Structure):
    _fields_ = [("position", F3), ("intensity", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("nodes", C.POINTER(NodeDesc)),
                ("n_primitives", C.c_int), ("primitives", C.POINTER(PrimitiveDesc)),
                ("n_vertices", C.c_uint32), ("positions", C.POINTER(C.c_float)),
                ("normals", C.POINTER(C.c_float)), ("uvs", C.POINTER(C.c_float)),
                ("n_indices", C.c_uint32), ("indices", C.POINTER(C.c_uint32)),
                ("n_materials", C.c_int), ("materials", C.POINTER(MaterialDesc)),
                ("n_textures", C.c_int), ("textures", C.POINTER(TextureDesc)),
                ("n_point_lights", C.c_int), ("point_lights", C.POINTER(PointLight)),
                ("ambient", C.c_float), ("sun_direction", F3), ("sun_intensity", C.c_float),
                ("default_material", MaterialDesc)]


class DofDesc(C.Structure):
    _fields_ = [("enabled", C.c_int), ("focus", C.c_float), ("aperture", C.c_float),
                ("max_radius", C.c_float), ("px_scale", C.c_float)]


SHADERS = ("phong_bilinear", "phong_nearest", "flat_bilinear", "flat_nearest", "color", "bilinear", "nearest",
           "phong", "flat")  # SGL_SHADER_* in order


class ViewDesc(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("w", C.c_int), ("h", C.c_int),
                ("view", F16), ("proj", F16), ("camera_pos", F3), ("dof", DofDesc), ("shader", C.c_int),
                ("layers", C.c_int)]


class Target(C.Structure):
    _fields_ = [("pixels", C.c_void_p), ("pitch", C.c_int), ("width", C.c_int), ("height", C.c_int),
                ("zbuffer", C.POINTER(C.c_float))]


class FrameStats(C.Structure):
    _fields_ = [("triangles", C.c_uint64), ("drawn_triangles", C.c_uint64), ("fragments", C.c_uint64),
                ("pixels", C.c_uint64), ("kernel_launches", C.c_uint32), ("reserved", C.c_uint32)]


class BatchOpts(C.Structure):
    _fields_ = [("tile", C.c_int), ("span_bin", C.c_int), ("use_graph", C.c_int)]


class BatchItem(C.Structure):
    _fields_ = [("scene_id", C.c_int), ("view", ViewDesc), ("target", Target), ("nodes", C.POINTER(NodeDesc)),
                ("n_nodes", C.c_int)]


class ServeOpts(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("max_batch", C.c_int), ("streams", C.c_int),
                ("copy_out", C.c_int)]


class Request(C.Structure):
    _fields_ = [("scene_id", C.c_int), ("view", ViewDesc), ("host_pixels", C.POINTER(C.c_uint32)),
                ("host_zbuffer", C.POINTER(C.c_float)), ("nodes", C.POINTER(NodeDesc)), ("n_nodes", C.c_int)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("submit_s", C.c_double), ("start_s", C.c_double), ("done_s", C.c_double),
                ("rendered_s", C.c_double), ("fragments", C.c_uint64)]


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class SceneDescHolder:
    """Owns the ctypes structures and numpy buffers behind a SceneDesc."""

    def __init__(self, scene):
        scene.finalize()
        self.scene = scene
        n_nodes = len(scene.node_parent)
        self.nodes = (NodeDesc * max(1, n_nodes))()
        for i in range(n_nodes):
            nd = self.nodes[i]
            nd.scale[:] = [float(v) for v in np.asarray(scene.node_scale[i], np.float32)]
            nd.rotation[:] = [float(v) for v in np.asarray(scene.node_rotation[i], np.float32).reshape(-1)]
            nd.translation[:] = [float(v) for v in np.asarray(scene.node_translation[i], np.float32)]
            nd.parent = int(scene.node_parent[i])
        n_prims = len(scene.primitives)
        self.prims = (PrimitiveDesc * max(1, n_prims))()
        for i, p in enumerate(scene.primitives):
            self.prims[i] = PrimitiveDesc(*[int(v) for v in p])
        self.positions = np.ascontiguousarray(scene.positions, np.float32)
        self.normals = np.ascontiguousarray(scene.normals, np.float32)
        self.uvs = np.ascontiguousarray(scene.uvs, np.float32)
        self.indices = np.ascontiguousarray(scene.indices, np.uint32)
        self.materials = (MaterialDesc * max(1, len(scene.materials)))()
        for i, m in enumerate(scene.materials):
            self.materials[i] = MaterialDesc(int(m[0]) & 0xFFFFFFFF, int(m[1]), int(m[2]), int(m[3]))
        self.texels = [np.ascontiguousarray(t, np.uint32) for t in scene.textures]
        self.textures = (TextureDesc * max(1, len(self.texels)))()
        for i, t in enumerate(self.texels):
            self.textures[i] = TextureDesc(_ptr(t, C.c_uint32), t.shape[1], t.shape[0])
        self.lights = (PointLight * max(1, len(scene.point_lights)))()
        for i, l in enumerate(scene.point_lights):
            self.lights[i].position[:] = [float(np.float32(l[0])), float(np.float32(l[1])), float(np.float32(l[2]))]
            self.lights[i].intensity = float(np.float32(l[3]))
        d = SceneDesc()
        d.n_nodes = n_nodes
        d.nodes = self.nodes
        d.n_primitives = n_prims
        d.primitives = self.prims
        d.n_vertices = len(self.positions)
        d.positions = _ptr(self.positions, C.c_float)
        d.normals = _ptr(self.normals, C.c_float)
        d.uvs = _ptr(self.uvs, C.c_float)
        d.n_indices = len(self.indices)
        d.indices = _ptr(self.indices, C.c_uint32)
        d.n_materials = len(scene.materials)
        d.materials = self.materials
        d.n_textures = len(self.texels)
        d.textures = self.textures
        d.n_point_lights = len(scene.point_lights)
        d.point_lights = self.lights
        d.ambient = float(np.float32(scene.ambient))
        d.sun_direction[:] = [float(v) for v in np.asarray(scene.sun_direction, np.float32)]
        d.sun_intensity = float(np.float32(scene.sun_intensity))
        d.default_material = MaterialDesc(0xFFFFFFFF, -1, 0, 32)
        self.desc = d

    def ref(self):
        return C.byref(self.desc)


def view_desc(v) -> ViewDesc:
    d = ViewDesc()
    d.x, d.y, d.w, d.h = int(v.x), int(v.y), int(v.w), int(v.h)
    d.view[:] = [float(x) for x in np.asarray(v.view, np.float32).reshape(-1)]
    d.proj[:] = [float(x) for x in np.asarray(v.proj, np.float32).reshape(-1)]
    d.camera_pos[:] = [float(x) for x in np.asarray(v.camera_pos, np.float32)]
    d.dof = DofDesc(1 if v.dof else 0, float(v.dof_focus), float(v.dof_aperture), float(v.dof_max_radius),
                    float(v.dof_px_scale))
    d.shader = int(getattr(v, "shader", 0))
    d.layers = int(getattr(v, "layers", 0))
    return d


class HostFrame:
    """A host BGRA8 surface plus the view's z-buffer."""

    def __init__(self, width: int, height: int, zw: int | None = None, zh: int | None = None, fill: int = 0):
        self.pixels = np.full((height, width), fill, np.uint32)
        self.zbuffer = np.zeros(((zh or height), (zw or width)), np.float32)

    def target(self) -> Target:
        t = Target()
        t.pixels = self.pixels.ctypes.data
        t.pitch = self.pixels.shape[1] * 4
        t.width = self.pixels.shape[1]
        t.height = self.pixels.shape[0]
        t.zbuffer = _ptr(self.zbuffer, C.c_float)
        return t
