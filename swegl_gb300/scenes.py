"""Seeded synthetic scenes for the swegl render path.

Every array produced here is bit-identical on any IEEE-754 host: only
elementwise +, -, *, /, sqrt, floor and integer hashing are used (numpy applies
no FMA contraction), and the trigonometric values come from the fixed
polynomial `sincos` below instead of the platform libm, whose last-bit
behaviour differs between x86-64 and aarch64.

Scenes mirror swegl's data model (swegl/data/model.hpp:20-178):
  * `cube(size)` is `make_cube` (model.hpp:254-325): 6 triangle fans of 4
    vertices with the 0.5 x 0.333 texture-atlas layout.
  * `uv_sphere(slices, stacks, r)` uses the strip layout of `make_sphere`
    (model.hpp:393-446): one TRIANGLE_STRIP primitive per longitude slice,
    2 * (stacks + 1) vertices and indices (stacks+1+s, s); with 64 x 32 that
    is 64 triangles per strip and 4096 per sphere.
  * Cameras follow camera_t (src/projection/camera.cpp:8-58): the view matrix
    starts as diag(1, 1, -1) (the camera looks down world -z) and the
    projection writes only rows 0-2 plus [3][2] = 1; x and y are divided by
    |z'| (swegl/render/vertex_shaders.hpp:65-70), so only P00, P11, P22, P23
    matter.  Vertical field of view 60 degrees, near 0.1, far 100.
"""
from __future__ import annotations

import functools
import math
from dataclasses import dataclass, field

import numpy as np

TRIANGLES, TRIANGLE_STRIP, TRIANGLE_FAN = 4, 5, 6

_MASK64 = np.uint64(0xFFFFFFFFFFFFFFFF)


# --------------------------------------------------------------------------
# deterministic random numbers: splitmix64 over a counter
# --------------------------------------------------------------------------
def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _MASK64
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _MASK64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _MASK64
    return z ^ (z >> np.uint64(31))


def hash64(*keys) -> np.ndarray:
    """Combine integer keys (scalars or broadcastable uint64 arrays)."""
    with np.errstate(over="ignore"):
        h = np.uint64(0x243F6A8885A308D3)
        for k in keys:
            h = _splitmix64(np.asarray(h, dtype=np.uint64) ^ np.asarray(k, dtype=np.uint64))
        return np.asarray(h, dtype=np.uint64)


class Rng:
    """Counter-based stream: draw i of stream `seed` is hash(seed, i)."""

    def __init__(self, seed: int):
        self.seed = np.uint64(seed)
        self.counter = 0

    def bits(self, n: int) -> np.ndarray:
        idx = np.arange(self.counter, self.counter + n, dtype=np.uint64)
        self.counter += n
        return hash64(self.seed, idx)

    def uniform(self, lo: float, hi: float, n: int) -> np.ndarray:
        u = (self.bits(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def integers(self, lo: int, hi_inclusive: int, n: int) -> np.ndarray:
        span = np.uint64(hi_inclusive - lo + 1)
        return (self.bits(n) % span).astype(np.int64) + lo


# --------------------------------------------------------------------------
# deterministic sin / cos (Cody-Waite reduction + Taylor, float64)
# --------------------------------------------------------------------------
_PIO2_HI = 1.5707963267341256e+00
_PIO2_LO = 6.0771005065061922e-11


def sincos(x) -> tuple[np.ndarray, np.ndarray]:
    x = np.asarray(x, dtype=np.float64)
    k = np.rint(x * (2.0 / math.pi))
    r = (x - k * _PIO2_HI) - k * _PIO2_LO
    r2 = r * r
    # Taylor series to degree 19 / 18 on |r| <= pi/4 (error < 1e-17).
    s = r
    term = r
    c = np.ones_like(r)
    cterm = np.ones_like(r)
    for n in range(1, 10):
        term = term * (-r2) / ((2 * n) * (2 * n + 1))
        s = s + term
        cterm = cterm * (-r2) / ((2 * n - 1) * (2 * n))
        c = c + cterm
    q = np.mod(k.astype(np.int64), 4)
    sin = np.where(q == 0, s, np.where(q == 1, c, np.where(q == 2, -s, -c)))
    cos = np.where(q == 0, c, np.where(q == 1, -s, np.where(q == 2, -c, s)))
    return sin, cos


def normalize_f32(v: np.ndarray) -> np.ndarray:
    """vector_t::normalize (swegl/projection/points.hpp:71-90) in float32."""
    v = np.asarray(v, dtype=np.float32)
    x, y, z = v[..., 0], v[..., 1], v[..., 2]
    l = np.sqrt(x * x + y * y + z * z)
    safe = np.where(l != 0, l, np.float32(1))
    out = np.stack([x / safe, y / safe, z / safe], axis=-1)
    return np.where((l != 0)[..., None], out, v).astype(np.float32)


# --------------------------------------------------------------------------
# matrices (row-major 4x4, matrix44_t conventions)
# --------------------------------------------------------------------------
def rot_y(a: float) -> np.ndarray:
    """matrix44_t::rotate_y applied to the identity (src/projection/matrix44.cpp:89-106)."""
    s, c = sincos(a)
    m = np.eye(4)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    return m


def rot_x(a: float) -> np.ndarray:
    """matrix44_t::rotate_x applied to the identity (src/projection/matrix44.cpp:70-87)."""
    s, c = sincos(a)
    m = np.eye(4)
    m[1, 1], m[1, 2], m[2, 1], m[2, 2] = c, s, -s, c
    return m


@functools.lru_cache(maxsize=16)
def _cot_half_fov(fov_y_deg: float) -> float:
    s, c = sincos(math.radians(fov_y_deg) / 2.0)
    return float(c / s)


def projection(w: int, h: int, fov_y_deg: float = 60.0, near: float = 0.1, far: float = 100.0) -> np.ndarray:
    cot = _cot_half_fov(fov_y_deg)
    aspect = w / h
    p = np.eye(4)
    p[0, 0] = cot / aspect
    p[1, 1] = cot
    p[2, 2] = far / (far - near)
    p[2, 3] = -far * near / (far - near)
    p[3, 2] = 1.0
    return p.astype(np.float32)


def _dot3(a, b) -> float:
    return float(a[0]) * float(b[0]) + float(a[1]) * float(b[1]) + float(a[2]) * float(b[2])


def _cross3(a, b) -> np.ndarray:
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]])


def matmul4(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """4x4 product with a fixed summation order (no BLAS)."""
    r = np.zeros((4, 4))
    for i in range(4):
        for j in range(4):
            acc = 0.0
            for k in range(4):
                acc = acc + float(a[i, k]) * float(b[k, j])
            r[i, j] = acc
    return r


def look_at_origin(position: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """View matrix of a camera at `position` looking at the origin, in the
    reference's convention (forward maps to +z of view space, up to +y)."""
    c = np.asarray(position, dtype=np.float64)
    f = -c / math.sqrt(_dot3(c, c))
    up = np.array([0.0, 1.0, 0.0])
    r = _cross3(f, up)
    if _dot3(r, r) < 1e-12:
        r = _cross3(f, np.array([0.0, 0.0, 1.0]))
    r = r / math.sqrt(_dot3(r, r))
    u = _cross3(r, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = r, u, f
    for i in range(3):
        m[i, 3] = -_dot3(m[i, :3], c)
    return m.astype(np.float32), c.astype(np.float32)


def camera_at_z(dist: float) -> tuple[np.ndarray, np.ndarray]:
    """camera_t() then translate(0, 0, -dist): camera on +z looking at the origin."""
    m = np.eye(4)
    m[2, 2] = -1.0
    m[2, 3] = dist
    return m.astype(np.float32), np.array([0.0, 0.0, dist], dtype=np.float32)


def camera_on_sphere(rng: Rng, radius: float) -> tuple[np.ndarray, np.ndarray]:
    """Uniform direction on the sphere (yaw U[0, 2pi), pitch asin(U[-1, 1]))."""
    z = rng.uniform(-1.0, 1.0, 1)[0]
    yaw = rng.uniform(0.0, 2.0 * math.pi, 1)[0]
    sy, cy = sincos(yaw)
    return _camera_at(z, float(sy), float(cy), radius)


def _camera_at(z: float, sy: float, cy: float, radius: float) -> tuple[np.ndarray, np.ndarray]:
    rxz = math.sqrt(max(0.0, 1.0 - z * z))
    d = np.array([rxz * cy, z, rxz * sy])
    return look_at_origin(radius * d)


# --------------------------------------------------------------------------
# scene container
# --------------------------------------------------------------------------
@dataclass
class View:
    x: int
    y: int
    w: int
    h: int
    view: np.ndarray
    proj: np.ndarray
    camera_pos: np.ndarray
    dof: bool = False
    dof_focus: float = 20.0
    dof_aperture: float = 0.05
    dof_max_radius: float = 16.0
    dof_px_scale: float = 0.0
    shader: int = 0  # SGL_SHADER_* (include/sgl.h)
    layers: int = 0  # transparency layers (0 = opaque)


@dataclass
class Scene:
    # nodes
    node_scale: list = field(default_factory=list)
    node_rotation: list = field(default_factory=list)
    node_translation: list = field(default_factory=list)
    node_parent: list = field(default_factory=list)
    # primitives: (node, mode, material, vertex_offset, vertex_count, index_offset, index_count)
    primitives: list = field(default_factory=list)
    positions: list = field(default_factory=list)
    normals: list = field(default_factory=list)
    uvs: list = field(default_factory=list)
    indices: list = field(default_factory=list)
    # materials: (color, texture, double_sided, shininess)
    materials: list = field(default_factory=list)
    textures: list = field(default_factory=list)  # uint32 (h, w) arrays
    point_lights: list = field(default_factory=list)  # (x, y, z, intensity)
    ambient: float = 0.1
    sun_direction: np.ndarray = field(default_factory=lambda: normalize_f32(np.array([-1.0, -1.0, -1.0])))
    sun_intensity: float = 0.7
    _nv: int = 0
    _ni: int = 0

    def add_node(self, translation=(0.0, 0.0, 0.0), rotation=None, scale=(1.0, 1.0, 1.0), parent=-1) -> int:
        self.node_scale.append(np.asarray(scale, dtype=np.float32))
        self.node_rotation.append(np.eye(4, dtype=np.float32) if rotation is None else np.asarray(rotation, np.float32))
        self.node_translation.append(np.asarray(translation, dtype=np.float32))
        self.node_parent.append(parent)
        return len(self.node_parent) - 1

    def add_primitive(self, node, mode, material, pos, nrm, uv, idx):
        pos = np.asarray(pos, np.float32).reshape(-1, 3)
        self.primitives.append((node, mode, material, self._nv, len(pos), self._ni, len(idx)))
        self.positions.append(pos)
        self.normals.append(np.asarray(nrm, np.float32).reshape(-1, 3))
        self.uvs.append(np.asarray(uv, np.float32).reshape(-1, 2))
        self.indices.append(np.asarray(idx, np.uint32))
        self._nv += len(pos)
        self._ni += len(idx)

    def finalize(self) -> "Scene":
        """Concatenate per-primitive arrays (idempotent)."""
        if isinstance(self.positions, list):
            self.positions = np.concatenate(self.positions) if self.positions else np.zeros((0, 3), np.float32)
            self.normals = np.concatenate(self.normals) if self.normals else np.zeros((0, 3), np.float32)
            self.uvs = np.concatenate(self.uvs) if self.uvs else np.zeros((0, 2), np.float32)
            self.indices = np.concatenate(self.indices) if self.indices else np.zeros((0,), np.uint32)
        return self

    @property
    def n_triangles(self) -> int:
        n = 0
        for (_, mode, _, _, _, _, ic) in self.primitives:
            n += ic // 3 if mode == TRIANGLES else max(0, ic - 2)
        return n

    def digest(self) -> str:
        """SHA-256 of every input array, to check that two hosts built the same scene."""
        import hashlib

        self.finalize()
        h = hashlib.sha256()
        for a in (self.positions, self.normals, self.uvs, self.indices,
                  np.asarray(self.primitives, np.int64), np.asarray(self.materials, np.int64),
                  np.asarray(self.node_scale, np.float32), np.asarray(self.node_rotation, np.float32),
                  np.asarray(self.node_translation, np.float32), np.asarray(self.node_parent, np.int64),
                  np.asarray(self.point_lights, np.float32).reshape(-1),
                  np.asarray([self.ambient, self.sun_intensity], np.float32), self.sun_direction):
            h.update(np.ascontiguousarray(a).tobytes())
        for t in self.textures:
            h.update(np.ascontiguousarray(t).tobytes())
        return h.hexdigest()


# --------------------------------------------------------------------------
# meshes
# --------------------------------------------------------------------------
def cube_mesh(size: float):
    """The six fans of make_cube (swegl/data/model.hpp:254-325)."""
    h = np.float32(size) / np.float32(2.0)
    f = lambda a: np.float32(a)
    faces = [
        # (positions, uvs, normal)
        ([(-h, h, h), (h, h, h), (h, h, -h), (-h, h, -h)], [(0.0, 0.0), (0.5, 0.0), (0.5, 0.333), (0.0, 0.333)], (0, 1, 0)),
        ([(-h, -h, h), (h, -h, h), (h, h, h), (-h, h, h)], [(0.5, 0.0), (1.0, 0.0), (1.0, 0.333), (0.5, 0.333)], (0, 0, 1)),
        ([(h, -h, h), (h, -h, -h), (h, h, -h), (h, h, h)], [(0.0, 0.333), (0.5, 0.333), (0.5, 0.667), (0.0, 0.667)], (1, 0, 0)),
        ([(h, -h, -h), (-h, -h, -h), (-h, h, -h), (h, h, -h)], [(0.5, 0.667), (1.0, 0.667), (1.0, 1.0), (0.5, 1.0)], (0, 0, -1)),
        ([(-h, -h, -h), (-h, -h, h), (-h, h, h), (-h, h, -h)], [(0.5, 0.333), (1.0, 0.333), (1.0, 0.667), (0.5, 0.667)], (-1, 0, 0)),
        ([(-h, -h, -h), (h, -h, -h), (h, -h, h), (-h, -h, h)], [(0.0, 0.667), (0.5, 0.667), (0.5, 1.0), (0.0, 1.0)], (0, -1, 0)),
    ]
    out = []
    for pos, uv, n in faces:
        p = np.array([[f(c) for c in v] for v in pos], np.float32)
        t = np.array(uv, dtype=np.float64).astype(np.float32)
        nn = np.tile(np.array(n, np.float32), (4, 1))
        out.append((p, nn, t, np.array([0, 1, 2, 3], np.uint32)))
    return out


def uv_sphere_mesh(slices: int, stacks: int, radius: float):
    """One strip per longitude slice, laid out like make_sphere
    (swegl/data/model.hpp:400-445): first row at longitude k, second row at
    k+1, latitude from the north pole (0, r, 0) down; indices (stacks+1+s, s)."""
    s_idx = np.arange(stacks + 1, dtype=np.float64)
    sin_t, cos_t = sincos(s_idx * (math.pi / stacks))
    k = np.arange(slices + 1, dtype=np.float64)
    sin_p, cos_p = sincos(k * (2.0 * math.pi / slices))
    r = float(radius)
    # ring[k, s] = (r sin(theta_s) cos(phi_k), r cos(theta_s), -r sin(theta_s) sin(phi_k))
    ring = np.empty((slices + 1, stacks + 1, 3), np.float64)
    ring[..., 0] = r * sin_t[None, :] * cos_p[:, None]
    ring[..., 1] = r * cos_t[None, :] + 0.0 * cos_p[:, None]
    ring[..., 2] = -r * sin_t[None, :] * sin_p[:, None]
    ring32 = ring.astype(np.float32)
    nrm32 = normalize_f32(ring32)
    u = (s_idx / stacks).astype(np.float32)
    out = []
    idx = np.empty(2 * (stacks + 1), np.uint32)
    idx[0::2] = np.arange(stacks + 1) + (stacks + 1)
    idx[1::2] = np.arange(stacks + 1)
    for b in range(slices):
        pos = np.concatenate([ring32[b], ring32[b + 1]])
        nrm = np.concatenate([nrm32[b], nrm32[b + 1]])
        v0 = np.full(stacks + 1, b / slices, np.float64).astype(np.float32)
        v1 = np.full(stacks + 1, (b + 1) / slices, np.float64).astype(np.float32)
        uv = np.concatenate([np.stack([u, v0], -1), np.stack([u, v1], -1)])
        out.append((pos, nrm, uv, idx.copy()))
    return out


# --------------------------------------------------------------------------
# textures
# --------------------------------------------------------------------------
def texture_uniform(seed: int, w: int, h: int) -> np.ndarray:
    """Uniform random RGB texels with alpha 255 (0xAARRGGBB)."""
    i = np.arange(w * h, dtype=np.uint64)
    rgb = (hash64(seed, 0x7E7, i) & np.uint64(0xFFFFFF)).astype(np.uint32)
    return (rgb | np.uint32(0xFF000000)).reshape(h, w)


def texture_value_noise(seed: int, size: int, octaves: int = 4, base_cells: int = 4) -> np.ndarray:
    """Tileable value noise, `octaves` octaves (cells base*2^o, amplitude 2^-o),
    smoothstep interpolation, one independent lattice per RGB channel."""
    coords = (np.arange(size, dtype=np.float64) + 0.5) / size
    total = np.zeros((3, size, size), np.float64)
    amp_sum = 0.0
    for o in range(octaves):
        cells = base_cells << o
        amp = 0.5 ** o
        amp_sum += amp
        t = coords * cells
        i0 = np.floor(t).astype(np.int64)
        fr = t - i0
        wgt = fr * fr * (3.0 - 2.0 * fr)
        i1 = (i0 + 1) % cells
        for ch in range(3):
            gx, gy = np.meshgrid(np.arange(cells, dtype=np.uint64), np.arange(cells, dtype=np.uint64))
            lat = (hash64(seed, 0x401, o, ch, gy, gx) >> np.uint64(40)).astype(np.float64) / float(1 << 24)
            a = lat[i0[:, None], i0[None, :]]
            b = lat[i0[:, None], i1[None, :]]
            c = lat[i1[:, None], i0[None, :]]
            d = lat[i1[:, None], i1[None, :]]
            wx = wgt[None, :]
            wy = wgt[:, None]
            top = a + (b - a) * wx
            bot = c + (d - c) * wx
            total[ch] += amp * (top + (bot - top) * wy)
    v = np.clip(np.floor(total / amp_sum * 256.0), 0, 255).astype(np.uint32)
    r, g, b = v[0], v[1], v[2]
    return (np.uint32(0xFF000000) | (r << np.uint32(16)) | (g << np.uint32(8)) | b).astype(np.uint32)


def texture_block_alpha(seed: int, w: int, h: int, block: int = 8) -> np.ndarray:
    """Uniform random RGB texels whose alpha is constant over block x block
    texel squares: per square 255 (3/8 of them), 0 (1/8) or uniform in
    1..254, so that bilinear filtering inside a square keeps its alpha."""
    i = np.arange(w * h, dtype=np.uint64)
    rgb = (hash64(seed, 0xA1F, i) & np.uint64(0xFFFFFF)).astype(np.uint32).reshape(h, w)
    by, bx = np.meshgrid(np.arange(h, dtype=np.uint64) // np.uint64(block),
                         np.arange(w, dtype=np.uint64) // np.uint64(block), indexing="ij")
    hv = hash64(seed, 0xB10C, by, bx)
    sel = (hv & np.uint64(7)).astype(np.uint32)
    rnd = (np.uint64(1) + (hv >> np.uint64(8)) % np.uint64(254)).astype(np.uint32)
    a = np.where(sel == 0, np.uint32(0), np.where(sel <= 3, np.uint32(255), rnd))
    return (rgb | (a << np.uint32(24))).astype(np.uint32)


# --------------------------------------------------------------------------
# the benchmark scenes
# --------------------------------------------------------------------------
CUBE_SEED = 1
SPHERES_SEED = 2


def cube_scene(seed: int = CUBE_SEED, tex_size: int = 256, size: float = 2.0) -> Scene:
    """Textured cube of side 2 rotated 30 degrees about Y then 20 about X;
    one seeded uniform-random 256x256 texture; sun (-1,-1,-1) normalised,
    ambient 0.1, shininess 32, no point lights."""
    s = Scene()
    s.textures.append(texture_uniform(seed, tex_size, tex_size))
    s.materials.append((0xFFFFFFFF, 0, 0, 32))
    rot = matmul4(rot_x(math.pi / 9.0), rot_y(math.pi / 6.0)).astype(np.float32)
    node = s.add_node(rotation=rot)
    for (p, n, t, i) in cube_mesh(size):
        s.add_primitive(node, TRIANGLE_FAN, 0, p, n, t, i)
    s.ambient = 0.1
    s.sun_intensity = 0.7
    return s.finalize()


def spheres_scene(n_spheres: int = 200, seed: int = SPHERES_SEED, n_textures: int = 8, tex_size: int = 1024,
                  slices: int = 64, stacks: int = 32, n_point_lights: int = 4, light_intensity: float = 50.0,
                  box: float = 20.0, r_min: float = 0.3, r_max: float = 2.0, shininess=(8, 128),
                  textures: list | None = None) -> Scene:
    """UV spheres with centres uniform in [-box, box]^3 and radii uniform in
    [r_min, r_max]; value-noise textures, one picked per sphere; per-sphere
    integer shininess uniform in `shininess`; sun plus point lights at
    uniform positions rejected when within 0.5 of a sphere surface."""
    rng = Rng(seed)
    s = Scene()
    if textures is not None:  # shared, prebuilt texture set
        s.textures = list(textures)
        n_textures = len(textures)
    else:
        for t in range(n_textures):
            s.textures.append(texture_value_noise(seed * 1000 + t, tex_size))
    centres = rng.uniform(-box, box, 3 * n_spheres).reshape(n_spheres, 3).astype(np.float32)
    radii = rng.uniform(r_min, r_max, n_spheres)
    tex_ids = rng.integers(0, n_textures - 1, n_spheres)
    if isinstance(shininess, tuple):
        shin = rng.integers(shininess[0], shininess[1], n_spheres)
    else:
        shin = np.full(n_spheres, int(shininess))
    mesh_cache = {}
    for i in range(n_spheres):
        s.materials.append((0xFFFFFFFF, int(tex_ids[i]), 0, int(shin[i])))
        node = s.add_node(translation=centres[i])
        key = float(radii[i])
        if key not in mesh_cache:
            mesh_cache[key] = uv_sphere_mesh(slices, stacks, key)
        for (p, n, t, idx) in mesh_cache[key]:
            s.add_primitive(node, TRIANGLE_STRIP, i, p, n, t, idx)
    lights = []
    while len(lights) < n_point_lights:
        p = rng.uniform(-box, box, 3)
        dc = centres.astype(np.float64) - p
        d = np.sqrt(dc[:, 0] * dc[:, 0] + dc[:, 1] * dc[:, 1] + dc[:, 2] * dc[:, 2]) - radii
        if d.min() >= 0.5:
            lights.append((float(np.float32(p[0])), float(np.float32(p[1])), float(np.float32(p[2])),
                           light_intensity))
    s.point_lights = lights
    s.ambient = 0.1
    s.sun_intensity = 0.7
    return s.finalize()


def view_for(w: int, h: int, view: np.ndarray, cam: np.ndarray, x: int = 0, y: int = 0, **dof) -> View:
    return View(x, y, w, h, view, projection(w, h), cam, **dof)


def cube_view(w: int = 640, h: int = 480) -> View:
    v, c = camera_at_z(5.0)
    return view_for(w, h, v, c)


def spheres_view(w: int = 1920, h: int = 1080, dist: float = 35.0) -> View:
    v, c = camera_at_z(dist)
    return view_for(w, h, v, c)


def log_uniform_int(rng: Rng, lo: int, hi: int) -> int:
    u = rng.uniform(0.0, 1.0, 1)[0]
    return int(min(hi, math.floor(lo * (hi / lo) ** u)))


def batch_views(n: int = 64, seed: int = 3, radius: float = 35.0, min_wh=(128, 128), max_wh=(1920, 1080)):
    """Seeded cameras on a sphere of `radius` looking at the centre, sizes
    log-uniform per axis between min_wh and max_wh."""
    rng = Rng(seed)
    views = []
    for _ in range(n):
        w = log_uniform_int(rng, min_wh[0], max_wh[0])
        h = log_uniform_int(rng, min_wh[1], max_wh[1])
        v, c = camera_on_sphere(rng, radius)
        views.append(view_for(w, h, v, c))
    return views


def rot_z(a: float) -> np.ndarray:
    """matrix44_t::rotate_z applied to the identity (src/projection/matrix44.cpp:108-125)."""
    s, c = sincos(a)
    m = np.eye(4)
    m[0, 0], m[0, 1], m[1, 0], m[1, 1] = c, s, -s, c
    return m


def mixed_scene(seed: int = 4) -> Scene:
    """Small scene exercising every input feature: a node hierarchy with
    non-uniform scale, triangle fans, strips and lists, a double-sided
    untextured material, a non-square texture and two point lights."""
    rng = Rng(seed)
    s = Scene()
    s.textures.append(texture_uniform(seed, 256, 256))
    s.textures.append(texture_value_noise(seed + 1, 64, octaves=3))
    s.textures.append(texture_uniform(seed + 2, 64, 32))            # non-square
    s.materials.append((0xFFFFFFFF, 0, 0, 32))
    s.materials.append((0xFF3080C0, -1, 1, 32))                     # untextured, double-sided
    s.materials.append((0xFFFFFFFF, 2, 1, 32))                      # non-square texture, double-sided
    s.materials.append((0xFFFFFFFF, 1, 0, 32))
    rot = matmul4(rot_y(0.4), rot_x(-0.3)).astype(np.float32)
    n0 = s.add_node(translation=(-1.2, 0.3, 0.0), rotation=rot, scale=(1.5, 0.7, 1.0))
    for (p, n, t, i) in cube_mesh(1.5):
        s.add_primitive(n0, TRIANGLE_FAN, 0, p, n, t, i)
    n1 = s.add_node(translation=(0.0, 1.2, 0.0), rotation=rot_z(0.6).astype(np.float32), parent=n0)
    for (p, n, t, i) in cube_mesh(0.5):
        s.add_primitive(n1, TRIANGLE_FAN, 1, p, n, t, i)
    # 40 random triangles as one TRIANGLES list
    n2 = s.add_node(translation=(1.3, -0.4, 0.3))
    pos = rng.uniform(-0.8, 0.8, 40 * 9).reshape(120, 3).astype(np.float32)
    nrm = normalize_f32(rng.uniform(-1.0, 1.0, 120 * 3).reshape(120, 3))
    uv = rng.uniform(0.0, 1.0, 240).reshape(120, 2).astype(np.float32)
    s.add_primitive(n2, TRIANGLES, 2, pos, nrm, uv, np.arange(120, dtype=np.uint32))
    n3 = s.add_node(translation=(0.4, 0.9, -1.0))
    for (p, n, t, idx) in uv_sphere_mesh(16, 8, 0.7):
        s.add_primitive(n3, TRIANGLE_STRIP, 3, p, n, t, idx)
    s.point_lights = [(0.5, 2.0, 1.5, 3.0), (-2.0, -0.5, 1.0, 1.5)]
    s.ambient = 0.15
    s.sun_intensity = 0.6
    return s.finalize()


def glass_scene(seed: int = 8) -> Scene:
    """Scene for transparency layers: an opaque textured cube behind stacked
    double-sided sheets and random triangles whose textures have block alpha
    (opaque, clear and translucent squares), a sphere with such a texture,
    and untextured materials whose colours carry alpha (seen by the
    material-colour shader)."""
    rng = Rng(seed)
    s = Scene()
    s.textures.append(texture_uniform(seed, 128, 128))
    s.textures.append(texture_block_alpha(seed + 1, 64, 64, 8))
    s.textures.append(texture_block_alpha(seed + 2, 128, 64, 16))
    s.materials.append((0xFFFFFFFF, 0, 0, 32))   # opaque texture
    s.materials.append((0x80FF4020, 1, 1, 32))   # block alpha, double-sided; colour alpha 128
    s.materials.append((0xC02060FF, 2, 1, 32))   # block alpha (coarser), double-sided; colour alpha 192
    s.materials.append((0x4040FF40, -1, 1, 32))  # untextured, colour alpha 64
    s.materials.append((0xFFFFFF00, -1, 0, 32))  # untextured, opaque colour
    n0 = s.add_node(translation=(0.0, 0.0, -1.5), rotation=matmul4(rot_y(0.5), rot_x(0.4)).astype(np.float32))
    for (p, n, t, i) in cube_mesh(1.6):
        s.add_primitive(n0, TRIANGLE_FAN, 0, p, n, t, i)
    # four stacked sheets (quads as fans), each a little nearer, alternating materials
    for k in range(4):
        z = -0.6 + 0.45 * k
        nk = s.add_node(translation=(0.15 * k - 0.2, 0.1 * k - 0.15, z), rotation=rot_z(0.2 * k).astype(np.float32))
        q = np.array([[-1.1, -0.8, 0.0], [1.1, -0.8, 0.0], [1.1, 0.8, 0.0], [-1.1, 0.8, 0.0]], np.float32)
        nq = np.tile(np.array([0.0, 0.0, 1.0], np.float32), (4, 1))
        uq = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]], np.float32)
        s.add_primitive(nk, TRIANGLE_FAN, 1 + (k % 3), q, nq, uq, np.arange(4, dtype=np.uint32))
    # 30 random triangles through the stack
    n5 = s.add_node(translation=(0.2, 0.0, -0.4))
    pos = rng.uniform(-1.0, 1.0, 30 * 9).reshape(90, 3).astype(np.float32)
    nrm = normalize_f32(rng.uniform(-1.0, 1.0, 90 * 3).reshape(90, 3))
    uv = rng.uniform(0.0, 1.0, 180).reshape(90, 2).astype(np.float32)
    s.add_primitive(n5, TRIANGLES, 2, pos[:45], nrm[:45], uv[:45], np.arange(45, dtype=np.uint32))
    s.add_primitive(n5, TRIANGLES, 4, pos[45:60], nrm[45:60], uv[45:60], np.arange(15, dtype=np.uint32))
    s.add_primitive(n5, TRIANGLES, 1, pos[60:], nrm[60:], uv[60:], np.arange(30, dtype=np.uint32))
    n6 = s.add_node(translation=(-0.9, 0.6, 0.3))
    for (p, n, t, idx) in uv_sphere_mesh(12, 6, 0.5):
        s.add_primitive(n6, TRIANGLE_STRIP, 1, p, n, t, idx)
    s.point_lights = [(0.5, 1.5, 2.0, 2.5)]
    s.ambient = 0.2
    s.sun_intensity = 0.6
    return s.finalize()


def clip_view(scene: Scene, sphere: int = 0, w: int = 320, h: int = 240, inside: float = 0.97) -> View:
    """Camera just inside sphere `sphere`'s surface, looking at its centre:
    the near plane cuts through many of its triangles."""
    c = np.asarray(scene.node_translation[sphere], np.float64)
    # radius of the sphere mesh = |first vertex of its first strip|
    prim = [p for p in scene.primitives if p[0] == sphere][0]
    v = np.asarray(scene.positions[prim[3]], np.float64)
    r = math.sqrt(_dot3(v, v))
    pos = c + np.array([0.0, 0.0, r * inside])
    m, _ = look_at_origin(pos - c)
    m = m.astype(np.float64)
    for i in range(3):
        m[i, 3] = -_dot3(m[i, :3], pos)
    return view_for(w, h, m.astype(np.float32), pos.astype(np.float32))


def look_at(position, target) -> tuple[np.ndarray, np.ndarray]:
    """View matrix of a camera at `position` looking at `target`."""
    pos = np.asarray(position, np.float64)
    m, _ = look_at_origin(pos - np.asarray(target, np.float64))
    m = m.astype(np.float64)
    for i in range(3):
        m[i, 3] = -_dot3(m[i, :3], pos)
    return m.astype(np.float32), pos.astype(np.float32)


def grid_scene(n: int = 40, extent: float = 10.0, seed: int = 6) -> Scene:
    """A textured n x n floor of quads (TRIANGLES list) at y = -0.5; with a
    camera standing on it many triangles cross the near plane."""
    s = Scene()
    s.textures.append(texture_value_noise(seed, 128, octaves=3))
    s.materials.append((0xFFFFFFFF, 0, 0, 32))
    node = s.add_node()
    g = np.arange(n + 1, dtype=np.float64)
    xs = (-extent + 2.0 * extent * g / n)
    X, Z = np.meshgrid(xs, xs)
    pos = np.stack([X, np.full_like(X, -0.5), Z], -1).reshape(-1, 3).astype(np.float32)
    uv = np.stack(np.meshgrid(g / n, g / n), -1).reshape(-1, 2).astype(np.float32)
    nrm = np.tile(np.array([0.0, 1.0, 0.0], np.float32), (len(pos), 1))
    idx = []
    for j in range(n):
        for i in range(n):
            a, b, c, d = j * (n + 1) + i, j * (n + 1) + i + 1, (j + 1) * (n + 1) + i, (j + 1) * (n + 1) + i + 1
            idx += [a, c, b, b, c, d]
    s.add_primitive(node, TRIANGLES, 0, pos, nrm, uv, np.asarray(idx, np.uint32))
    s.point_lights = [(0.0, 1.0, -3.0, 2.0)]
    return s.finalize()


def mixed_size_scene(seed: int = 7) -> Scene:
    """A floor of one 3,200-triangle list (beyond the fused geometry pass's
    primitive limits) with three cubes and a sphere standing on it (within
    them): a scene whose primitives take both geometry passes."""
    s = Scene()
    s.textures.append(texture_value_noise(seed, 128, octaves=3))
    s.textures.append(texture_uniform(seed + 1, 64, 64))
    s.materials.append((0xFFFFFFFF, 0, 0, 32))
    s.materials.append((0xFFFFFFFF, 1, 1, 48))
    floor = s.add_node()
    n, extent = 40, 10.0
    g = np.arange(n + 1, dtype=np.float64)
    xs = (-extent + 2.0 * extent * g / n)
    X, Z = np.meshgrid(xs, xs)
    pos = np.stack([X, np.full_like(X, -0.5), Z], -1).reshape(-1, 3).astype(np.float32)
    uv = np.stack(np.meshgrid(g / n, g / n), -1).reshape(-1, 2).astype(np.float32)
    nrm = np.tile(np.array([0.0, 1.0, 0.0], np.float32), (len(pos), 1))
    idx = []
    for j in range(n):
        for i in range(n):
            a, b, c, d = j * (n + 1) + i, j * (n + 1) + i + 1, (j + 1) * (n + 1) + i, (j + 1) * (n + 1) + i + 1
            idx += [a, c, b, b, c, d]
    s.add_primitive(floor, TRIANGLES, 0, pos, nrm, uv, np.asarray(idx, np.uint32))
    for k, (x, z) in enumerate(((-1.5, -2.0), (1.0, -1.0), (0.0, -3.5))):
        nk = s.add_node(translation=(x, -0.1, z), rotation=rot_y(0.3 * k + 0.2).astype(np.float32))
        for (p, nm, t, i) in cube_mesh(0.8):
            s.add_primitive(nk, TRIANGLE_FAN, 1, p, nm, t, i)
    ns = s.add_node(translation=(0.5, 0.2, -2.2))
    for (p, nm, t, i) in uv_sphere_mesh(16, 8, 0.7):
        s.add_primitive(ns, TRIANGLE_STRIP, 1, p, nm, t, i)
    s.point_lights = [(0.0, 1.5, -1.0, 3.0), (-2.0, 1.0, 1.0, 2.0)]
    return s.finalize()


SERVE_TRIANGLES = (10_000, 50_000, 100_000, 250_000, 500_000, 800_000, 1_200_000, 2_000_000)


def serving_scenes(seed: int = 50, tex_size: int = 1024):
    """Eight scenes built like the 200-sphere scene with ceil(T / 4096) spheres
    for T in SERVE_TRIANGLES; they share one set of 8 value-noise textures."""
    textures = [texture_value_noise(seed * 1000 + t, tex_size) for t in range(8)]
    out = []
    for k, t in enumerate(SERVE_TRIANGLES):
        n = -(-t // 4096)
        out.append(spheres_scene(n_spheres=n, seed=seed + 1 + k, textures=textures))
    return out


def serving_requests(n: int, seed: int = 60, rate: float = 2000.0, n_scenes: int = 8, radius: float = 35.0,
                     min_wh=(64, 64), max_wh=(3840, 2160), dof_p: float = 0.5):
    """A seeded request stream: Poisson arrivals at `rate`/s, a uniform scene,
    a camera on a sphere of `radius`, viewport sides log-uniform between
    min_wh and max_wh, depth of field with probability dof_p (focus 20,
    aperture 0.05, at most 16 px).  Returns [(arrival_s, scene_index, View)].

    Request i takes draws 7i ... 7i + 6 of the stream `seed`, in this order:
    inter-arrival time, scene, width, height, camera z, camera yaw, depth of
    field.  The draws are made in one vectorised pass (the same counter-hash
    values a draw-at-a-time Rng would give)."""
    rng = Rng(seed)
    bits = rng.bits(7 * n).reshape(n, 7) if n > 0 else np.zeros((0, 7), np.uint64)
    u = (bits >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    scene = (bits[:, 1] % np.uint64(n_scenes)).astype(np.int64)
    cz = -1.0 + 2.0 * u[:, 4]
    yaw = 0.0 + (2.0 * math.pi - 0.0) * u[:, 5]
    sy, cy = sincos(yaw)
    t = 0.0
    out = []
    for i in range(n):
        t += -math.log(1.0 - float(u[i, 0])) / rate
        w = int(min(max_wh[0], math.floor(min_wh[0] * (max_wh[0] / min_wh[0]) ** u[i, 2])))
        h = int(min(max_wh[1], math.floor(min_wh[1] * (max_wh[1] / min_wh[1]) ** u[i, 3])))
        m, c = _camera_at(float(cz[i]), float(sy[i]), float(cy[i]), radius)
        v = view_for(w, h, m, c)
        v.dof = bool(u[i, 6] < dof_p)
        out.append((t, int(scene[i]), v))
    return out
