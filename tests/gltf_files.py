"""Writers of synthetic glTF / GLB scenes and PNG / BMP images for the
loader tests (no third-party encoder is available: PNG uses the standard
library's zlib, the rest is plain packing)."""
from __future__ import annotations

import base64
import json
import math
import os
import struct
import zlib

import numpy as np

# --------------------------------------------------------------------- PNG --
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _chunk(kind: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _pack_row(samples: np.ndarray, depth: int) -> bytes:
    """One row of samples (already interleaved by channel) at `depth` bits."""
    if depth == 16:
        return samples.astype(">u2").tobytes()
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    per = 8 // depth
    n = len(samples)
    out = bytearray((n * depth + 7) // 8)
    for i, v in enumerate(samples):
        out[i // per] |= (int(v) & ((1 << depth) - 1)) << (8 - depth * (i % per + 1))
    return bytes(out)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter(rows, bpp, rng):
    out = bytearray()
    prev = bytes(len(rows[0])) if rows else b""
    for row in rows:
        f = int(rng.integers(0, 5))
        fr = bytearray(len(row))
        for i in range(len(row)):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][f]
            fr[i] = (row[i] - pred) & 0xFF
        out += bytes([f]) + fr
        prev = row
    return bytes(out)


def encode_png(samples: np.ndarray, ctype: int, depth: int, interlace: bool = False, palette=None, trns=None,
               seed: int = 0) -> bytes:
    """samples: (h, w, channels) integers at `depth`; rows filtered with
    random filter types."""
    h, w, ch = samples.shape
    rng = np.random.default_rng(seed)
    bpp = max(1, ch * depth // 8)
    raw = b""
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    for (x0, y0, dx, dy) in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        rows = [_pack_row(sub[y].reshape(-1), depth) for y in range(sub.shape[0])]
        raw += _filter(rows, bpp, rng)
    out = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 1 if interlace else 0))
    if palette is not None:
        out += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        out += _chunk(b"tRNS", bytes(trns))
    comp = zlib.compress(raw, 6)
    # split the stream over two IDAT chunks
    out += _chunk(b"IDAT", comp[:len(comp) // 2]) + _chunk(b"IDAT", comp[len(comp) // 2:])
    return out + _chunk(b"IEND", b"")


def png_expected(samples, ctype, depth, palette=None, trns=None) -> np.ndarray:
    """The texels libpng's transforms in read_png_file give (image.cpp:119-166):
    8-bit RGBA, 16-bit samples to their high byte, low-depth grey scaled up,
    tRNS to alpha, grey replicated; then 0xAARRGGBB."""
    s = samples.astype(np.uint32)
    h, w, _ = s.shape

    def to8(v):
        return {1: v * 255, 2: v * 85, 4: v * 17, 8: v, 16: v >> 8}[depth]

    a = np.full((h, w), 255, np.uint32)
    if ctype == 3:
        pal = np.asarray(palette, np.uint32)
        rgb = pal[s[..., 0]]
        if trns is not None:
            ta = np.full(len(pal), 255, np.uint32)
            ta[:len(trns)] = list(trns)
            a = ta[s[..., 0]]
        r, g, b = rgb[..., 0], rgb[..., 1], rgb[..., 2]
    elif ctype in (0, 4):
        r = g = b = to8(s[..., 0])
        if ctype == 4:
            a = to8(s[..., 1])
        elif trns is not None:
            key = (trns[0] << 8) | trns[1]
            a = np.where(s[..., 0] == key, 0, 255).astype(np.uint32)
    else:
        r, g, b = to8(s[..., 0]), to8(s[..., 1]), to8(s[..., 2])
        if ctype == 6:
            a = to8(s[..., 3])
        elif trns is not None:
            kr, kg, kb = (trns[0] << 8) | trns[1], (trns[2] << 8) | trns[3], (trns[4] << 8) | trns[5]
            a = np.where((s[..., 0] == kr) & (s[..., 1] == kg) & (s[..., 2] == kb), 0, 255).astype(np.uint32)
    return ((a << 24) | (r << 16) | (g << 8) | b).astype(np.uint32)


# --------------------------------------------------------------------- BMP --
def encode_bmp(rgb: np.ndarray) -> bytes:
    """A standard bottom-up 24-bit BMP (rows padded to 4 bytes)."""
    h, w, _ = rgb.shape
    pad = (4 - (w * 3) % 4) % 4
    body = b""
    for y in range(h - 1, -1, -1):
        body += rgb[y, :, ::-1].astype(np.uint8).tobytes() + b"\0" * pad
    hdr = struct.pack("<2sIHHI", b"BM", 54 + len(body), 0, 0, 54)
    info = struct.pack("<IiiHHIIiiII", 40, w, h, 1, 24, 0, len(body), 2835, 2835, 0, 0)
    return hdr + info + body


# -------------------------------------------------------------------- glTF --
class GltfBuilder:
    """Accumulates buffer views and accessors in one binary buffer."""

    def __init__(self):
        self.bin = bytearray()
        self.j = {"asset": {"version": "2.0"}, "bufferViews": [], "accessors": [], "meshes": [], "nodes": [],
                  "materials": [], "textures": [], "images": [], "animations": []}

    def view(self, data: bytes, stride: int = 0) -> int:
        while len(self.bin) % 4:
            self.bin += b"\0"
        bv = {"buffer": 0, "byteOffset": len(self.bin), "byteLength": len(data)}
        if stride:
            bv["byteStride"] = stride
        self.bin += data
        self.j["bufferViews"].append(bv)
        return len(self.j["bufferViews"]) - 1

    def accessor(self, arr: np.ndarray, ctype: int, typ: str, stride: int = 0, offset: int = 0) -> int:
        data = np.ascontiguousarray(arr).tobytes()
        if stride:
            # interleave: element i at i * stride
            esz = arr.dtype.itemsize * (arr.shape[1] if arr.ndim > 1 else 1)
            buf = bytearray(stride * len(arr))
            for i in range(len(arr)):
                buf[i * stride:i * stride + esz] = np.ascontiguousarray(arr[i]).tobytes()
            data = bytes(buf)
        bvi = self.view(b"\0" * offset + data, stride)
        a = {"bufferView": bvi, "componentType": ctype, "count": len(arr), "type": typ}
        if offset:
            a["byteOffset"] = offset
        self.j["accessors"].append(a)
        return len(self.j["accessors"]) - 1

    def write(self, path: str, glb: bool, external_bin: bool = False):
        j = dict(self.j)
        j = {k: v for k, v in j.items() if v != []}
        if glb:
            j["buffers"] = [{"byteLength": len(self.bin)}]
            js = json.dumps(j).encode()
            js += b" " * ((4 - len(js) % 4) % 4)
            binb = bytes(self.bin) + b"\0" * ((4 - len(self.bin) % 4) % 4)
            total = 12 + 8 + len(js) + 8 + len(binb)
            out = struct.pack("<4sII", b"glTF", 2, total) + struct.pack("<I4s", len(js), b"JSON") + js
            out += struct.pack("<I4s", len(binb), b"BIN\0") + binb
            with open(path, "wb") as fh:
                fh.write(out)
        else:
            if external_bin:
                name = os.path.splitext(os.path.basename(path))[0] + ".bin"
                with open(os.path.join(os.path.dirname(path), name), "wb") as fh:
                    fh.write(bytes(self.bin))
                j["buffers"] = [{"byteLength": len(self.bin), "uri": name}]
            else:
                j["buffers"] = [{"byteLength": len(self.bin),
                                 "uri": "data:application/octet-stream;base64," + base64.b64encode(bytes(self.bin)).decode()}]
            with open(path, "w") as fh:
                json.dump(j, fh)


def quat(axis, angle):
    ax = np.asarray(axis, np.float64)
    ax = ax / np.linalg.norm(ax)
    s = math.sin(angle / 2)
    return [float(ax[0] * s), float(ax[1] * s), float(ax[2] * s), float(math.cos(angle / 2))]


def _cube(size):
    from swegl_gb300 import scenes as S

    return S.cube_mesh(size)


def build_test_scene(dirpath: str, glb: bool, seed: int = 3) -> str:
    """A scene exercising the loader: a node hierarchy with TRS, quaternion
    and matrix nodes; fans, strips and lists with 16- and 32-bit indices and
    an interleaved vertex buffer; a mesh without primitives and a mesh used
    twice; materials with and without pbrMetallicRoughness, base colours,
    double sides and textures (a PNG in a buffer view or as a data URI, an
    external PNG and BMP); translation, rotation and scale animations."""
    from swegl_gb300 import scenes as S

    rng = np.random.default_rng(seed)
    g = GltfBuilder()
    # images
    tex_a = rng.integers(0, 256, size=(32, 48, 4)).astype(np.uint8)
    tex_a[..., 3] = 255
    png_a = encode_png(tex_a, 6, 8, seed=1)
    tex_b = rng.integers(0, 256, size=(16, 16, 3)).astype(np.uint8)
    png_b = encode_png(tex_b, 2, 8, interlace=True, seed=2)
    tex_c = rng.integers(0, 256, size=(8, 10, 3)).astype(np.uint8)
    with open(os.path.join(dirpath, "tex_c.bmp"), "wb") as fh:
        fh.write(encode_bmp(tex_c))
    with open(os.path.join(dirpath, "tex_b.png"), "wb") as fh:
        fh.write(png_b)
    if glb:
        g.j["images"].append({"bufferView": g.view(png_a), "mimeType": "image/png"})
    else:
        g.j["images"].append({"uri": "data:image/png;base64," + base64.b64encode(png_a).decode()})
    g.j["images"].append({"uri": "tex_b.png"})
    g.j["images"].append({"uri": "tex_c.bmp"})
    g.j["textures"] = [{"source": 2}, {"source": 0}, {"source": 1}]
    g.j["materials"] = [
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 1}}},
        {"pbrMetallicRoughness": {"baseColorFactor": [0.8, 0.3, 0.1, 1.0]}, "doubleSided": True},
        {"doubleSided": True},  # no pbr: white, single-sided
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 2}, "metallicFactor": 0.5}, "doubleSided": True},
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "roughnessFactor": 0.2}},
    ]
    meshes = []
    # mesh 0: the cube's six fans, 16-bit indices
    prims = []
    for k, (p, n, t, i) in enumerate(_cube(1.2)):
        prims.append({"attributes": {"POSITION": g.accessor(p, 5126, "VEC3"), "NORMAL": g.accessor(n, 5126, "VEC3"),
                                     "TEXCOORD_0": g.accessor(t, 5126, "VEC2")},
                      "indices": g.accessor(i.astype(np.uint16), 5123, "SCALAR"), "mode": 6, "material": k % 2 * 4})
    meshes.append({"primitives": prims})
    meshes.append({"name": "empty"})  # no primitives: skipped when meshes are numbered
    # mesh 2 (loader index 1): a UV sphere as strips, 32-bit indices, interleaved positions
    prims = []
    for (p, n, t, i) in S.uv_sphere_mesh(12, 6, 0.6):
        prims.append({"attributes": {"POSITION": g.accessor(p, 5126, "VEC3", stride=24),
                                     "NORMAL": g.accessor(n, 5126, "VEC3", offset=8),
                                     "TEXCOORD_0": g.accessor(t, 5126, "VEC2")},
                      "indices": g.accessor(i.astype(np.uint32), 5125, "SCALAR"), "mode": 5, "material": 3})
    meshes.append({"primitives": prims})
    # mesh 3 (loader index 2): random triangles, one list without normals, one without indices, one of lines
    p = rng.uniform(-0.7, 0.7, size=(30, 3)).astype(np.float32)
    t = rng.uniform(0, 1, size=(30, 2)).astype(np.float32)
    meshes.append({"primitives": [
        {"attributes": {"POSITION": g.accessor(p, 5126, "VEC3"), "TEXCOORD_0": g.accessor(t, 5126, "VEC2")},
         "indices": g.accessor(np.arange(30, dtype=np.uint16)[::-1].copy(), 5123, "SCALAR"), "material": 1},
        {"attributes": {"POSITION": g.accessor(p, 5126, "VEC3")}, "material": 0},
        {"attributes": {"POSITION": g.accessor(p, 5126, "VEC3")}, "indices": g.accessor(np.arange(6, dtype=np.uint16), 5123, "SCALAR"),
         "mode": 1},
    ]})
    # mesh 4 (loader index 3): a quad fan with the untextured no-pbr material
    q = np.array([[-2, -2, -1.5], [2, -2, -1.5], [2, 2, -1.5], [-2, 2, -1.5]], np.float32)
    meshes.append({"primitives": [{"attributes": {"POSITION": g.accessor(q, 5126, "VEC3"),
                                                  "NORMAL": g.accessor(np.tile([[0, 0, 1]], (4, 1)).astype(np.float32), 5126, "VEC3")},
                                   "indices": g.accessor(np.arange(4, dtype=np.uint16), 5123, "SCALAR"),
                                   "mode": 6, "material": 2}]})
    g.j["meshes"] = meshes
    m = np.eye(4)
    m[:3, :3] = np.diag([1.2, 0.8, 1.0]) @ np.array([[0.8, -0.6, 0], [0.6, 0.8, 0], [0, 0, 1]])
    m[:3, 3] = [0.9, -0.4, 0.2]
    g.j["nodes"] = [
        {"children": [1, 2], "translation": [0.0, 0.1, -0.5], "rotation": quat([0, 1, 0], 0.4)},
        {"mesh": 0, "translation": [-1.0, 0.0, 0.0], "scale": [1.0, 0.9, 1.1], "rotation": quat([1, 1, 0], 0.3)},
        {"mesh": 1, "matrix": [float(v) for v in m.T.reshape(-1)], "children": [3]},
        {"mesh": 2, "translation": [0.3, 0.6, 0.4]},
        {"mesh": 0, "translation": [1.5, 1.5, 0.0]},  # mesh 0 again: no primitives
        {"mesh": 3},
    ]
    times = np.array([0.0, 0.5, 1.25, 2.0], np.float32)
    tr = np.array([[-1.0, 0, 0], [-1.2, 0.3, 0], [-0.8, -0.2, 0.1], [-1.0, 0, 0]], np.float32)
    rot = np.array([quat([0, 1, 0], a) for a in (0.0, 1.0, 2.5, 0.2)], np.float32)
    sc = np.array([[1, 1, 1], [1.3, 1.0, 0.7]], np.float32)
    ti, tt, tr_, ts = (g.accessor(times, 5126, "SCALAR"), g.accessor(times[:2].copy(), 5126, "SCALAR"),
                       g.accessor(rot, 5126, "VEC4"), g.accessor(sc, 5126, "VEC3"))
    g.j["animations"] = [
        {"samplers": [{"input": ti, "output": g.accessor(tr, 5126, "VEC3")}, {"input": ti, "output": tr_}],
         "channels": [{"sampler": 0, "target": {"node": 1, "path": "translation"}},
                      {"sampler": 1, "target": {"node": 3, "path": "rotation"}}]},
        {"samplers": [{"input": tt, "output": ts}],
         "channels": [{"sampler": 0, "target": {"node": 0, "path": "scale"}}]},
    ]
    path = os.path.join(dirpath, "scene.glb" if glb else "scene.gltf")
    g.write(path, glb, external_bin=not glb and seed % 2 == 1)
    return path


# -------------------------------------------------------------------- JPEG --
ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20,
                   13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52,
                   45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])


def _dct_matrix():
    c = np.zeros((8, 8))
    for k in range(8):
        for n in range(8):
            c[k, n] = (math.sqrt(0.125) if k == 0 else 0.5) * math.cos((2 * n + 1) * k * math.pi / 16)
    return c


def _huff_lengths(freq: dict) -> dict:
    """Code lengths <= 16 with no all-ones code (a reserved dummy symbol,
    then the length adjustment of T.81 Annex K.2)."""
    import heapq

    syms = dict(freq)
    syms[256] = 1  # reserved
    heap = [(f, i, [s]) for i, (s, f) in enumerate(sorted(syms.items()))]
    heapq.heapify(heap)
    depth = {s: 0 for s in syms}
    if len(heap) == 1:
        depth[heap[0][2][0]] = 1
    cnt = len(heap)
    while len(heap) > 1:
        f1, _, a = heapq.heappop(heap)
        f2, _, b = heapq.heappop(heap)
        for s in a + b:
            depth[s] += 1
        cnt += 1
        heapq.heappush(heap, (f1 + f2, cnt, a + b))
    bits = [0] * 40
    for s, d in depth.items():
        bits[d] += 1
    for i in range(39, 16, -1):
        while bits[i] > 0:
            j = i - 2
            while bits[j] == 0:
                j -= 1
            bits[i] -= 2
            bits[i - 1] += 1
            bits[j + 1] += 2
            bits[j] -= 1
    i = 16
    while bits[i] == 0:
        i -= 1
    bits[i] -= 1  # drop the reserved symbol's code
    order = sorted(freq, key=lambda s: (-freq[s], s))
    lengths, k = {}, 0
    for L in range(1, 17):
        for _ in range(bits[L]):
            lengths[order[k]] = L
            k += 1
    return lengths


def _canonical(lengths: dict):
    """DHT body (counts, values) and the code of each symbol."""
    order = sorted(lengths, key=lambda s: (lengths[s], s))
    counts = [0] * 16
    for s in order:
        counts[lengths[s] - 1] += 1
    codes, code, prev = {}, 0, 0
    for s in order:
        code <<= lengths[s] - prev
        prev = lengths[s]
        codes[s] = (code, lengths[s])
        code += 1
    return counts, order, codes


def _cat(v: int) -> int:
    return 0 if v == 0 else int(abs(v)).bit_length()


def _jpeg_coefficients(rgb: np.ndarray, sampling, quality: int, grey: bool):
    """The quantised DCT coefficients of an (h, w, 3) uint8 image as a JFIF
    encoder makes them: YCbCr, luma sampled `sampling` (h, v) times the
    chroma, float DCT, scaled standard-shaped quantisers."""
    h, w, _ = rgb.shape
    f = rgb.astype(np.float64)
    y = 0.299 * f[..., 0] + 0.587 * f[..., 1] + 0.114 * f[..., 2]
    cb = -0.168736 * f[..., 0] - 0.331264 * f[..., 1] + 0.5 * f[..., 2] + 128
    cr = 0.5 * f[..., 0] - 0.418688 * f[..., 1] - 0.081312 * f[..., 2] + 128
    planes = [y] if grey else [y, cb, cr]
    hs, vs = (1, 1) if grey else sampling
    factors = [(hs, vs)] + [(1, 1)] * (len(planes) - 1)
    hmax, vmax = hs, vs
    mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
    base_l = np.array([16, 11, 10, 16, 24, 40, 51, 61] * 8).reshape(8, 8) * 0 + np.add.outer(np.arange(8), np.arange(8)) * 6 + 8
    scale = 5000 / quality if quality < 50 else 200 - 2 * quality
    q_l = np.clip((base_l * scale + 50) // 100, 1, 255).astype(np.int64)
    q_c = np.clip(((base_l + 10) * scale + 50) // 100, 1, 255).astype(np.int64)
    qts = [q_l, q_c]
    C = _dct_matrix()
    comps = []
    for k, (pl, (ch, cv)) in enumerate(zip(planes, factors)):
        dw, dh = -(-w * ch // hmax), -(-h * cv // vmax)
        sx, sy = hmax // ch, vmax // cv
        pad = np.pad(pl, ((0, dh * sy - h), (0, dw * sx - w)), mode="edge")
        ds = pad.reshape(dh, sy, dw, sx).mean(axis=(1, 3))
        ds = np.clip(np.round(ds), 0, 255)
        bw, bh = mcux * ch, mcuy * cv
        full = np.pad(ds, ((0, bh * 8 - dh), (0, bw * 8 - dw)), mode="edge") - 128
        blocks = full.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3)
        coef = np.einsum("ij,abjk,lk->abil", C, blocks, C)
        qt = qts[0 if k == 0 else 1]
        qc = np.round(coef / qt).astype(np.int64)
        comps.append(dict(id=k + 1, h=ch, v=cv, tq=0 if k == 0 else 1, coef=qc, bw=bw, bh=bh, dw=dw, dh=dh))
    return dict(h=h, w=w, comps=comps, qts=qts, hmax=hmax, vmax=vmax, mcux=mcux, mcuy=mcuy)


def _jpeg_header(out: bytearray, cf: dict, sof_marker: int, ntab: int):
    """SOI, JFIF, quantisation tables and the frame header."""
    out += b"\xff\xd8"
    out += b"\xff\xe0" + struct.pack(">H", 16) + b"JFIF\0" + bytes([1, 1, 0, 0, 1, 0, 1, 0, 0])
    for t in range(ntab):
        out += b"\xff\xdb" + struct.pack(">H", 67) + bytes([t]) + bytes(cf["qts"][t].reshape(-1)[ZIGZAG].astype(np.uint8))
    sof = bytes([8]) + struct.pack(">HH", cf["h"], cf["w"]) + bytes([len(cf["comps"])])
    for c in cf["comps"]:
        sof += bytes([c["id"], (c["h"] << 4) | c["v"], c["tq"]])
    out += bytes([0xFF, sof_marker]) + struct.pack(">H", 2 + len(sof)) + sof


def encode_jpeg(rgb: np.ndarray, sampling=(2, 2), quality: int = 80, restart: int = 0, grey: bool = False,
                interleaved: bool = True):
    """A baseline JPEG of an (h, w, 3) uint8 image: JFIF YCbCr, luma sampled
    `sampling` (h, v) times the chroma, float DCT, scaled standard-shaped
    quantisers, per-file Huffman tables, optional restart interval and
    separate scans per component.  Returns (bytes, info) with the quantised
    coefficients of every block (natural order) for checking."""
    cf = _jpeg_coefficients(rgb, sampling, quality, grey)
    h, w, comps, qts = cf["h"], cf["w"], cf["comps"], cf["qts"]
    hmax, vmax, mcux, mcuy = cf["hmax"], cf["vmax"], cf["mcux"], cf["mcuy"]
    # symbols per scan
    scans = [list(range(len(comps)))] if interleaved else [[k] for k in range(len(comps))]
    seqs = []  # per scan: list of (component, (by, bx)) in coding order, with restart flags
    for sc in scans:
        seq = []
        if len(sc) > 1:
            for my in range(mcuy):
                for mx in range(mcux):
                    seq.append([(k, my * comps[k]["v"] + v, mx * comps[k]["h"] + hh) for k in sc
                                for v in range(comps[k]["v"]) for hh in range(comps[k]["h"])])
        else:
            c = comps[sc[0]]
            for by in range(-(-c["dh"] // 8)):
                for bx in range(-(-c["dw"] // 8)):
                    seq.append([(sc[0], by, bx)])
        seqs.append(seq)
    dc_freq = [dict(), dict()]
    ac_freq = [dict(), dict()]
    coded = []  # per scan, per MCU: list of (table, [(sym, bits, nbits)...])
    for seq in seqs:
        pred = {}
        out_scan = []
        for n, mcu in enumerate(seq):
            if restart and n % restart == 0:
                pred = {}
            items = []
            for (k, by, bx) in mcu:
                c = comps[k]
                t = 0 if k == 0 else 1
                zz = c["coef"][by, bx].reshape(-1)[ZIGZAG]
                diff = int(zz[0]) - pred.get(k, 0)
                pred[k] = int(zz[0])
                s = _cat(diff)
                dc_freq[t][s] = dc_freq[t].get(s, 0) + 1
                syms = [("dc", t, s, diff)]
                run = 0
                last = max([i for i in range(1, 64) if zz[i] != 0], default=0)
                for i in range(1, last + 1):
                    v = int(zz[i])
                    if v == 0:
                        run += 1
                        continue
                    while run > 15:
                        syms.append(("ac", t, 0xF0, 0))
                        ac_freq[t][0xF0] = ac_freq[t].get(0xF0, 0) + 1
                        run -= 16
                    rs = (run << 4) | _cat(v)
                    syms.append(("ac", t, rs, v))
                    ac_freq[t][rs] = ac_freq[t].get(rs, 0) + 1
                    run = 0
                if last < 63:
                    syms.append(("ac", t, 0x00, 0))
                    ac_freq[t][0] = ac_freq[t].get(0, 0) + 1
                items.extend(syms)
            out_scan.append(items)
        coded.append(out_scan)
    ntab = 1 if grey else 2
    dc_codes, ac_codes, dht = [], [], b""
    for t in range(ntab):
        for cls, freq, store in ((0, dc_freq[t], dc_codes), (1, ac_freq[t], ac_codes)):
            counts, order, codes = _canonical(_huff_lengths(freq))
            store.append(codes)
            body = bytes([(cls << 4) | t]) + bytes(counts) + bytes(order)
            dht += b"\xff\xc4" + struct.pack(">H", 2 + len(body)) + body
    out = bytearray()
    _jpeg_header(out, cf, 0xC0, ntab)
    out += dht
    if restart:
        out += b"\xff\xdd" + struct.pack(">HH", 4, restart)
    for sc, scan in zip(scans, coded):
        sos = bytes([len(sc)])
        for k in sc:
            t = 0 if k == 0 else 1
            sos += bytes([comps[k]["id"], (t << 4) | t])
        sos += bytes([0, 63, 0])
        out += b"\xff\xda" + struct.pack(">H", 2 + len(sos)) + sos
        acc, nacc = 0, 0
        data = bytearray()

        def put(code, n):
            nonlocal acc, nacc
            acc = (acc << n) | code
            nacc += n
            while nacc >= 8:
                byte = (acc >> (nacc - 8)) & 0xFF
                data.append(byte)
                if byte == 0xFF:
                    data.append(0)
                nacc -= 8
            acc &= (1 << nacc) - 1 if nacc else 0

        def flush():
            nonlocal acc, nacc
            if nacc:
                put((1 << (8 - nacc)) - 1, 8 - nacc)

        for n, items in enumerate(scan):
            if restart and n and n % restart == 0:
                flush()
                data += bytes([0xFF, 0xD0 + ((n // restart - 1) % 8)])
            for (kind, t, sym, val) in items:
                code, ln = (dc_codes if kind == "dc" else ac_codes)[t][sym]
                put(code, ln)
                s = sym if kind == "dc" else (sym & 15)
                if s:
                    put(val if val > 0 else val + (1 << s) - 1, s)
        flush()
        out += data
    out += b"\xff\xd9"
    info = dict(width=w, height=h, comps=comps, qts=qts, hmax=hmax, vmax=vmax)
    return bytes(out), info


class _BitWriter:
    """An entropy-coded segment: bits MSB first, 0xFF bytes stuffed."""

    def __init__(self):
        self.data = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, code: int, n: int):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((code >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.data.append(self.acc)
                if self.acc == 0xFF:
                    self.data.append(0)
                self.acc = self.n = 0

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)


def _bits_of(v: int, s: int) -> int:
    return v if v > 0 else v + (1 << s) - 1


def encode_jpeg_progressive(rgb: np.ndarray, sampling=(2, 2), quality: int = 80, restart: int = 0,
                            grey: bool = False):
    """The same coefficients as encode_jpeg, written as a progressive JPEG
    (SOF2, ITU T.81 Annex G): a DC scan of all components with a point
    transform of 1, its refinement; for luma AC bands 1..5 and 6..63 with a
    point transform of 2 and two refinement scans; for chroma one AC band
    1..63 with a point transform of 1 and one refinement.  End-of-band runs
    span blocks (up to 32767), refinement scans send correction bits for the
    coefficients already nonzero, and each scan has its own Huffman tables.
    Returns (bytes, info) like encode_jpeg."""
    cf = _jpeg_coefficients(rgb, sampling, quality, grey)
    comps = cf["comps"]
    nc = len(comps)
    scans = [(list(range(nc)), 0, 0, 0, 1), (list(range(nc)), 0, 0, 1, 0),
             ([0], 1, 5, 0, 2), ([0], 6, 63, 0, 2)]
    scans += [([k], 1, 63, 0, 1) for k in range(1, nc)]
    scans += [([0], 1, 63, 2, 1), ([0], 1, 63, 1, 0)]
    scans += [([k], 1, 63, 1, 0) for k in range(1, nc)]
    out = bytearray()
    _jpeg_header(out, cf, 0xC2, 1 if grey else 2)
    if restart:
        out += b"\xff\xdd" + struct.pack(">HH", 4, restart)

    def blocks_of(sc):
        """Coding units: MCUs of an interleaved scan, blocks of one component."""
        if len(sc) > 1:
            return [[(k, my * comps[k]["v"] + v, mx * comps[k]["h"] + hh) for k in sc
                     for v in range(comps[k]["v"]) for hh in range(comps[k]["h"])]
                    for my in range(cf["mcuy"]) for mx in range(cf["mcux"])]
        c = comps[sc[0]]
        return [[(sc[0], by, bx)] for by in range(-(-c["dh"] // 8)) for bx in range(-(-c["dw"] // 8))]

    for sc, ss, se, ah, al in scans:
        units = blocks_of(sc)
        ev = []  # per unit: events ("sym", table, symbol) or ("bits", value, n) or ("rst",)
        state = {"eobrun": 0, "be": []}
        table = lambda k: 0 if k == 0 else 1

        def emit_eob(out_ev, t):
            if state["eobrun"]:
                r = state["eobrun"].bit_length() - 1
                out_ev.append(("sym", t, r << 4))
                if r:
                    out_ev.append(("bits", state["eobrun"] - (1 << r), r))
                for bit in state["be"]:
                    out_ev.append(("bits", bit, 1))
                state["eobrun"], state["be"] = 0, []

        pred = {}
        for n, unit in enumerate(units):
            u = []
            if restart and n and n % restart == 0:
                if ss:
                    emit_eob(u, table(sc[0]))
                u.append(("rst",))
                pred = {}
            for (k, by, bx) in unit:
                zz = comps[k]["coef"][by, bx].reshape(-1)[ZIGZAG]
                t = table(k)
                if ss == 0 and ah == 0:
                    dc = int(zz[0]) >> al
                    diff = dc - pred.get(k, 0)
                    pred[k] = dc
                    s = _cat(diff)
                    u.append(("sym", t, s))
                    if s:
                        u.append(("bits", _bits_of(diff, s), s))
                elif ss == 0:
                    u.append(("bits", (int(zz[0]) >> al) & 1, 1))
                elif ah == 0:
                    vals = [int(np.sign(v)) * (abs(int(v)) >> al) for v in zz[ss:se + 1]]
                    r = 0
                    for v in vals:
                        if v == 0:
                            r += 1
                            continue
                        emit_eob(u, t)
                        while r > 15:
                            u.append(("sym", t, 0xF0))
                            r -= 16
                        s = _cat(v)
                        u.append(("sym", t, (r << 4) | s))
                        u.append(("bits", _bits_of(v, s), s))
                        r = 0
                    if r:
                        state["eobrun"] += 1
                        if state["eobrun"] == 0x7FFF:
                            emit_eob(u, t)
                else:
                    absv = [abs(int(v)) >> al for v in zz[ss:se + 1]]
                    eob = max([i for i, a in enumerate(absv) if a == 1], default=-1)
                    r, br = 0, []
                    for i, a in enumerate(absv):
                        if a == 0:
                            r += 1
                            continue
                        while r > 15 and i <= eob:
                            emit_eob(u, t)
                            u.append(("sym", t, 0xF0))
                            u.extend(("bits", bit, 1) for bit in br)
                            br = []
                            r -= 16
                        if a > 1:
                            br.append(a & 1)
                            continue
                        emit_eob(u, t)
                        u.append(("sym", t, (r << 4) | 1))
                        u.append(("bits", 1 if zz[ss + i] > 0 else 0, 1))
                        u.extend(("bits", bit, 1) for bit in br)
                        br, r = [], 0
                    if r or br:
                        state["eobrun"] += 1
                        state["be"].extend(br)
                        if state["eobrun"] == 0x7FFF or len(state["be"]) > 900:
                            emit_eob(u, t)
            ev.append(u)
        if ss:
            emit_eob(ev[-1], table(sc[0]))
        # one Huffman table per table id used in the scan (DC tables for a
        # first DC scan, AC tables for AC scans; a DC refinement needs none)
        freq = {}
        for u in ev:
            for e in u:
                if e[0] == "sym":
                    freq.setdefault(e[1], {})
                    freq[e[1]][e[2]] = freq[e[1]].get(e[2], 0) + 1
        codes = {}
        cls = 0 if ss == 0 else 1
        for t, fq in sorted(freq.items()):
            counts, order, cd = _canonical(_huff_lengths(fq))
            codes[t] = cd
            body = bytes([(cls << 4) | t]) + bytes(counts) + bytes(order)
            out += b"\xff\xc4" + struct.pack(">H", 2 + len(body)) + body
        sos = bytes([len(sc)])
        for k in sc:
            sos += bytes([comps[k]["id"], (table(k) << 4) | table(k)])
        sos += bytes([ss, se, (ah << 4) | al])
        out += b"\xff\xda" + struct.pack(">H", 2 + len(sos)) + sos
        bw = _BitWriter()
        rst = 0
        for u in ev:
            for e in u:
                if e[0] == "sym":
                    code, ln = codes[e[1]][e[2]]
                    bw.put(code, ln)
                elif e[0] == "bits":
                    bw.put(e[1], e[2])
                else:
                    bw.flush()
                    bw.data += bytes([0xFF, 0xD0 + rst % 8])
                    rst += 1
        bw.flush()
        out += bw.data
    out += b"\xff\xd9"
    info = dict(width=cf["w"], height=cf["h"], comps=comps, qts=cf["qts"], hmax=cf["hmax"], vmax=cf["vmax"])
    return bytes(out), info
