"""CPU restatement of swegl's glTF loader, scene_t::animate and BMP reader.

TEST INFRASTRUCTURE ONLY (the checker): used by tests/ to check the
library's host loaders (swegl_gb300/csrc/sgl_gltf.cpp, sgl_image.cpp).

Follows, in the reference (gbizzotto/swegl):
  load_scene / load_scene_glb / load_scene_gltf   src/data/gltf.cpp:388-464
  load_scene_json                                 src/data/gltf.cpp:55-386
  accessor_t                                      src/data/gltf.cpp:13-53
  matrix44_t::from_quaternion                     swegl/projection/matrix44.hpp:34-43
  scene_t::animate, animation_channel_t::get_steps swegl/data/model.hpp:109-177
  vec4f_t::normalize                              swegl/projection/vec2f.hpp:67-77
  read_bmp_file                                   src/misc/image.cpp:29-83
  read_png_file (libpng's transforms)             src/misc/image.cpp:92-172
  read_jpeg_file (libjpeg default decompression) src/misc/image.cpp:183-255
Arithmetic is numpy float32 in the reference's order of operations.  The
reference's own loader is compiled too (oracle/ref, with a stand-in for its
un-vendored nlohmann/json include, shim/json.hpp) and the library's loader is
checked against its output (tests/test_gltf_cpu.py,
test_loader_matches_the_reference_loader); its quaternion and animation
arithmetic against the compiled reference's from_quaternion and
scene_t::animate (oracle/ref/ref_harness.cpp).  PNG is
lossless (any correct decoder gives libpng's texels); the JPEG pixel path
restates libjpeg's published default decompression, and with libjpeg absent
here its parity with libjpeg is unpinned.
"""
from __future__ import annotations

import base64
import json
import os
import struct

import numpy as np

from swegl_gb300 import scenes as S

F = np.float32


def from_quaternion(q0, q1, q2, q3) -> np.ndarray:
    """matrix44_t::from_quaternion (matrix44.hpp:34-43), row-major 4x4."""
    q0, q1, q2, q3 = F(q0), F(q1), F(q2), F(q3)
    two, one = F(2), F(1)
    return np.array([
        [two * (q0 * q0 + q1 * q1) - one, two * (q1 * q2 - q0 * q3), two * (q1 * q3 + q0 * q2), F(0)],
        [two * (q1 * q2 + q0 * q3), two * (q0 * q0 + q2 * q2) - one, two * (q2 * q3 - q0 * q1), F(0)],
        [two * (q1 * q3 - q0 * q2), two * (q2 * q3 + q0 * q1), two * (q0 * q0 + q3 * q3) - one, F(0)],
        [F(0), F(0), F(0), F(1)]], np.float32)


def _len3(x, y, z):
    return F(np.sqrt(F(F(F(x * x) + F(y * y)) + F(z * z))))


def _colour_byte(f) -> int:
    """(unsigned char)(255 * f) (gltf.cpp:128-132): float product, then the
    conversion to int and the low byte."""
    v = F(255) * F(f)
    if not (-2147483648.0 < float(v) < 2147483648.0):
        return 0
    return int(np.trunc(float(v))) & 0xFF


def read_bmp(data: bytes) -> np.ndarray:
    """read_bmp_file (image.cpp:29-83): 24-bit BGR rows from byte 54,
    bottom-up, skipping (width*3)%4 bytes after each row."""
    w, h = struct.unpack_from("<ii", data, 18)
    pad = (w * 3) % 4
    out = np.zeros((h, w), np.uint32)
    p = 54
    for row in range(h - 1, -1, -1):
        px = np.frombuffer(data, np.uint8, 3 * w, p).reshape(w, 3).astype(np.uint32)
        out[row] = 0xFF000000 | (px[:, 2] << 16) | (px[:, 1] << 8) | px[:, 0]
        p += 3 * w + pad
    return out


def read_png(data: bytes) -> np.ndarray:
    """read_png_file (image.cpp:92-172) restated on the PNG specification:
    every colour type and depth to 8-bit RGBA (16-bit samples keep their
    high byte, low-depth grey scales up, tRNS becomes alpha, grey is
    replicated), Adam7 included; 0xAARRGGBB texels."""
    import zlib

    pos, idat, plte, trns = 8, b"", None, None
    while pos + 8 <= len(data):
        ln = struct.unpack_from(">I", data, pos)[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + ln]
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, inter = struct.unpack(">IIBBBBB", body[:13])
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3).astype(np.uint32)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
        pos += 12 + ln
    raw = zlib.decompress(idat)
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp = max(1, ch * depth // 8)
    samples = np.zeros((h, w, ch), np.uint32)
    passes = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)] \
        if inter else [(0, 0, 1, 1)]
    at = 0
    for (x0, y0, dx, dy) in passes:
        if x0 >= w or y0 >= h:
            continue
        pw, ph = (w - x0 + dx - 1) // dx, (h - y0 + dy - 1) // dy
        rb = (pw * ch * depth + 7) // 8
        prev = bytearray(rb)
        for py in range(ph):
            f, row = raw[at], bytearray(raw[at + 1:at + 1 + rb])
            at += 1 + rb
            for i in range(rb):
                a = row[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                if f == 1:
                    row[i] = (row[i] + a) & 0xFF
                elif f == 2:
                    row[i] = (row[i] + b) & 0xFF
                elif f == 3:
                    row[i] = (row[i] + ((a + b) >> 1)) & 0xFF
                elif f == 4:
                    p_ = a + b - c
                    pa, pb, pc = abs(p_ - a), abs(p_ - b), abs(p_ - c)
                    row[i] = (row[i] + (a if pa <= pb and pa <= pc else (b if pb <= pc else c))) & 0xFF
            prev = row
            if depth == 16:
                vals = np.frombuffer(bytes(row), ">u2").astype(np.uint32)
            elif depth == 8:
                vals = np.frombuffer(bytes(row), np.uint8).astype(np.uint32)
            else:
                bits = np.unpackbits(np.frombuffer(bytes(row), np.uint8))
                k = len(bits) // depth
                vals = bits[:k * depth].reshape(k, depth).dot(1 << np.arange(depth - 1, -1, -1)).astype(np.uint32)
            samples[y0 + py * dy, x0::dx][:pw] = vals[:pw * ch].reshape(pw, ch)
    to8 = {1: 255, 2: 85, 4: 17, 8: 1}
    s8 = (samples >> 8) if depth == 16 else samples * to8[depth]
    a = np.full((h, w), 255, np.uint32)
    if ctype == 3:
        rgb = plte[samples[..., 0]]
        r, g, b = rgb[..., 0], rgb[..., 1], rgb[..., 2]
        if trns is not None:
            ta = np.full(len(plte), 255, np.uint32)
            ta[:len(trns)] = list(trns)
            a = ta[samples[..., 0]]
    elif ctype in (0, 4):
        r = g = b = s8[..., 0]
        if ctype == 4:
            a = s8[..., 1]
        elif trns is not None:
            a = np.where(samples[..., 0] == ((trns[0] << 8) | trns[1]), 0, 255).astype(np.uint32)
    else:
        r, g, b = s8[..., 0], s8[..., 1], s8[..., 2]
        if ctype == 6:
            a = s8[..., 3]
        elif trns is not None:
            key = [(trns[2 * c] << 8) | trns[2 * c + 1] for c in range(3)]
            a = np.where((samples[..., 0] == key[0]) & (samples[..., 1] == key[1]) & (samples[..., 2] == key[2]),
                         0, 255).astype(np.uint32)
    return ((a << 24) | (r << 16) | (g << 8) | b).astype(np.uint32)


def decode_image(name: str, data: bytes) -> np.ndarray:
    """read_image_file (image.cpp:20-27) for PNG and BMP."""
    n = name.lower()
    if n.endswith("png"):
        return read_png(data)
    if n.endswith("bmp"):
        return read_bmp(data)
    raise ValueError(f"image {name}: only PNG and BMP are restated")


class _Accessor:
    """accessor_t (gltf.cpp:13-53): stride from the buffer view, else the
    tight size of the element; data from the accessor's byte offset."""

    def __init__(self, views, a):
        bv_data, bv_stride = views[a["bufferView"]]
        self.count = a["count"]
        stride = bv_stride
        if stride == 0:
            cs = {5120: 1, 5121: 1, 5122: 2, 5123: 2, 5125: 4, 5126: 4}[a["componentType"]]
            nc = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}[a["type"]]
            stride = cs * nc
        self.stride = stride
        self.data = bv_data[a.get("byteOffset", 0):]

    def f32(self, i, off):
        o = off + i * self.stride
        return F(np.frombuffer(self.data, np.float32, 1, o)[0])

    def u16(self, i):
        o = i * self.stride
        b = self.data[o:o + 2] + b"\0\0"
        return b[0] | (b[1] << 8)


class GltfResult:
    def __init__(self):
        self.scene = S.Scene()
        self.animations = []  # [(end_time, [(node, path, [(t, (4 floats))])])]


def _uri_bytes(root, uri):
    if uri.startswith("data:"):
        return base64.b64decode(uri.split(",", 1)[1])
    with open(os.path.join(root, uri), "rb") as fh:
        return fh.read()


def load_scene(path: str, decode_image) -> GltfResult:
    """load_scene (gltf.cpp:455-464).  `decode_image(name, bytes)` decodes
    one image (the reference's read_image_file / read_png_file)."""
    root = os.path.dirname(path)
    with open(path, "rb") as fh:
        raw = fh.read()
    if path.lower().endswith("glb"):
        total = struct.unpack_from("<I", raw, 8)[0]
        chunks, at = [], 12
        while at < total:
            ln = struct.unpack_from("<I", raw, at)[0]
            chunks.append(raw[at + 8:at + 8 + ln])
            at += 8 + ln
        j = json.loads(chunks[0].decode())
        bin_chunk = chunks[1] if len(chunks) > 1 else b""
    else:
        j = json.loads(raw.decode())
        bin_chunk = None
    buffers = []
    for b in j.get("buffers", []):
        data = _uri_bytes(root, b["uri"]) if "uri" in b else bin_chunk
        buffers.append(data[:b["byteLength"]])
    return _load_json(root, j, buffers, decode_image)


def _load_json(root, j, buffers, decode_image) -> GltfResult:
    """load_scene_json (gltf.cpp:55-386)."""
    r = GltfResult()
    s = r.scene
    views = []
    for bv in j.get("bufferViews", []):
        data = buffers[bv["buffer"]]
        off = bv.get("byteOffset", 0)
        views.append((data[off:off + bv["byteLength"]], bv.get("byteStride", 0)))
    acc = [_Accessor(views, a) for a in j.get("accessors", [])]
    for im in j.get("images", []):  # gltf.cpp:74-110
        if "uri" in im:
            name = im["uri"] if not im["uri"].startswith("data:") else (".png" if "image/png" in im["uri"] else ".jpg")
            s.textures.append(decode_image(name, _uri_bytes(root, im["uri"])))
        else:
            data, _ = views[im["bufferView"]]
            s.textures.append(decode_image(".png" if im["mimeType"] == "image/png" else ".jpg", data))
    for m in j.get("materials", []):  # gltf.cpp:112-154
        ds = 1 if m.get("doubleSided", False) else 0
        if "pbrMetallicRoughness" not in m:
            s.materials.append((0xFFFFFFFF, -1, 0, 32))
            continue
        pbr = m["pbrMetallicRoughness"]
        b = g = rr = a = 255
        if "baseColorFactor" in pbr:
            f = pbr["baseColorFactor"]
            b, g, rr, a = _colour_byte(f[2]), _colour_byte(f[1]), _colour_byte(f[0]), _colour_byte(f[3])
        img = -1
        if "baseColorTexture" in pbr:
            img = j["textures"][pbr["baseColorTexture"]["index"]]["source"]
        s.materials.append(((a << 24) | (rr << 16) | (g << 8) | b, img, ds, 32))
    temp = []  # gltf.cpp:156-203: meshes with primitives only
    for mesh in j.get("meshes", []):
        if "primitives" not in mesh:
            continue
        prims = []
        for p in mesh["primitives"]:
            ap = acc[p["attributes"]["POSITION"]]
            n = ap.count
            pos = np.array([[ap.f32(i, 4 * c) for c in range(3)] for i in range(n)], np.float32).reshape(n, 3)
            nrm = np.zeros((n, 3), np.float32)
            uv = np.zeros((n, 2), np.float32)
            if "NORMAL" in p["attributes"]:
                an = acc[p["attributes"]["NORMAL"]]
                for i in range(min(n, an.count)):
                    nrm[i] = [an.f32(i, 4 * c) for c in range(3)]
            if "TEXCOORD_0" in p["attributes"]:
                at = acc[p["attributes"]["TEXCOORD_0"]]
                for i in range(min(n, at.count)):
                    uv[i] = [at.f32(i, 4), at.f32(i, 0)]  # x from +4, y from +0 (gltf.cpp:184-185)
            idx = np.zeros((0,), np.uint32)
            if "indices" in p:
                ai = acc[p["indices"]]
                idx = np.array([ai.u16(i) for i in range(ai.count)], np.uint32)  # read as uint16 (gltf.cpp:196)
            prims.append((p.get("mode", 4), p.get("material", -1), pos, nrm, uv, idx))
        temp.append(prims)
    taken = set()
    nodes = j.get("nodes", [])
    children = []
    pos_all, nrm_all, uv_all, idx_all = [], [], [], []
    nv = ni = 0
    for k, jn in enumerate(nodes):  # gltf.cpp:205-313
        scale = np.ones(3, np.float32)
        rot = np.eye(4, dtype=np.float32)
        trans = np.zeros(3, np.float32)
        if "rotation" in jn:
            q = jn["rotation"]
            rot = from_quaternion(q[0], q[1], q[2], q[3])
        if "translation" in jn:
            trans = np.array(jn["translation"], np.float32)
        if "scale" in jn:
            scale = np.array(jn["scale"], np.float32)
        if "matrix" in jn:
            mm = np.array(jn["matrix"], np.float32).reshape(4, 4).T.copy()  # column-major to row-major
            trans = np.array([mm[0, 3], mm[1, 3], mm[2, 3]], np.float32)
            scale = np.array([_len3(*mm[0, :3]), _len3(*mm[1, :3]), _len3(*mm[2, :3])], np.float32)
            mm[0, 3] = mm[1, 3] = mm[2, 3] = F(0)
            for c in range(3):
                if scale[c] != 0:
                    for rr in range(3):
                        mm[rr, c] = F(mm[rr, c] / scale[c])
            rot = mm
        s.node_scale.append(scale)
        s.node_rotation.append(rot)
        s.node_translation.append(trans)
        s.node_parent.append(-1)
        if "mesh" in jn and jn["mesh"] not in taken:  # primitives are moved to the first user (gltf.cpp:296)
            taken.add(jn["mesh"])
            for (mode, mat, pos, nrm, uv, idx) in temp[jn["mesh"]]:
                if mode not in (4, 5, 6):
                    continue
                s.primitives.append((k, mode, mat, nv, len(pos), ni, len(idx)))
                pos_all.append(pos)
                nrm_all.append(nrm)
                uv_all.append(uv)
                idx_all.append(idx)
                nv += len(pos)
                ni += len(idx)
        children.append(jn.get("children", []))
    for k, ch in enumerate(children):
        for c in ch:
            s.node_parent[c] = k
    s.positions = np.concatenate(pos_all) if pos_all else np.zeros((0, 3), np.float32)
    s.normals = np.concatenate(nrm_all) if nrm_all else np.zeros((0, 3), np.float32)
    s.uvs = np.concatenate(uv_all) if uv_all else np.zeros((0, 2), np.float32)
    s.indices = np.concatenate(idx_all) if idx_all else np.zeros((0,), np.uint32)
    s.ambient, s.sun_intensity = 0.0, 0.0
    s.sun_direction = np.zeros(3, np.float32)
    for ja in j.get("animations", []):  # gltf.cpp:322-385
        end, chans = F(0), []
        for jc in ja["channels"]:
            smp = ja["samplers"][jc["sampler"]]
            path = {"scale": 0, "rotation": 1, "translation": 2}.get(jc["target"]["path"], 3)
            times, values = acc[smp["input"]], acc[smp["output"]]
            steps = []
            for i in range(times.count):
                v = [F(0), F(0), F(0), F(1)]
                ncomp = 4 if path == 1 else (0 if path == 3 else 3)
                for c in range(ncomp):
                    v[c] = values.f32(i, 4 * c)
                steps.append((times.f32(i, 0), tuple(v)))
            steps.sort(key=lambda st: st[0])
            end = max(end, steps[-1][0])
            chans.append((jc["target"]["node"], path, steps))
        r.animations.append((F(end), chans))
    return r


def animate(result: GltfResult, seconds: float) -> None:
    """scene_t::animate (model.hpp:146-177) on the result's nodes."""
    s = result.scene
    for end, chans in result.animations:
        rel = F(np.fmod(F(seconds), end))
        for node, path, steps in chans:
            times = [st[0] for st in steps]
            k = 0  # lower_bound: first step whose time is not below rel
            while k < len(times) and times[k] < rel:
                k += 1
            if k == len(times):
                before = after = steps[-1]
            elif k == 0:
                before = after = steps[0]
            else:
                before, after = steps[k - 1], steps[k]
            if after[0] == before[0]:
                f = [F(v) for v in before[1]]
            else:
                wa = F(F(after[0] - rel) / F(after[0] - before[0]))
                wb = F(F(rel - before[0]) / F(after[0] - before[0]))
                f = [F(F(before[1][c] * wa) + F(after[1][c] * wb)) for c in range(4)]
            if path == 1:
                ln = F(np.sqrt(F(F(F(F(f[0] * f[0]) + F(f[1] * f[1])) + F(f[2] * f[2])) + F(f[3] * f[3]))))
                if ln != 0:
                    f = [F(v / ln) for v in f]
                s.node_rotation[node] = from_quaternion(*f)
            elif path == 2:
                s.node_translation[node] = np.array(f[:3], np.float32)
            elif path == 0:
                s.node_scale[node] = np.array(f[:3], np.float32)


# ------------------------------------------------------------------ JPEG --
def _idct_islow(coef: np.ndarray, q: np.ndarray) -> np.ndarray:
    """libjpeg's accurate integer IDCT (jidctint.c, the LL&M flow graph in
    13-bit fixed point; columns with 2 extra bits, then rows) of blocks
    (..., 8, 8) of quantised coefficients; samples level-shifted and
    clamped (values wrapped mod 1024 first, as its masked table lookup)."""
    CB, P1 = 13, 2
    F = dict(a=2446, b=3196, c=4433, d=6270, e=7373, f=9633, g=12299, h=15137, i=16069, j=16819, k=20995, l=25172)
    x = coef.astype(np.int64) * q.astype(np.int64)

    def flow(v, scale_shift, out_shift):
        # v[..., n] for n = 0..7 along the transformed axis
        z2, z3 = v[..., 2], v[..., 6]
        z1 = (z2 + z3) * F["c"]
        t2 = z1 + z3 * (-F["h"])
        t3 = z1 + z2 * F["d"]
        t0 = (v[..., 0] + v[..., 4]) << CB
        t1 = (v[..., 0] - v[..., 4]) << CB
        t10, t13, t11, t12 = t0 + t3, t0 - t3, t1 + t2, t1 - t2
        t0, t1, t2, t3 = v[..., 7], v[..., 5], v[..., 3], v[..., 1]
        z1, z2, z3, z4 = t0 + t3, t1 + t2, t0 + t2, t1 + t3
        z5 = (z3 + z4) * F["f"]
        t0, t1, t2, t3 = t0 * F["a"], t1 * F["j"], t2 * F["l"], t3 * F["g"]
        z1, z2, z3, z4 = z1 * -F["e"], z2 * -F["k"], z3 * -F["i"] + z5, z4 * -F["b"] + z5
        t0, t1, t2, t3 = t0 + z1 + z3, t1 + z2 + z4, t2 + z2 + z3, t3 + z1 + z4
        ds = lambda a: (a + (1 << (out_shift - 1))) >> out_shift
        return np.stack([ds(t10 + t3), ds(t11 + t2), ds(t12 + t1), ds(t13 + t0),
                         ds(t13 - t0), ds(t12 - t1), ds(t11 - t2), ds(t10 - t3)], -1)

    cols = np.swapaxes(x, -1, -2)  # [..., col, row]: transform along rows index
    ws = flow(cols, 0, CB - P1)    # [..., col, row-out]
    dc_only = np.all(cols[..., 1:] == 0, axis=-1)
    ws = np.where(dc_only[..., None], (cols[..., :1] << P1), ws)
    ws = np.swapaxes(ws, -1, -2)   # [..., row, col]
    out = flow(ws, 0, CB + P1 + 3)
    dc_only = np.all(ws[..., 1:] == 0, axis=-1)
    out = np.where(dc_only[..., None], (ws[..., :1] + (1 << (P1 + 2))) >> (P1 + 3), out)
    v = out & 1023
    v = np.where(v >= 512, v - 1024, v) + 128
    return np.clip(v, 0, 255)


def _upsample(plane: np.ndarray, dw: int, dh: int, hx: int, vx: int) -> np.ndarray:
    """libjpeg's fancy (triangle) upsampling for 2x1, 2x2 (and libjpeg-turbo's
    1x2), edge samples repeated; replication otherwise or when the
    component is 2 samples wide or less."""
    p = plane[:dh, :dw].astype(np.int64)
    if hx == 1 and vx == 1:
        return p
    up = np.vstack([p[:1], p[:-1]])
    dn = np.vstack([p[1:], p[-1:]])
    if hx == 2 and vx == 1 and dw > 2:
        o = np.zeros((dh, 2 * dw), np.int64)
        left = np.hstack([p[:, :1], p[:, :-1]])
        right = np.hstack([p[:, 1:], p[:, -1:]])
        o[:, 0::2] = (3 * p + left + 1) >> 2
        o[:, 1::2] = (3 * p + right + 2) >> 2
        o[:, 0], o[:, -1] = p[:, 0], p[:, -1]
        return o
    if hx == 2 and vx == 2 and dw > 2:
        o = np.zeros((2 * dh, 2 * dw), np.int64)
        for half, nb in ((0, up), (1, dn)):
            cs = 3 * p + nb
            last = np.hstack([cs[:, :1], cs[:, :-1]])
            nxt = np.hstack([cs[:, 1:], cs[:, -1:]])
            ev = (3 * cs + last + 8) >> 4
            od = (3 * cs + nxt + 7) >> 4
            ev[:, 0] = (4 * cs[:, 0] + 8) >> 4
            od[:, -1] = (4 * cs[:, -1] + 7) >> 4
            o[half::2, 0::2] = ev
            o[half::2, 1::2] = od
        return o
    if hx == 1 and vx == 2:
        o = np.zeros((2 * dh, dw), np.int64)
        o[0::2] = (3 * p + up + 1) >> 2
        o[1::2] = (3 * p + dn + 2) >> 2
        return o
    return np.repeat(np.repeat(p, vx, 0), hx, 1)


def jpeg_pixels(info: dict) -> np.ndarray:
    """The texels libjpeg's default decompression gives for the quantised
    coefficients of a JPEG (read_jpeg_file, image.cpp:183-255): IDCT,
    upsampling, then YCbCr -> RGB with 16 fraction bits (grey replicated)."""
    w, h, hmax, vmax = info["width"], info["height"], info["hmax"], info["vmax"]
    full = []
    for c in info["comps"]:
        s = _idct_islow(c["coef"], info["qts"][c["tq"]])  # (bh, bw, 8, 8)
        plane = s.transpose(0, 2, 1, 3).reshape(c["bh"] * 8, c["bw"] * 8)
        full.append(_upsample(plane, c["dw"], c["dh"], hmax // c["h"], vmax // c["v"])[:h, :w])
    if len(full) == 1:
        g = full[0].astype(np.uint32)
        return (0xFF000000 | (g << 16) | (g << 8) | g).astype(np.uint32)
    fix = lambda x: int(x * 65536.0 + 0.5)
    xs = np.arange(256, dtype=np.int64) - 128
    cr_r = (fix(1.40200) * xs + (1 << 15)) >> 16
    cb_b = (fix(1.77200) * xs + (1 << 15)) >> 16
    cr_g = -fix(0.71414) * xs
    cb_g = -fix(0.34414) * xs + (1 << 15)
    y, cb, cr = full
    r = np.clip(y + cr_r[cr], 0, 255).astype(np.uint32)
    g = np.clip(y + ((cb_g[cb] + cr_g[cr]) >> 16), 0, 255).astype(np.uint32)
    b = np.clip(y + cb_b[cb], 0, 255).astype(np.uint32)
    return (0xFF000000 | (r << 16) | (g << 8) | b).astype(np.uint32)
