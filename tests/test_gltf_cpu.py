"""glTF ingestion and image decoding (host side, no GPU): the library's
loaders (sgl_gltf_load, sgl_gltf_animate, sgl_image_load) against the
oracle restatement of the reference's loader, animation and image readers
(oracle/gltf_oracle.py), whose quaternion and animation arithmetic is in turn
checked against the compiled reference when it is available here.

Bar: bit-exact (every float compared by its bits, every texel exactly)."""
import ctypes as C
import os
import zlib

import numpy as np
import pytest

import gltf_files as GF
import oracle
from oracle import gltf_oracle as GO


@pytest.fixture(scope="module")
def lib():
    from swegl_gb300.runtime import library

    return library()


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


# ----------------------------------------------------------------- images --
PNG_CASES = [
    # (ctype, depth, interlace, with tRNS)
    (0, 1, False, False), (0, 2, True, False), (0, 4, False, True), (0, 8, False, True), (0, 16, True, True),
    (2, 8, False, False), (2, 8, True, True), (2, 16, False, True),
    (3, 1, False, False), (3, 2, True, True), (3, 4, False, True), (3, 8, True, True),
    (4, 8, False, False), (4, 16, True, False),
    (6, 8, False, False), (6, 8, True, False), (6, 16, False, False),
]


@pytest.mark.parametrize("ctype,depth,interlace,trns", PNG_CASES)
def test_png_every_colour_type_and_depth(lib, tmp_path, ctype, depth, interlace, trns):
    from swegl_gb300.gltf import load_image

    rng = np.random.default_rng(ctype * 100 + depth + (7 if interlace else 0))
    h, w = 13, 11  # odd sizes: partial bytes and every Adam7 pass
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    top = (1 << depth) - 1
    palette = None
    if ctype == 3:
        n_pal = min(top + 1, 37)
        palette = rng.integers(0, 256, size=(n_pal, 3))
        samples = rng.integers(0, n_pal, size=(h, w, 1))
    else:
        samples = rng.integers(0, top + 1, size=(h, w, ch))
    t = None
    if trns:
        if ctype == 3:
            t = bytes(rng.integers(0, 256, size=min(len(palette), 5)).astype(np.uint8))
        elif ctype == 0:
            v = int(samples[2, 3, 0])
            t = bytes([v >> 8, v & 0xFF])
        else:
            v = samples[4, 5]
            t = b"".join(bytes([int(c) >> 8, int(c) & 0xFF]) for c in v)
    data = GF.encode_png(samples, ctype, depth, interlace, palette, t, seed=ctype + depth)
    path = str(tmp_path / "t.png")
    with open(path, "wb") as fh:
        fh.write(data)
    exp = GF.png_expected(samples, ctype, depth, palette, t)
    got = load_image(path)
    assert np.array_equal(got, exp)
    assert np.array_equal(GO.read_png(data), exp)  # the restatement agrees


@pytest.mark.parametrize("level,strategy", [(0, zlib.Z_DEFAULT_STRATEGY), (1, zlib.Z_FIXED), (9, zlib.Z_DEFAULT_STRATEGY),
                                            (6, zlib.Z_HUFFMAN_ONLY), (6, zlib.Z_RLE)])
def test_inflate_stored_fixed_and_dynamic_blocks(lib, tmp_path, level, strategy):
    """The PNG decoder's own inflater on streams of every deflate block type."""
    from swegl_gb300.gltf import load_image

    rng = np.random.default_rng(level)
    img = np.zeros((40, 300, 4), np.uint8)
    img[..., :3] = rng.integers(0, 4, size=(40, 300, 3)) * 60  # repetitive: long matches
    img[..., 3] = 255
    raw = b"".join(b"\0" + img[y].tobytes() for y in range(40))
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    comp = co.compress(raw) + co.flush()
    import struct

    def chunk(k, b):
        return struct.pack(">I", len(b)) + k + b + struct.pack(">I", zlib.crc32(k + b) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 300, 40, 8, 6, 0, 0, 0)) + \
        chunk(b"IDAT", comp) + chunk(b"IEND", b"")
    path = str(tmp_path / "z.png")
    with open(path, "wb") as fh:
        fh.write(png)
    exp = GF.png_expected(img.astype(np.uint32), 6, 8)
    assert np.array_equal(load_image(path), exp)


@pytest.mark.parametrize("w", [1, 2, 3, 4, 5, 7, 8])
def test_bmp_follows_the_reference_reader(lib, tmp_path, w):
    """read_bmp_file skips (width*3)%4 bytes per row: standard files of
    widths with other padding read as the reference reads them."""
    from swegl_gb300.gltf import load_image

    rng = np.random.default_rng(w)
    rgb = rng.integers(0, 256, size=(6, w, 3))
    data = GF.encode_bmp(rgb)
    data += b"\0" * 64  # the reference's reads may run past a standard file's last row
    path = str(tmp_path / "t.bmp")
    with open(path, "wb") as fh:
        fh.write(data)
    exp = GO.read_bmp(data)
    assert np.array_equal(load_image(path), exp)
    if (w * 3) % 4 in (0, 2):
        # padding agrees with the standard one: the image itself
        std = (0xFF000000 | (rgb[..., 0] << 16) | (rgb[..., 1] << 8) | rgb[..., 2]).astype(np.uint32)
        assert np.array_equal(exp, std)


JPEG_CASES = [(s, r, i, g) for s in [(1, 1), (2, 1), (2, 2), (1, 2)]
              for (r, i, g) in [(0, True, False), (3, True, False), (0, False, False), (2, True, True)]]


@pytest.mark.parametrize("sampling,restart,interleaved,grey", JPEG_CASES)
def test_jpeg_matches_the_libjpeg_restatement(lib, tmp_path, sampling, restart, interleaved, grey):
    """Baseline JPEGs (per-file Huffman tables, every luma sampling of 2x1,
    2x2, 1x2, restart intervals, one scan per component, grey) decoded by
    the library equal the restated libjpeg pixel path applied to the
    encoder's own quantised coefficients; the image is close to its source."""
    from swegl_gb300.gltf import load_image

    yy, xx = np.mgrid[0:29, 0:37]
    smooth = np.stack([(xx * 7) % 256, (yy * 9) % 256, ((xx + yy) * 5) % 256], -1).astype(np.uint8)
    narrow = np.random.default_rng(2).integers(0, 256, size=(21, 5, 3)).astype(np.uint8)  # chroma <= 2 wide
    for img in (smooth, narrow):
        for q in (30, 95):
            data, info = GF.encode_jpeg(img, sampling, q, restart, grey=grey, interleaved=interleaved)
            path = str(tmp_path / "t.jpg")
            with open(path, "wb") as fh:
                fh.write(data)
            got = load_image(path)
            assert np.array_equal(got, GO.jpeg_pixels(info)), (img.shape, q)
    data, info = GF.encode_jpeg(smooth, (1, 1), 95, 0)
    with open(str(tmp_path / "s.jpeg"), "wb") as fh:
        fh.write(data)
    got = load_image(str(tmp_path / "s.jpeg"))
    rgb = np.stack([(got >> 16) & 255, (got >> 8) & 255, got & 255], -1).astype(int)
    assert np.abs(rgb - smooth.astype(int)).mean() < 3.0


PROGRESSIVE_CASES = [(s, r, g) for s in [(1, 1), (2, 1), (2, 2), (1, 2)] for (r, g) in [(0, False), (3, False), (0, True)]]


@pytest.mark.parametrize("sampling,restart,grey", PROGRESSIVE_CASES)
def test_progressive_jpeg_matches_the_libjpeg_restatement(lib, tmp_path, sampling, restart, grey):
    """Progressive JPEGs (SOF2: a DC scan with a point transform and its
    refinement, AC bands with point transforms, end-of-band runs across
    blocks and AC refinement scans with correction bits; restart intervals;
    grey) decode to exactly the pixels of the baseline file that holds the
    same coefficients: the restated libjpeg pixel path on the encoder's
    quantised coefficients."""
    from swegl_gb300.gltf import load_image

    yy, xx = np.mgrid[0:29, 0:37]
    smooth = np.stack([(xx * 7) % 256, (yy * 9) % 256, ((xx + yy) * 5) % 256], -1).astype(np.uint8)
    noisy = np.random.default_rng(5).integers(0, 256, size=(40, 56, 3)).astype(np.uint8)
    for img in (smooth, noisy):
        for q in (30, 95):
            data, info = GF.encode_jpeg_progressive(img, sampling, q, restart, grey=grey)
            assert data[2:].find(b"\xff\xc2") >= 0
            path = str(tmp_path / "p.jpg")
            with open(path, "wb") as fh:
                fh.write(data)
            got = load_image(path)
            exp = GO.jpeg_pixels(info)
            assert np.array_equal(got, exp), (img.shape, q)
            base, _ = GF.encode_jpeg(img, sampling, q, restart, grey=grey)
            with open(str(tmp_path / "b.jpg"), "wb") as fh:
                fh.write(base)
            assert np.array_equal(load_image(str(tmp_path / "b.jpg")), got)


def test_bad_images_are_errors_not_crashes(lib, tmp_path):
    from swegl_gb300.gltf import load_image
    from swegl_gb300.runtime import SglError

    for name, data in [("a.png", b"\x89PNG\r\n\x1a\n" + b"\0" * 30), ("b.png", b"not a png"), ("c.bmp", b"BM" + b"\0" * 10),
                       ("d.jpg", b"\xff\xd8\xff"), ("e.tga", b"\0" * 100)]:
        p = str(tmp_path / name)
        with open(p, "wb") as fh:
            fh.write(data)
        with pytest.raises(SglError):
            load_image(p)


# ------------------------------------------------------------------- glTF --
def scene_arrays(s):
    s.finalize()
    return {
        "node_scale": bits(np.array(s.node_scale)), "node_rotation": bits(np.array(s.node_rotation)),
        "node_translation": bits(np.array(s.node_translation)), "node_parent": np.array(s.node_parent),
        "primitives": np.array(s.primitives, np.int64), "positions": bits(s.positions), "normals": bits(s.normals),
        "uvs": bits(s.uvs), "indices": np.asarray(s.indices, np.uint32),
        "materials": np.array(s.materials, np.int64) & 0xFFFFFFFF,
        "textures": [np.asarray(t, np.uint32) for t in s.textures],
    }


def assert_same_scene(a, b):
    A, B = scene_arrays(a), scene_arrays(b)
    for k in A:
        if k == "textures":
            assert len(A[k]) == len(B[k])
            for x, y in zip(A[k], B[k]):
                assert np.array_equal(x, y), "texture differs"
        else:
            assert A[k].shape == B[k].shape and np.array_equal(A[k], B[k]), f"{k} differs"


@pytest.mark.parametrize("glb,seed", [(True, 3), (False, 4), (False, 5)])
def test_loader_matches_the_restatement(lib, tmp_path, glb, seed):
    """GLB with images in buffer views; .gltf with a base64 buffer (seed 4) or
    an external .bin (seed 5), images as data URIs and files."""
    from swegl_gb300.gltf import GltfScene

    path = GF.build_test_scene(str(tmp_path), glb, seed=seed)
    g = GltfScene(path)
    ours = g.scene()
    ref = GO.load_scene(path, GO.decode_image)
    assert_same_scene(ours, ref.scene)
    # the quirks are really exercised
    assert len(ours.primitives) == 6 + 12 + 3  # cube fans, sphere strips, two lists and the quad (lines dropped)
    assert sum(1 for p in ours.primitives if p[0] == 4) == 0  # the second user of mesh 0 has no primitives
    assert g.animation_count == 2
    g.close()


def test_animation_matches_the_restatement(lib, tmp_path):
    from swegl_gb300.gltf import GltfScene

    path = GF.build_test_scene(str(tmp_path), True)
    g = GltfScene(path)
    ref = GO.load_scene(path, GO.decode_image)
    for t in [0.0, 0.3, 0.5, 0.99, 1.25, 1.7, 2.0, 2.6, 7.31, 1e-7]:
        nodes = g.animate(t)
        GO.animate(ref, t)
        s = ref.scene
        for i in range(len(s.node_parent)):
            assert np.array_equal(bits(nodes[i].scale[:]), bits(s.node_scale[i])), (t, i)
            assert np.array_equal(bits(nodes[i].rotation[:]), bits(np.asarray(s.node_rotation[i]).reshape(-1))), (t, i)
            assert np.array_equal(bits(nodes[i].translation[:]), bits(s.node_translation[i])), (t, i)
    g.close()


def test_bad_gltf_files_are_errors(lib, tmp_path):
    from swegl_gb300.gltf import GltfScene
    from swegl_gb300.runtime import SglError

    cases = {"a.gltf": b"{", "b.gltf": b'{"buffers":[{"byteLength":10}]}', "c.glb": b"glTF\x02\0\0\0",
             "d.txt": b"{}", "e.gltf": b'{"meshes":[{"primitives":[{"attributes":{"POSITION":3}}]}]}'}
    for name, data in cases.items():
        p = str(tmp_path / name)
        with open(p, "wb") as fh:
            fh.write(data)
        with pytest.raises(SglError):
            GltfScene(p)
    with pytest.raises(SglError):
        GltfScene(str(tmp_path / "missing.glb"))


# ---------------------------------------- pins against the compiled reference --
needs_ref = pytest.mark.skipif(not oracle.reference_available(), reason="reference sources not present")


@needs_ref
def test_from_quaternion_matches_the_reference():
    ref = oracle.reference()
    rng = np.random.default_rng(9)
    out = (C.c_float * 16)()
    for _ in range(500):
        q = rng.normal(size=4).astype(np.float32) * np.float32(rng.choice([0.1, 1.0, 3.0]))
        qa = (C.c_float * 4)(*[float(v) for v in q])
        ref.ref_from_quaternion(qa, out)
        assert np.array_equal(bits(np.array(out[:])), bits(GO.from_quaternion(*q).reshape(-1)))


@needs_ref
def test_animate_matches_the_reference(tmp_path):
    """The restated scene_t::animate against the reference's own on the test
    scene's animations (and so, through the test above, the library's)."""
    from swegl_gb300 import abi

    ref_lib = oracle.reference()
    path = GF.build_test_scene(str(tmp_path), True)
    res = GO.load_scene(path, GO.decode_image)
    chans = [c for _, cs in res.animations for c in cs]
    ch_first, ch_node, ch_path, st_first, times, values = [0], [], [], [0], [], []
    for _, cs in res.animations:
        for node, pth, steps in cs:
            ch_node.append(node)
            ch_path.append(pth)
            for t, v in steps:
                times.append(float(t))
                values.extend(float(x) for x in v)
            st_first.append(len(times))
        ch_first.append(ch_first[-1] + len(cs))
    assert len(chans) == 3
    I = lambda a: (C.c_int * len(a))(*a)
    Fa = lambda a: (C.c_float * len(a))(*a)
    for t in [0.0, 0.3, 0.5, 1.25, 1.7, 2.0, 2.6, 7.31]:
        holder = abi.SceneDescHolder(res.scene)
        n = len(res.scene.node_parent)
        rc = ref_lib.ref_animate(holder.nodes, n, len(res.animations), I(ch_first), I(ch_node), I(ch_path),
                                 I(st_first), Fa(times), Fa(values), C.c_float(t))
        assert rc == 0
        GO.animate(res, t)
        s = res.scene
        for i in range(n):
            nd = holder.nodes[i]
            assert np.array_equal(bits(nd.scale[:]), bits(s.node_scale[i])), (t, i)
            assert np.array_equal(bits(nd.rotation[:]), bits(np.asarray(s.node_rotation[i]).reshape(-1))), (t, i)
            assert np.array_equal(bits(nd.translation[:]), bits(s.node_translation[i])), (t, i)


def _flatten_reference(r):
    """The reference loader's scene_t in the library's flat scene layout: nodes
    in order (parents from their children lists); each node's primitives as
    the renderer draws them (triangle lists, strips and fans; the other modes
    draw nothing, renderer.cpp:195-230), without the two spare vertices the
    loader appends to each primitive (gltf.cpp:174-175)."""
    from swegl_gb300 import scenes as S

    s = S.Scene()
    parent = [-1] * len(r.nodes)
    for k, n in enumerate(r.nodes):
        for c in n["children"]:
            parent[c] = k
    nv = ni = 0
    pos, nrm, uv, idx = [], [], [], []
    for k, n in enumerate(r.nodes):
        s.node_scale.append(n["scale"])
        s.node_rotation.append(n["rotation"])
        s.node_translation.append(n["translation"])
        s.node_parent.append(parent[k])
        for p in n["primitives"]:
            if p["mode"] not in (4, 5, 6):
                continue
            v = p["vertices"][:-2]
            s.primitives.append((k, p["mode"], p["material"], nv, len(v), ni, len(p["indices"])))
            pos.append(v[:, 0:3])
            nrm.append(v[:, 3:6])
            uv.append(v[:, 6:8])
            idx.append(p["indices"])
            nv += len(v)
            ni += len(p["indices"])
    s.positions, s.normals, s.uvs = np.concatenate(pos), np.concatenate(nrm), np.concatenate(uv)
    s.indices = np.concatenate(idx).astype(np.uint32)
    # materials as the library keeps them: colour, texture, double sided, shininess
    s.materials = [(c, t, ds, 32) for (c, _m, _r, t, ds) in r.materials]
    return s


@needs_ref
@pytest.mark.parametrize("glb,seed", [(True, 3), (False, 5)])
def test_loader_matches_the_reference_loader(lib, tmp_path, glb, seed):
    """The library's loader against the reference's own (src/data/gltf.cpp,
    compiled by oracle/ref with a stand-in for its un-vendored nlohmann/json
    include): node transforms and hierarchy, every primitive's vertices,
    texture coordinates, normals and indices (bit-exact), materials, image
    count, root nodes and animation channels.  A GLB with a PNG in a buffer
    view, and a .gltf with an external buffer (the reference reads buffers
    only from files)."""
    from swegl_gb300.gltf import GltfScene

    path = GF.build_test_scene(str(tmp_path), glb, seed=seed)
    ref = oracle.reference_gltf(path)
    g = GltfScene(path)
    ours = g.scene()
    A, B = scene_arrays(ours), scene_arrays(_flatten_reference(ref))
    for k in A:
        if k == "textures":
            assert len(A[k]) == ref.images
        else:
            assert A[k].shape == B[k].shape and np.array_equal(A[k], B[k]), f"{k} differs from the reference loader"
    assert ref.roots == [k for k, p in enumerate(ours.node_parent) if p < 0]
    # animation channels: the restatement's, which the library's animate()
    # follows (test_animation_matches_the_restatement), against the reference's
    res = GO.load_scene(path, GO.decode_image)
    assert g.animation_count == len(ref.animations) == len(res.animations)
    for (e0, c0), (e1, c1) in zip(ref.animations, res.animations):
        assert bits(e0) == bits(e1)
        assert [(n, p) for n, p, _ in c0] == [(n, p) for n, p, _ in c1]
        for (_, _, s0), (_, _, s1) in zip(c0, c1):
            assert np.array_equal(bits(np.array([[t, *v] for t, v in s0])), bits(np.array([[t, *v] for t, v in s1])))
    g.close()


@needs_ref
def test_loaded_scene_renders_as_the_reference_renders_it(tmp_path):
    """The restated loader's scene, lit and animated, rendered by the oracle
    restatement and by the compiled reference renderer: identical."""
    from swegl_gb300 import scenes as S

    path = GF.build_test_scene(str(tmp_path), True)
    res = GO.load_scene(path, GO.decode_image)
    s = res.scene
    s.ambient, s.sun_intensity = 0.15, 0.6
    s.sun_direction = S.normalize_f32(np.array([-0.5, -1.0, -0.7]))
    s.point_lights = [(0.5, 1.5, 2.5, 2.0)]
    GO.animate(res, 0.8)
    m, c = S.look_at((0.4, 0.6, 3.8), (0.0, 0.0, -0.3))
    v = S.view_for(240, 180, m, c)
    for layers in (0, 3):
        v.layers = layers
        a = oracle.render(s, [v], 0, "reference")
        b = oracle.render(s, [v], 0, "restatement")
        assert np.array_equal(a.pixels, b.pixels)
        assert np.array_equal(a.zbuffer.view(np.uint32), b.zbuffer.view(np.uint32))
        assert int((a.pixels != 0).sum()) > 3000
