"""CPU checks of the C ABI: the library loads, exports every entry point that
include/sgl.h declares, and the ctypes structures match the C layout."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from swegl_gb300 import abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sgl.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"SGL_API\s+[\w\s\*]+?\b(sgl_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return C.CDLL(build.LIB)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "sgl_render" in names and "sgl_scene_upload" in names and len(names) >= 10


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_no_device_is_reported_not_crashed(lib):
    """On a host without a GPU sgl_create returns SGL_ERR_NO_DEVICE."""
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    lib.sgl_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    assert lib.sgl_create(C.byref(h), 0) == -7
    lib.sgl_status_string.restype = C.c_char_p
    assert lib.sgl_status_string(-7) == b"no CUDA device"


def test_host_alloc_refuses_bad_arguments(lib):
    """sgl_host_alloc checks its arguments before any CUDA call: zero bytes or
    no output pointer is SGL_ERR_INVALID; freeing NULL is a no-op."""
    lib.sgl_host_alloc.argtypes = [C.c_size_t, C.c_int, C.POINTER(C.c_void_p)]
    lib.sgl_host_free.argtypes = [C.c_void_p]
    p = C.c_void_p(1)
    assert lib.sgl_host_alloc(0, 1, C.byref(p)) == -1
    assert p.value is None
    assert lib.sgl_host_alloc(64, 0, None) == -1
    assert lib.sgl_host_free(None) == 0


STRUCTS = {
    "sgl_node_desc": abi.NodeDesc, "sgl_primitive_desc": abi.PrimitiveDesc, "sgl_material_desc": abi.MaterialDesc,
    "sgl_texture_desc": abi.TextureDesc, "sgl_point_light": abi.PointLight, "sgl_scene_desc": abi.SceneDesc,
    "sgl_dof_desc": abi.DofDesc, "sgl_view": abi.ViewDesc, "sgl_target": abi.Target,
    "sgl_frame_stats": abi.FrameStats, "sgl_batch_opts": abi.BatchOpts, "sgl_batch_item": abi.BatchItem,
    "sgl_serve_opts": abi.ServeOpts, "sgl_request": abi.Request, "sgl_request_result": abi.RequestResult,
}


def test_ctypes_layout_matches_header():
    src = '#include <stdio.h>\n#include <stddef.h>\n#include "sgl.h"\nint main(void){\n'
    for name in STRUCTS:
        src += f'printf("{name} %zu\\n", sizeof({name}));\n'
    src += 'printf("view.dof %zu\\n", offsetof(sgl_view, dof));\n'
    src += 'printf("scene.default_material %zu\\n", offsetof(sgl_scene_desc, default_material));\n'
    src += 'printf("batch_item.nodes %zu\\n", offsetof(sgl_batch_item, nodes));\nreturn 0;}\n'
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    sizes = dict(line.split() for line in out.strip().splitlines())
    for name, cls in STRUCTS.items():
        assert int(sizes[name]) == C.sizeof(cls), name
    assert int(sizes["view.dof"]) == abi.ViewDesc.dof.offset
    assert int(sizes["scene.default_material"]) == abi.SceneDesc.default_material.offset
    assert int(sizes["batch_item.nodes"]) == abi.BatchItem.nodes.offset
