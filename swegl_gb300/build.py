"""Compile the CUDA library in-tree: swegl_gb300/_build/libsgl.so, and the
same library with device-side bounds checks, libsgl_check.so (the kernels of
raster.cu compiled with -DSGL_BOUNDS_CHECK; see sgl_check_status in
include/sgl.h).

One -gencode (sm_103a), translation units compiled in parallel, no cmake.
Flags that matter for parity: -fmad=false (no fused multiply-add), IEEE
division / square root (no fast-math) on the device, -ffp-contract=off on the
host.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsgl.so")
LIB_CHECK = os.path.join(BUILD, "libsgl_check.so")

SOURCES = ["raster.cu", "sgl_api.cpp", "sgl_scene.cpp", "sgl_lane.cpp", "sgl_serve.cpp", "noalloc.cu", "sgl_gltf.cpp",
           "sgl_image.cpp"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags() -> list[str]:
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
            "-ftz=false", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off,-fvisibility=hidden",
            "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


CHECKED = "raster.cu"  # the translation unit with the kernels; compiled again with the checks


def _compile(job) -> str:
    src, checked = job
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ("_check.o" if checked else ".o"))
    path = os.path.join(CSRC, src)
    lang = [] if src.endswith(".cu") else ["-x", "cu"]
    cmd = [nvcc(), *_flags(), *(["-DSGL_BOUNDS_CHECK=1"] if checked else []), *lang, "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(LIB_CHECK):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(LIB_CHECK))
    inc = os.path.join(ROOT, "include")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(inc, f) for f in os.listdir(inc)] + [__file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _link(objs, lib):
    tmp = lib + ".tmp"
    cmd = [nvcc(), ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    jobs = [(CHECKED, True)] + [(src, False) for src in SOURCES]  # the longest first
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(_compile, jobs))
    checked_obj, plain = objs[0], objs[1:]
    _link(plain, LIB)
    _link([checked_obj if o.endswith(os.sep + "raster.o") else o for o in plain], LIB_CHECK)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
