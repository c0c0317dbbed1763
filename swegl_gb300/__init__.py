"""GB300-native renderer for swegl scenes.

Layout:
  csrc/      sm_103a kernels (raster.cu) and the C-ABI runtime (sgl_api.cpp)
  build.py   in-tree compile of csrc into _build/libsgl.so
  abi.py     ctypes mirror of include/sgl.h
  runtime.py Python binding of the C ABI (no CPU fallback)
  scenes.py  seeded synthetic scenes, bit-reproducible across hosts
"""
__all__ = ["abi", "scenes", "runtime", "build"]
