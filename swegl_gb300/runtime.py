"""Python binding of the C ABI (include/sgl.h) over ctypes.

This mirrors the reference's render interface for tests and benchmarks:
`Renderer.render(scene_id, views)` is swegl::render(scene, vp0, vp1, ...)
(swegl/render/renderer.hpp:27-34) for the Phong + bilinear pixel shader, with
each view written to its own surface (or a shared one) and z-buffer.

The GPU library is required: there is no CPU fallback.  Loading fails loudly
when swegl_gb300/_build/libsgl.so has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsgl.so")
# the same library with device-side bounds checks (sgl_check_status)
LIB_CHECK_PATH = os.path.join(HERE, "_build", "libsgl_check.so")

_libs = {}


class SglError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def library(checked: bool = False) -> C.CDLL:
    """The in-tree CUDA library (raises if it was not built); `checked`: the
    build with device-side bounds checks."""
    path = LIB_CHECK_PATH if checked else LIB_PATH
    if path not in _libs:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(path)
        P = C.POINTER
        sigs = {
            "sgl_version": ([], C.c_int),
            "sgl_status_string": ([C.c_int], C.c_char_p),
            "sgl_create": ([P(C.c_void_p), C.c_int], C.c_int),
            "sgl_destroy": ([C.c_void_p], None),
            "sgl_last_error": ([C.c_void_p], C.c_char_p),
            "sgl_scene_upload": ([C.c_void_p, P(abi.SceneDesc), P(C.c_int)], C.c_int),
            "sgl_scene_release": ([C.c_void_p, C.c_int], C.c_int),
            "sgl_scene_set_nodes": ([C.c_void_p, C.c_int, P(abi.NodeDesc), C.c_int], C.c_int),
            "sgl_scene_set_lights": ([C.c_void_p, C.c_int, C.c_float, P(C.c_float), C.c_float, P(abi.PointLight),
                                      C.c_int], C.c_int),
            "sgl_scene_info": ([C.c_void_p, C.c_int, P(C.c_uint64), P(C.c_uint64), P(C.c_uint64)], C.c_int),
            "sgl_render": ([C.c_void_p, C.c_int, P(abi.ViewDesc), P(abi.Target), C.c_int, C.c_int, C.c_void_p,
                            P(abi.FrameStats)], C.c_int),
            "sgl_render_debug": ([C.c_void_p, C.c_int, P(abi.ViewDesc), P(abi.Target), P(C.c_uint32), P(C.c_uint8),
                                  P(abi.FrameStats)], C.c_int),
            "sgl_profile": ([C.c_void_p, C.c_int], C.c_int),
            "sgl_check_status": ([C.c_void_p, P(C.c_uint32), P(C.c_uint64), P(C.c_uint32), C.c_int], C.c_int),
            "sgl_render_batch": ([C.c_void_p, P(abi.BatchItem), C.c_int, P(abi.BatchOpts), C.c_void_p,
                                  P(abi.FrameStats)], C.c_int),
            "sgl_autotune": ([C.c_void_p, P(abi.BatchItem), C.c_int, P(abi.BatchOpts)], C.c_int),
            "sgl_dof": ([C.c_void_p, P(abi.ViewDesc), P(abi.Target), P(abi.Target), C.c_int, C.c_void_p], C.c_int),
            "sgl_render_noalloc": ([C.c_void_p, C.c_int, P(abi.ViewDesc), P(abi.Target), C.c_void_p], C.c_int),
            "sgl_server_create": ([C.c_void_p, P(abi.ServeOpts), P(C.c_void_p)], C.c_int),
            "sgl_server_submit": ([C.c_void_p, P(abi.Request), P(C.c_uint64)], C.c_int),
            "sgl_server_poll": ([C.c_void_p, C.c_uint64, P(abi.RequestResult)], C.c_int),
            "sgl_server_wait": ([C.c_void_p, C.c_uint64, C.c_double, P(abi.RequestResult)], C.c_int),
            "sgl_server_drain": ([C.c_void_p, C.c_double], C.c_int),
            "sgl_server_submit_batch": ([C.c_void_p, P(abi.Request), C.c_int, P(C.c_uint64), P(C.c_int)], C.c_int),
            "sgl_server_wait_batch": ([C.c_void_p, P(C.c_uint64), C.c_int, C.c_double, P(abi.RequestResult)],
                                      C.c_int),
            "sgl_server_destroy": ([C.c_void_p], None),
            "sgl_server_stats": ([C.c_void_p, P(C.c_uint64), P(C.c_uint64), P(C.c_uint64)], C.c_int),
            "sgl_profile_read": ([C.c_void_p, C.c_int, P(C.c_char_p), P(C.c_double), P(C.c_uint64)], C.c_int),
            "sgl_gltf_load": ([C.c_char_p, P(C.c_void_p), C.c_char_p, C.c_size_t], C.c_int),
            "sgl_gltf_scene": ([C.c_void_p], P(abi.SceneDesc)),
            "sgl_gltf_animation_count": ([C.c_void_p], C.c_int),
            "sgl_gltf_animate": ([C.c_void_p, C.c_float, P(abi.NodeDesc)], C.c_int),
            "sgl_gltf_free": ([C.c_void_p], None),
            "sgl_image_load": ([C.c_char_p, P(P(C.c_uint32)), P(C.c_int), P(C.c_int), C.c_char_p, C.c_size_t],
                               C.c_int),
            "sgl_image_free": ([P(C.c_uint32)], None),
            "sgl_host_alloc": ([C.c_size_t, C.c_int, P(C.c_void_p)], C.c_int),
            "sgl_host_free": ([C.c_void_p], C.c_int),
        }
        for name, (args, res) in sigs.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _libs[path] = lib
    return _libs[path]


def host_buffer(n_words: int, write_combined: bool = True, checked: bool = False) -> np.ndarray:
    """Page-locked host memory from sgl_host_alloc as a uint32 array (for
    request frames; write-combined by default), freed when the array and
    every view of it are gone."""
    import weakref

    lib = library(checked)
    p = C.c_void_p()
    st = lib.sgl_host_alloc(4 * int(n_words), 1 if write_combined else 0, C.byref(p))
    if st != 0:
        raise SglError(st, f"sgl_host_alloc of {4 * int(n_words)} bytes failed")
    buf = (C.c_uint32 * int(n_words)).from_address(p.value)
    weakref.finalize(buf, lib.sgl_host_free, p.value)
    return np.frombuffer(buf, dtype=np.uint32)


class Renderer:
    """One sgl context on one CUDA device."""

    def __init__(self, device: int = 0, checked: bool = False):
        self.lib = library(checked)
        h = C.c_void_p()
        st = self.lib.sgl_create(C.byref(h), device)
        if st != 0:
            raise SglError(st, "sgl_create failed")
        self.ctx = h
        self._holders = {}

    def close(self):
        if self.ctx:
            self.lib.sgl_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check_status(self, reset: bool = False) -> dict:
        """The device-side bounds checks' record (a Renderer on the checked
        library): the first failure's check code and index, and the count."""
        code, index, count = C.c_uint32(), C.c_uint64(), C.c_uint32()
        self._check(self.lib.sgl_check_status(self.ctx, C.byref(code), C.byref(index), C.byref(count),
                                              1 if reset else 0))
        return {"code": code.value, "index": index.value, "count": count.value}

    def _check(self, st: int):
        if st != 0:
            raise SglError(st, self.lib.sgl_last_error(self.ctx).decode(errors="replace"))

    # scenes ---------------------------------------------------------------
    def upload(self, scene) -> int:
        holder = abi.SceneDescHolder(scene)
        sid = C.c_int()
        self._check(self.lib.sgl_scene_upload(self.ctx, C.byref(holder.desc), C.byref(sid)))
        return sid.value

    def release(self, scene_id: int):
        self._check(self.lib.sgl_scene_release(self.ctx, scene_id))

    def scene_info(self, scene_id: int) -> dict:
        t, v, b = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._check(self.lib.sgl_scene_info(self.ctx, scene_id, C.byref(t), C.byref(v), C.byref(b)))
        return {"triangles": t.value, "vertices": v.value, "device_bytes": b.value}

    # rendering ------------------------------------------------------------
    def render(self, scene_id: int, views, shared_surface=None, stats: bool = False, background=None):
        """Render `views` in order into host surfaces (one per view, or one
        shared surface of size `shared_surface`, holding `background` before
        the render).  Returns (frames, stats)."""
        if shared_surface:
            surf = abi.HostFrame(*shared_surface)
            if background is not None:
                surf.pixels[...] = background
            frames = []
            for v in views:
                f = abi.HostFrame(*shared_surface, zw=v.w, zh=v.h)
                f.pixels = surf.pixels
                frames.append(f)
        else:
            frames = [abi.HostFrame(v.w, v.h) for v in views]
        vd = (abi.ViewDesc * len(views))(*[abi.view_desc(v) for v in views])
        td = (abi.Target * len(views))(*[f.target() for f in frames])
        fs = abi.FrameStats()
        self._check(self.lib.sgl_render(self.ctx, scene_id, vd, td, len(views), 0, None,
                                        C.byref(fs) if stats else None))
        return frames, (_stats_dict(fs) if stats else None)

    def render_device(self, scene_id: int, views, targets, stream: int = 0, stats: bool = False):
        """Render into device buffers (targets: list of abi.Target with device pointers)."""
        vd = (abi.ViewDesc * len(views))(*[abi.view_desc(v) for v in views])
        td = (abi.Target * len(views))(*targets)
        fs = abi.FrameStats()
        self._check(self.lib.sgl_render(self.ctx, scene_id, vd, td, len(views), 1, C.c_void_p(stream),
                                        C.byref(fs) if stats else None))
        return _stats_dict(fs) if stats else None

    def render_debug(self, scene_id: int, view):
        """One view with the per-pixel winner slot and per-slot setup flags."""
        info = self.scene_info(scene_id)
        frame = abi.HostFrame(view.w, view.h)
        winner = np.empty((view.h, view.w), np.uint32)
        flags = np.zeros(2 * max(1, info["triangles"]), np.uint8)
        fs = abi.FrameStats()
        vd = abi.view_desc(view)
        td = frame.target()
        self._check(self.lib.sgl_render_debug(self.ctx, scene_id, C.byref(vd), C.byref(td),
                                              winner.ctypes.data_as(C.POINTER(C.c_uint32)),
                                              flags.ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(fs)))
        return frame, winner, flags, _stats_dict(fs)

    # batches --------------------------------------------------------------
    def render_batch(self, items, tile: int = 0, span_bin: int = 0, use_graph: bool = True, stream: int = 0,
                     stats: bool = False):
        """items: list of (scene_id, view, abi.Target with device pointers)
        or (scene_id, view, target, nodes): `nodes` an abi.NodeDesc array of
        every node of the scene, the item's own pose."""
        arr = (abi.BatchItem * len(items))()
        for i, it in enumerate(items):
            sid, v, t = it[0], it[1], it[2]
            arr[i].scene_id = sid
            arr[i].view = abi.view_desc(v)
            arr[i].target = t
            if len(it) > 3 and it[3] is not None:
                arr[i].nodes = C.cast(it[3], C.POINTER(abi.NodeDesc))
                arr[i].n_nodes = len(it[3])
        opts = abi.BatchOpts(tile, span_bin, 1 if use_graph else 0)
        fs = abi.FrameStats()
        self._check(self.lib.sgl_render_batch(self.ctx, arr, len(items), C.byref(opts), C.c_void_p(stream),
                                              C.byref(fs) if stats else None))
        return _stats_dict(fs) if stats else None

    def autotune(self, items) -> dict:
        arr = (abi.BatchItem * len(items))()
        for i, (sid, v, t) in enumerate(items):
            arr[i].scene_id = sid
            arr[i].view = abi.view_desc(v)
            arr[i].target = t
        opts = abi.BatchOpts()
        self._check(self.lib.sgl_autotune(self.ctx, arr, len(items), C.byref(opts)))
        return {"tile": opts.tile, "span_bin": opts.span_bin, "use_graph": opts.use_graph}

    # depth of field -------------------------------------------------------
    def dof(self, view, pixels: np.ndarray, zbuffer: np.ndarray) -> np.ndarray:
        """The depth-of-field gather on a host frame (h, w) and its z-buffer."""
        h, w = pixels.shape
        src = np.ascontiguousarray(pixels, np.uint32)
        z = np.ascontiguousarray(zbuffer, np.float32)
        out = np.zeros_like(src)
        vd = abi.view_desc(view)
        vd.x = vd.y = 0
        t_in = abi.Target(src.ctypes.data, 4 * w, w, h, z.ctypes.data_as(C.POINTER(C.c_float)))
        t_out = abi.Target(out.ctypes.data, 4 * w, w, h, None)
        self._check(self.lib.sgl_dof(self.ctx, C.byref(vd), C.byref(t_in), C.byref(t_out), 0, None))
        return out

    def server(self, budget_bytes: int = 0, max_batch: int = 0, streams: int = 0, copy_out: bool = True):
        return Server(self, budget_bytes, max_batch, streams, copy_out)

    # per-kernel device timing ----------------------------------------------
    def profile(self, enable: bool = True):
        self._check(self.lib.sgl_profile(self.ctx, 1 if enable else 0))

    def profile_read(self) -> dict:
        out = {}
        k = 0
        while True:
            name, ms, n = C.c_char_p(), C.c_double(), C.c_uint64()
            st = self.lib.sgl_profile_read(self.ctx, k, C.byref(name), C.byref(ms), C.byref(n))
            if st == -4:
                break
            self._check(st)
            out[name.value.decode()] = {"total_ms": ms.value, "launches": n.value}
            k += 1
        return out


def _stats_dict(fs: abi.FrameStats) -> dict:
    return {"triangles": fs.triangles, "drawn_triangles": fs.drawn_triangles, "fragments": fs.fragments,
            "pixels": fs.pixels, "kernel_launches": fs.kernel_launches}


class Server:
    """The continuous-batching request loop of the library (sgl_server_*)."""

    def __init__(self, renderer: Renderer, budget_bytes=0, max_batch=0, streams=0, copy_out=True):
        self.r = renderer
        self.lib = renderer.lib
        opts = abi.ServeOpts(budget_bytes, max_batch, streams, 1 if copy_out else 0)
        h = C.c_void_p()
        self.r._check(self.lib.sgl_server_create(self.r.ctx, C.byref(opts), C.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, scene_id: int, view, host_pixels: np.ndarray | None = None,
               host_zbuffer: np.ndarray | None = None, nodes=None) -> int:
        """`nodes`: an abi.NodeDesc array (every node of the scene) to render
        this request with, e.g. GltfScene.animate(t)."""
        req = abi.Request()
        req.scene_id = scene_id
        req.view = abi.view_desc(view)
        if nodes is not None:
            req.nodes = C.cast(nodes, C.POINTER(abi.NodeDesc))
            req.n_nodes = len(nodes)
        if host_pixels is not None:
            req.host_pixels = host_pixels.ctypes.data_as(C.POINTER(C.c_uint32))
        if host_zbuffer is not None:
            req.host_zbuffer = host_zbuffer.ctypes.data_as(C.POINTER(C.c_float))
        t = C.c_uint64()
        st = self.lib.sgl_server_submit(self.h, C.byref(req), C.byref(t))
        if st != 0:
            raise SglError(st, "sgl_server_submit")
        self._keep[t.value] = (host_pixels, host_zbuffer)
        return t.value

    @staticmethod
    def requests(items) -> "C.Array":
        """An abi.Request array for submit_many: items of (scene_id, view) or
        (scene_id, view, host_pixels, host_zbuffer), host buffers as numpy
        arrays (the caller keeps them alive until the results)."""
        arr = (abi.Request * len(items))()
        for r, it in zip(arr, items):
            r.scene_id = it[0]
            r.view = abi.view_desc(it[1])
            if len(it) > 2 and it[2] is not None:
                r.host_pixels = it[2].ctypes.data_as(C.POINTER(C.c_uint32))
            if len(it) > 3 and it[3] is not None:
                r.host_zbuffer = it[3].ctypes.data_as(C.POINTER(C.c_float))
        return arr

    def submit_many(self, reqs) -> np.ndarray:
        """Queue an abi.Request array (Server.requests) in one call; returns
        the tickets."""
        tickets = np.zeros(len(reqs), np.uint64)
        queued = C.c_int()
        st = self.lib.sgl_server_submit_batch(self.h, reqs, len(reqs), tickets.ctypes.data_as(C.POINTER(C.c_uint64)),
                                              C.byref(queued))
        if st != 0:
            raise SglError(st, f"sgl_server_submit_batch (queued {queued.value} of {len(reqs)})")
        return tickets

    def wait_many(self, tickets: np.ndarray, timeout_s: float = 60.0) -> "C.Array":
        """Wait for every ticket; returns their abi.RequestResult array."""
        tickets = np.ascontiguousarray(tickets, np.uint64)
        res = (abi.RequestResult * len(tickets))()
        st = self.lib.sgl_server_wait_batch(self.h, tickets.ctypes.data_as(C.POINTER(C.c_uint64)), len(tickets),
                                            timeout_s, res)
        if st != 0:
            raise SglError(st, "sgl_server_wait_batch")
        return res

    def _result(self, res: abi.RequestResult) -> dict:
        return {"status": res.status, "submit_s": res.submit_s, "start_s": res.start_s, "done_s": res.done_s,
                "rendered_s": res.rendered_s,
                "fragments": res.fragments}

    def poll(self, ticket: int):
        res = abi.RequestResult()
        st = self.lib.sgl_server_poll(self.h, ticket, C.byref(res))
        if st == -9:
            return None
        if st != 0:
            raise SglError(st, "sgl_server_poll")
        self._keep.pop(ticket, None)
        return self._result(res)

    def wait(self, ticket: int, timeout_s: float = 60.0) -> dict:
        res = abi.RequestResult()
        st = self.lib.sgl_server_wait(self.h, ticket, timeout_s, C.byref(res))
        if st != 0:
            raise SglError(st, "sgl_server_wait")
        self._keep.pop(ticket, None)
        return self._result(res)

    def drain(self, timeout_s: float = 120.0):
        st = self.lib.sgl_server_drain(self.h, timeout_s)
        if st != 0:
            raise SglError(st, "sgl_server_drain")

    def stats(self) -> dict:
        b, k, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.r._check(self.lib.sgl_server_stats(self.h, C.byref(b), C.byref(k), C.byref(c)))
        return {"batches": b.value, "kernels": k.value, "completed": c.value}

    def close(self):
        if self.h:
            self.lib.sgl_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
