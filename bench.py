#!/usr/bin/env python
"""Benchmark of the GB300 swegl renderer; prints ONE JSON line (rank 0).

Default workload, `serve` (the metric): 8 device-resident scenes of 200-style
UV spheres with 10k, 50k, 100k, 250k, 500k, 800k, 1.2M and 2M triangles; a
seeded request stream (Poisson arrivals at 2000 requests/s, uniform scene,
camera on a sphere of radius 35, viewport sides log-uniform 64..3840 x
64..2160, depth of field with probability 0.5) served by the library's
continuous-batching loop under a 40 GB budget.

  value     served frames/s at saturation: each step submits 4096 requests
            of the stream at once and drains them (closed loop).  Timed with
            CUDA events on the default stream, which the serving streams are
            ordered with.
  sequential_frames_per_s  the same requests through the plain
            one-frame-per-launch renderer, one call after another.
  latency   p50/p99/p999 with the requests submitted at their Poisson
            arrival times (open loop) for --duration seconds (60 by
            default), every frame copied to write-combined page-locked host
            memory (sgl_host_alloc): delivered
            (frame in the caller's buffers) and rendered (frame complete in
            device memory) latencies of the same run.
  e2e       closed loop through the public API, every frame (colour + depth)
            copied to write-combined page-locked host memory, in pipelined
            chunks of 256 requests for at least 2 s.
Request descriptors are packed before the timed regions (the application's
own work); a step queues them with one sgl_server_submit_batch call.
  roofline  the plain renderer's 1080p frame of the 200-sphere scene
            (819,200 triangles): algorithmic bytes / device time, against the
            measured HBM copy bandwidth; per-stage times from CUDA events.

Inputs are larger than L2: the 8 resident scenes hold ~1.9 GB.  Under
torchrun (N > 1) every rank serves its own stream (replicas, no collective);
value sums the frames of all ranks over the max-over-ranks time.

--workload frame times the plain renderer alone on the 1080p frame.
--workload batch64 times 64 viewports of uneven size in one graph-captured
launch sequence (autotuned tile and span bin) against the same views one
frame per launch sequence.
--workload layers times a 1080p frame with 4 transparency layers of the
200-sphere scene whose textures carry block alpha (translucent spheres).
--impl reference times the reference's CPU algorithm (the oracle's C
restatement, oracle/sgl_oracle.c) on all host threads on the same requests.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "served frames/s + p50/p99 latency vs one-frame-per-launch, same GPU, <=1 LSB RGB"


# ----------------------------------------------------------------- helpers --
def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_traffic(name: str):
    """Per-frame DRAM traffic from the committed ncu summary (profiles/)."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_frame:"):
            return float(line.split(":", 1)[1])
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def frame_alg_bytes(scene, w: int, h: int, dof: bool = False) -> int:
    """Algorithmic bytes of one frame: 32 B per vertex (position, normal, uv),
    4 B per index, 4 B per texel of every texture, 8 B per viewport pixel
    (BGRA8 colour + FP32 depth written once); with depth of field 12 B more
    per pixel (the gather reads colour and depth once and writes colour)."""
    texels = sum(int(t.size) for t in scene.textures)
    return 32 * len(scene.positions) + 4 * len(scene.indices) + 4 * texels + (20 if dof else 8) * w * h


# The plain-renderer frame workloads: (config name, viewport, depth of field,
# committed ncu traffic summary)
FRAMES = {
    "frame": ("spheres200_1080p_frame", (1920, 1080), False, "frame_1080p_traffic.md"),
    "dof": ("spheres200_4k_dof_frame", (3840, 2160), True, "frame_4k_dof_traffic.md"),
}


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def device_target(torch, w: int, h: int):
    from swegl_gb300 import abi

    pix = torch.zeros((h, w), dtype=torch.int32, device="cuda")
    zb = torch.zeros((h, w), dtype=torch.float32, device="cuda")
    t = abi.Target()
    t.pixels = pix.data_ptr()
    t.pitch = 4 * w
    t.width, t.height = w, h
    t.zbuffer = C.cast(C.c_void_p(zb.data_ptr()), C.POINTER(C.c_float))
    return (pix, zb), t


def max_over_ranks(torch, dist, x: float, device: str = "cuda") -> float:
    """Replicas: the job's time is the slowest rank's."""
    if not dist:
        return x
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(torch, dist, x: float, device: str = "cuda") -> float:
    if not dist:
        return x
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def replica_throughput(frames_per_rank: int, world: int, max_ms: float) -> float:
    """Whole-job frames/s of independent replicas: all ranks' frames over the
    slowest rank's time."""
    return world * frames_per_rank / (max_ms / 1e3)


# ------------------------------------------------------- single-frame stage --
def frame_measure(r, torch, steps: int, warmup: int, with_e2e: bool, kind: str = "frame"):
    """The plain renderer on a frame of the 200-sphere scene (the 1080p
    frame, or the 3840x2160 frame with depth of field: focus 20, aperture
    0.05, radius at most 16 px, 32 taps); 4 resident copies of the scene
    (~400 MB, above the 129 MB L2) rendered in rotation."""
    from swegl_gb300 import abi
    from swegl_gb300 import scenes as S

    _, (w, h), dof, _ = FRAMES[kind]
    scene = S.spheres_scene()
    v = S.spheres_view(w, h)
    v.dof = dof
    copies = [r.upload(scene) for _ in range(4)]
    stream = torch.cuda.Stream()
    _bufs, tgt = device_target(torch, v.w, v.h)

    def step(k):
        r.render_device(copies[k % len(copies)], [v], [tgt], stream=stream.cuda_stream)

    for k in range(warmup):
        step(k)
    torch.cuda.synchronize()
    stats = r.render_device(copies[0], [v], [tgt], stream=stream.cuda_stream, stats=True)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        starts[k].record(stream)
        step(k)
        ends[k].record(stream)
    torch.cuda.synchronize()
    frame_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / steps
    # per-stage times in a separate pass: the stage events add their own gaps
    r.profile(True)
    for k in range(steps):
        step(k)
    torch.cuda.synchronize()
    prof = r.profile_read()
    r.profile(False)
    out = {"frame_ms": frame_ms, "stats": stats, "prof": prof, "alg_bytes": frame_alg_bytes(scene, v.w, v.h, dof),
           "kind": kind,
           "gpu_frame": (_bufs[0].cpu().numpy().view(np.uint32), _bufs[1].cpu().numpy())}
    if with_e2e:
        host_pix = torch.zeros((v.h, v.w), dtype=torch.int32).pin_memory()
        host_z = torch.zeros((v.h, v.w), dtype=torch.float32).pin_memory()
        htgt = abi.Target()
        htgt.pixels = host_pix.data_ptr()
        htgt.pitch = 4 * v.w
        htgt.width, htgt.height = v.w, v.h
        htgt.zbuffer = C.cast(C.c_void_p(host_z.data_ptr()), C.POINTER(C.c_float))
        vd = (abi.ViewDesc * 1)(abi.view_desc(v))
        td = (abi.Target * 1)(htgt)
        for k in range(warmup):
            r.lib.sgl_render(r.ctx, copies[k % 4], vd, td, 1, 0, None, None)
        t0 = time.perf_counter()
        for k in range(steps):
            st = r.lib.sgl_render(r.ctx, copies[k % 4], vd, td, 1, 0, None, None)
            if st != 0:
                raise RuntimeError(f"sgl_render failed: {st}")
        out["e2e_fps"] = steps / (time.perf_counter() - t0)
        out["view_bytes"] = C.sizeof(abi.ViewDesc)
        out["frame_bytes"] = 8 * v.w * v.h
    for c in copies:
        r.release(c)
    out["scene"] = scene
    out["view"] = v
    return out


def roofline_of(fm: dict) -> dict:
    peaks = measured_peaks()
    _, (w, h), dof, traffic = FRAMES[fm.get("kind", "frame")]
    achieved = fm["alg_bytes"] / (fm["frame_ms"] / 1e3) / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / peaks["hbm_gbs"], 4), "peak_source": peaks["source"],
            "unit_of_work": "one %dx%d frame%s of the 819,200-triangle scene (%d algorithmic bytes)"
                            % (w, h, " with depth of field" if dof else "", fm["alg_bytes"]),
            "frame_us": round(1e3 * fm["frame_ms"], 2),
            "traffic": profile_traffic(traffic)}


def kernels_of(fm: dict) -> dict:
    return {k: {"avg_us": round(1e3 * d["total_ms"] / max(1, d["launches"]), 2)} for k, d in fm["prof"].items()
            if d["launches"]}


# --------------------------------------------------------------- workloads --
def run_frame(args, rank, world, local_rank):
    import torch

    from swegl_gb300.runtime import Renderer

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    r = Renderer(local_rank)
    if dist:
        dist.barrier()
    with ClockSampler(local_rank) as clocks:
        fm = frame_measure(r, torch, args.steps, args.warmup, True, args.workload)
    frame_ms = max_over_ranks(torch, dist, fm["frame_ms"])
    name, (w, h), dof, _ = FRAMES[args.workload]
    fps = world * 1e3 / frame_ms
    e2e = sum_over_ranks(torch, dist, fm["e2e_fps"]) if dist else fm["e2e_fps"]
    prof = fm["prof"]
    out = {
        "metric": "frames/s (plain renderer, one %dx%d frame%s per launch sequence)"
                  % (w, h, " with depth of field" if dof else ""),
        "value": round(fps, 2), "unit": "frames/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(frame_ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded scenes, swegl_gb300/scenes.py)",
        "config": {"workload": name, "triangles": fm["scene"].n_triangles, "viewport": "%dx%d" % (w, h),
                   "l2": "inputs larger than L2: 4 resident scene copies in rotation"},
        "gfragments_per_s": round(fm["stats"]["fragments"] * fps / 1e9, 3),
        "kernels": kernels_of(fm),
        "dominant_kernel": max(prof.items(), key=lambda kv: kv[1]["total_ms"])[0] if prof else None,
        "roofline": roofline_of(fm),
        "e2e": {"value": round(e2e, 2), "unit": "frames/s", "h2d_bytes_per_step": fm["view_bytes"],
                "d2h_bytes_per_step": fm["frame_bytes"]},
        "gpu_launches": int(fm["stats"]["kernel_launches"]) * args.steps,
        "clocks": clocks.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_frame_baseline(fm["scene"], fm["view"], args, fm["gpu_frame"])
    r.close()
    if dist:
        dist.destroy_process_group()
    return out if rank == 0 else None


def cpu_frame_baseline(scene, view, args, gpu_frame=None) -> dict:
    import oracle

    threads = cpu_threads()
    # single-thread latency of one frame (median of 3), then throughput on every thread
    lat = []
    for _ in range(3):
        t1 = time.perf_counter()
        oracle.render(scene, [view])
        lat.append(time.perf_counter() - t1)
    first = oracle.render_parallel(scene, [view] * threads, threads)
    # about args.cpu_seconds of host work, one frame per thread at a time
    n, t0 = 0, time.perf_counter()
    while n < args.cpu_frames and (time.perf_counter() - t0) < args.cpu_seconds:
        oracle.render_parallel(scene, [view] * threads, threads)
        n += threads
    dt = time.perf_counter() - t0
    out = {"value": round(n / dt, 3), "unit": "frames/s", "cores": threads, "kind": "port",
           "sample": f"{n} frames of the {view.w}x{view.h} frame{' with depth of field' if view.dof else ''} "
                     f"on {threads} threads ({dt:.1f} s)",
           "single_thread_ms": round(1e3 * statistics.median(lat), 2)}
    if gpu_frame is not None:
        out["parity"] = parity_of([gpu_frame], first[:1])
    return out


# ------------------------------------------------------ transparency layers --
def layers_scene_view():
    """The 200-sphere scene (819,200 triangles) with 8 block-alpha textures
    (1024^2, 64-texel squares: 3/8 opaque, 1/8 clear, 1/2 translucent) and its
    1080p camera with 4 transparency layers."""
    from swegl_gb300 import scenes as S

    texs = [S.texture_block_alpha(900 + t, 1024, 1024, 64) for t in range(8)]
    scene = S.spheres_scene(textures=texs)
    v = S.spheres_view(1920, 1080)
    v.layers = 4
    return scene, v


def run_layers(args, rank, world, local_rank):
    import torch

    from swegl_gb300 import abi
    from swegl_gb300.runtime import Renderer

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    r = Renderer(local_rank)
    scene, v = layers_scene_view()
    copies = [r.upload(scene) for _ in range(2)]  # ~270 MB in rotation, above L2
    stream = torch.cuda.Stream()
    bufs, tgt = device_target(torch, v.w, v.h)

    def step(k):
        r.render_device(copies[k % len(copies)], [v], [tgt], stream=stream.cuda_stream)

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    stats = r.render_device(copies[0], [v], [tgt], stream=stream.cuda_stream, stats=True)
    gpu_frame = (bufs[0].cpu().numpy().view(np.uint32).copy(), bufs[1].cpu().numpy().copy())
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        for k in range(args.steps):
            starts[k].record(stream)
            step(k)
            ends[k].record(stream)
        torch.cuda.synchronize()
    frame_ms = max_over_ranks(torch, dist, sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / args.steps)
    r.profile(True)
    for k in range(args.steps):
        step(k)
    torch.cuda.synchronize()
    prof = r.profile_read()
    r.profile(False)
    # end to end: host surface and depth buffer through sgl_render
    host_pix = torch.zeros((v.h, v.w), dtype=torch.int32).pin_memory()
    host_z = torch.zeros((v.h, v.w), dtype=torch.float32).pin_memory()
    htgt = abi.Target()
    htgt.pixels = host_pix.data_ptr()
    htgt.pitch = 4 * v.w
    htgt.width, htgt.height = v.w, v.h
    htgt.zbuffer = C.cast(C.c_void_p(host_z.data_ptr()), C.POINTER(C.c_float))
    vd = (abi.ViewDesc * 1)(abi.view_desc(v))
    td = (abi.Target * 1)(htgt)
    for k in range(args.warmup):
        r.lib.sgl_render(r.ctx, copies[k % 2], vd, td, 1, 0, None, None)
    t0 = time.perf_counter()
    for k in range(args.steps):
        st = r.lib.sgl_render(r.ctx, copies[k % 2], vd, td, 1, 0, None, None)
        if st != 0:
            raise RuntimeError(f"sgl_render failed: {st}")
    e2e_fps = args.steps / (time.perf_counter() - t0)
    e2e = sum_over_ranks(torch, dist, e2e_fps) if dist else e2e_fps
    fps = world * 1e3 / frame_ms
    fm = {"frame_ms": frame_ms, "prof": prof, "alg_bytes": frame_alg_bytes(scene, v.w, v.h)}
    out = {
        "metric": "frames/s (1080p frame with 4 transparency layers)",
        "value": round(fps, 2), "unit": "frames/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(frame_ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded scene, swegl_gb300/scenes.py)",
        "config": {"workload": "translucent_spheres200_1080p_4layers", "triangles": scene.n_triangles,
                   "viewport": "1920x1080", "layers": v.layers,
                   "l2": "inputs larger than L2: 2 resident scene copies in rotation"},
        "fragments": int(stats["fragments"]),
        "kernels": kernels_of(fm),
        "dominant_kernel": max(prof.items(), key=lambda kv: kv[1]["total_ms"])[0] if prof else None,
        "e2e": {"value": round(e2e, 2), "unit": "frames/s", "h2d_bytes_per_step": 4 * v.w * v.h + C.sizeof(abi.ViewDesc),
                "d2h_bytes_per_step": 8 * v.w * v.h},
        "gpu_launches": int(stats["kernel_launches"]) * args.steps,
        "clocks": clocks.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_frame_baseline(scene, v, args, gpu_frame)
    for c in copies:
        r.release(c)
    r.close()
    if dist:
        dist.destroy_process_group()
    return out if rank == 0 else None


# ----------------------------------------------------------- 64-view batch --
def run_batch64(args, rank, world, local_rank):
    """64 viewports of the 200-sphere scene (seeded cameras on a sphere of
    radius 35, sizes log-uniform 128x128 ... 1920x1080) in one graph-captured
    launch sequence with the autotuner's tile and span bin, against the same
    64 views through the plain one-frame-per-launch renderer."""
    import torch

    from swegl_gb300 import scenes as S
    from swegl_gb300.runtime import Renderer

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    r = Renderer(local_rank)
    scene = S.spheres_scene()
    views = S.batch_views(64)
    copies = [r.upload(scene) for _ in range(4)]  # ~400 MB in rotation, above L2
    bufs, tgts = [], []
    for v in views:
        b, t = device_target(torch, v.w, v.h)
        bufs.append(b)
        tgts.append(t)
    items = lambda c: [(c, v, t) for v, t in zip(views, tgts)]  # noqa: E731
    chosen = r.autotune(items(copies[0]))
    stream = torch.cuda.Stream()

    def step(k):
        r.render_batch(items(copies[k % len(copies)]), tile=chosen["tile"], span_bin=chosen["span_bin"],
                       use_graph=True, stream=stream.cuda_stream)

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    st = r.render_batch(items(copies[0]), tile=chosen["tile"], span_bin=chosen["span_bin"], use_graph=True,
                        stream=stream.cuda_stream, stats=True)
    torch.cuda.synchronize()
    gpu_frames = [(p.cpu().numpy().view(np.uint32).copy(), z.cpu().numpy().copy()) for (p, z) in bufs]
    if dist:
        dist.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local_rank) as clocks:
        for k in range(args.steps):
            starts[k].record(stream)
            step(k)
            ends[k].record(stream)
        torch.cuda.synchronize()
    batch_ms = max_over_ranks(torch, dist, sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / args.steps)
    # the same 64 views one frame per launch sequence
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for k in range(2):
        for i, v in enumerate(views):
            r.render_device(copies[k % len(copies)], [v], [tgts[i]], stream=stream.cuda_stream)
    torch.cuda.synchronize()
    seq = []
    for k in range(args.steps):
        e0.record(stream)
        for i, v in enumerate(views):
            r.render_device(copies[k % len(copies)], [v], [tgts[i]], stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        seq.append(e0.elapsed_time(e1))
    seq_ms = max_over_ranks(torch, dist, sum(seq) / len(seq))
    # end to end: the batch, then every frame (colour + depth) to pinned host memory
    host = [(torch.empty((v.h, v.w), dtype=torch.int32).pin_memory(),
             torch.empty((v.h, v.w), dtype=torch.float32).pin_memory()) for v in views]
    d2h = sum(8 * v.w * v.h for v in views)
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(k)
        with torch.cuda.stream(stream):
            for (hp, hz), (dp, dz) in zip(host, bufs):
                hp.copy_(dp, non_blocking=True)
                hz.copy_(dz, non_blocking=True)
        stream.synchronize()
    e2e_fps = 64 * args.steps / (time.perf_counter() - t0)
    from swegl_gb300 import abi

    fps = world * 64 * 1e3 / batch_ms
    px = sum(v.w * v.h for v in views)
    alg = sum(frame_alg_bytes(scene, v.w, v.h) for v in views)
    peaks = measured_peaks()
    achieved = alg / (batch_ms / 1e3) / 1e9
    out = {
        "metric": "frames/s (64 viewports of uneven size in one graph-captured launch sequence)",
        "value": round(fps, 2), "unit": "frames/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(batch_ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded scene and cameras, swegl_gb300/scenes.py)",
        "config": {"workload": "spheres200_64_viewports_batch", "triangles": scene.n_triangles, "views": 64,
                   "pixels": px, "viewports": "log-uniform 128x128..1920x1080, cameras on a sphere of radius 35",
                   "autotuned": chosen,
                   "l2": "inputs larger than L2: 4 resident scene copies in rotation, 64 frames of %d MB"
                         % (8 * px // 1000000)},
        "sequential_frames_per_s": round(world * 64 * 1e3 / seq_ms, 2),
        "batched_over_sequential": round(seq_ms / batch_ms, 3),
        "gfragments_per_s": round(st["fragments"] * world * 1e3 / batch_ms / 1e9, 3),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4), "peak_source": peaks["source"],
                     "unit_of_work": "64 views, each charged the algorithmic bytes of a frame of the scene "
                                     "(%d bytes in all)" % alg, "traffic": None},
        "e2e": {"value": round(e2e_fps, 2), "unit": "frames/s", "h2d_bytes_per_step": 64 * C.sizeof(abi.BatchItem),
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(st["kernel_launches"]) * args.steps,
        "clocks": clocks.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle

        threads = cpu_threads()
        t1 = time.perf_counter()
        cpu_frames = oracle.render_parallel(scene, views, threads)
        dt = time.perf_counter() - t1
        out["cpu_baseline"] = {"value": round(64 / dt, 3), "unit": "frames/s", "cores": threads, "kind": "port",
                               "sample": f"the 64 views on {threads} threads ({dt:.1f} s)",
                               "parity": parity_of(gpu_frames, cpu_frames)}
    for c in copies:
        r.release(c)
    r.close()
    if dist:
        dist.destroy_process_group()
    return out if rank == 0 else None


def serve_config(args) -> dict:
    from swegl_gb300 import scenes as S

    return {"workload": "serving: 8 resident scenes, Poisson 2000 req/s, viewports 64^2..3840x2160, DoF p=0.5",
            "scene_triangles": list(S.SERVE_TRIANGLES), "requests_per_step": args.requests_per_step,
            "budget_bytes": args.budget, "max_batch": args.max_batch, "streams": args.streams,
            "latency_duration_s": args.duration, "arrival_rate": 2000,
            "timed_requests": args.steps * args.requests_per_step,
            "l2": "inputs larger than L2: 8 resident scenes of ~1.9 GB"}


def run_serve(args, rank, world, local_rank):
    import torch

    from swegl_gb300 import scenes as S
    from swegl_gb300.runtime import Renderer

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    scenes = S.serving_scenes()
    r = Renderer(local_rank)
    sids = [r.upload(sc) for sc in scenes]
    M = args.requests_per_step
    reqs = S.serving_requests((args.warmup + args.steps) * M, seed=60 + rank)
    srv = r.server(budget_bytes=args.budget, max_batch=args.max_batch, streams=args.streams, copy_out=False)
    # the request descriptors of every step, packed before the timed region
    # (the application's own work); each step queues its requests with one
    # sgl_server_submit_batch call and waits for all of them
    from swegl_gb300.runtime import Server

    def pack(chunk):
        return Server.requests([(sids[k], v) for (_, k, v) in chunk])

    def serve_chunk(packed, server):
        server.submit_many(packed)
        server.drain(600.0)

    steps_packed = [pack(reqs[s * M:(s + 1) * M]) for s in range(args.warmup + args.steps)]

    # warm-up: graphs captured, pools grown
    for s in range(args.warmup):
        serve_chunk(steps_packed[s], srv)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    b0 = srv.stats()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local_rank) as clocks:
        for s in range(args.steps):
            torch.cuda.synchronize()
            starts[s].record()
            serve_chunk(steps_packed[args.warmup + s], srv)
            ends[s].record()
            torch.cuda.synchronize()
    b1 = srv.stats()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = max_over_ranks(torch, dist, sum(step_ms))
    value = replica_throughput(args.steps * M, world, total_ms)
    timed = reqs[args.warmup * M:]

    # sequential one-frame-per-launch on the same requests (a bounded prefix):
    # sgl_render per request on device targets, descriptors packed beforehand
    from swegl_gb300 import abi

    n_seq = min(len(timed), args.seq_requests)
    big = max(v.w * v.h for (_, _, v) in timed[:n_seq])
    _bufs, tgt = device_target(torch, 3840, max(1, -(-big // 3840)))
    stream = torch.cuda.Stream()
    seq_desc = [(sids[k], abi.view_desc(v), _retarget(tgt, v)) for (_, k, v) in timed[:n_seq]]

    def render_one(sid, vd, td):
        st = r.lib.sgl_render(r.ctx, sid, C.byref(vd), C.byref(td), 1, 1, C.c_void_p(stream.cuda_stream), None)
        if st != 0:
            raise RuntimeError(f"sgl_render failed: {st}")

    for d in seq_desc[:8]:
        render_one(*d)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for d in seq_desc:
        render_one(*d)
    e1.record(stream)
    torch.cuda.synchronize()
    seq_fps = n_seq / (e0.elapsed_time(e1) / 1e3)
    # the batched loop on the very same prefix, for a like-for-like ratio
    prefix = pack(timed[:n_seq])
    torch.cuda.synchronize()
    e0.record()
    serve_chunk(prefix, srv)
    e1.record()
    torch.cuda.synchronize()
    batched_same_fps = n_seq / (e0.elapsed_time(e1) / 1e3)

    srv.close()
    # e2e: closed loop with every frame copied to page-locked host memory.
    # The frames go to write-combined memory: copies into ordinary page-locked
    # memory slowed down the longer the host had been running (29.8 k frames/s
    # on a fresh host, 19.9-27.0 k a minute later, with the device-only rate
    # and the raw copy rate unchanged), into write-combined memory they did not
    # (27.6-28.1 k in both states)
    e2e = e2e_run(r, torch, sids, timed, args)

    # open-loop latency at the Poisson arrival times, frames delivered to the host
    lat = latency_run(r, torch, sids, args.duration, 70 + rank, args)

    kshares = serve_kernel_shares(r, torch, sids, timed[:args.profile_requests], args.max_batch)
    fm = frame_measure(r, torch, 10, 3, False)
    gpu_launches = int(b1["kernels"] - b0["kernels"])
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded scenes and request stream, swegl_gb300/scenes.py)",
        "config": serve_config(args),
        "sequential_frames_per_s": round(seq_fps, 2),
        "batched_frames_per_s_same_requests": round(batched_same_fps, 2),
        "sequential_requests": n_seq,
        "latency_ms": lat,
        "kernels": kshares,
        "batches": int(b1["batches"] - b0["batches"]),
        "frame_1080p": {"frames_per_s": round(1e3 / fm["frame_ms"], 1), "kernels": kernels_of(fm)},
        "roofline": roofline_of(fm),
        "e2e": {"value": round(e2e["fps"], 2), "unit": "frames/s", "h2d_bytes_per_step": e2e["h2d"],
                "d2h_bytes_per_step": e2e["d2h"], "step": "%d requests submitted together" % args.e2e_chunk,
                "host_frames": "write-combined page-locked memory (sgl_host_alloc)",
                "chunks": e2e["chunks"], "requests": e2e["requests"], "seconds": round(e2e["seconds"], 2)},
        "gpu_launches": gpu_launches,
        "clocks": clocks.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        gpu_frames = gpu_sample_frames(r, sids, timed[:args.cpu_requests])
        out["cpu_baseline"] = cpu_serve_baseline(scenes, timed, args, gpu_frames)
    r.close()
    if dist:
        dist.destroy_process_group()
    return out if rank == 0 else None


def serve_kernel_shares(r, torch, sids, sample, batch: int) -> dict:
    """Device time per kernel of the serving stream's work: the sample's
    requests in batches of `batch` (in arrival order, as the serving loop forms
    them at saturation), launched directly with CUDA events around each kernel
    (sgl_profile), in microseconds per request and as shares."""
    from swegl_gb300 import abi

    if not sample:
        return {}
    per = max(2 * v.w * v.h for (_, _, v) in sample)
    pool = torch.zeros(batch * per + 16, dtype=torch.int32, device="cuda")
    base = pool.data_ptr()
    batches = []
    for i in range(0, len(sample), batch):
        items, off = [], 0
        for (_, k, v) in sample[i:i + batch]:
            t = abi.Target()
            t.pixels = base + 4 * off
            t.pitch = 4 * v.w
            t.width, t.height = v.w, v.h
            t.zbuffer = C.cast(C.c_void_p(base + 4 * (off + v.w * v.h)), C.POINTER(C.c_float))
            off += 2 * v.w * v.h
            items.append((sids[k], v, t))
        batches.append(items)
    r.render_batch(batches[0], use_graph=False)
    torch.cuda.synchronize()
    r.profile(True)
    for items in batches:
        r.render_batch(items, use_graph=False)
    torch.cuda.synchronize()
    prof = r.profile_read()
    r.profile(False)
    total = sum(d["total_ms"] for d in prof.values()) or 1.0
    return {"requests": len(sample), "batch": batch,
            "per_kernel": {k: {"us_per_request": round(1e3 * d["total_ms"] / len(sample), 2),
                               "share": round(d["total_ms"] / total, 3)}
                           for k, d in prof.items() if d["launches"]}}


def _retarget(tgt, v):
    from swegl_gb300 import abi

    t = abi.Target()
    t.pixels = tgt.pixels
    t.pitch = 4 * v.w
    t.width, t.height = v.w, v.h
    t.zbuffer = tgt.zbuffer
    return t


def _pct(a: np.ndarray) -> dict:
    return {"p50": round(float(np.percentile(a, 50)), 3), "p99": round(float(np.percentile(a, 99)), 3),
            "p999": round(float(np.percentile(a, 99.9)), 3), "mean": round(float(a.mean()), 3)}


class PinnedRing:
    """Host frame buffers for the requests in flight, carved in order from one
    pinned pool (write-combined, sgl_host_alloc); a region is reused once the
    requests holding it are done (their results are collected then)."""

    def __init__(self, torch, srv, nbytes: int):
        from swegl_gb300.runtime import host_buffer

        self.pool = host_buffer(nbytes // 4)
        self.n = self.pool.size
        self.srv = srv
        self.head = 0
        self.live = []  # (ticket, start, end) in submission order
        self.results = {}

    def _retire_first(self):
        t, _, _ = self.live.pop(0)
        self.results[t] = self.srv.wait(t, 600.0)

    def take(self, words: int):
        if words > self.n:
            raise RuntimeError("frame larger than the pinned ring")
        if self.head + words > self.n:
            self.head = 0
        lo, hi = self.head, self.head + words
        while self.live and any(not (e <= lo or s >= hi) for (_, s, e) in self.live):
            self._retire_first()
        self.head = hi
        return lo, hi

    def submit(self, sid, v):
        px = v.w * v.h
        lo, hi = self.take(2 * px)
        pix = self.pool[lo:lo + px].reshape(v.h, v.w)
        z = self.pool[lo + px:hi].view(np.float32).reshape(v.h, v.w)
        t = self.srv.submit(sid, v, pix, z)
        self.live.append((t, lo, hi))
        return t

    def finish(self):
        while self.live:
            self._retire_first()
        return self.results


def latency_run(r, torch, sids, duration: float, seed: int, args) -> dict:
    """Open loop: the requests of a seeded stream submitted at their Poisson
    arrival times for `duration` seconds, through a server that copies every
    frame (colour + depth) to pinned host memory.  Two latencies per request:
    delivered (submit -> frame in the caller's host buffers) and rendered
    (submit -> frame complete in device memory, before its copy)."""
    from swegl_gb300 import scenes as S

    stream_reqs = S.serving_requests(int(2000 * duration * 1.05) + 16, seed=seed)
    stream_reqs = [q for q in stream_reqs if q[0] <= duration]
    srv = r.server(budget_bytes=args.budget, max_batch=args.max_batch, streams=args.streams, copy_out=True)
    ring = PinnedRing(torch, srv, args.ring_bytes)
    t0 = time.perf_counter()
    tickets = []
    for (arrival, k, v) in stream_reqs:
        while True:
            dt = arrival - (time.perf_counter() - t0)
            if dt <= 0:
                break
            if dt > 0.0005:
                time.sleep(dt - 0.0003)
        tickets.append(ring.submit(sids[k], v))
    res = ring.finish()
    wall = time.perf_counter() - t0
    srv.close()
    results = [res[t] for t in tickets]
    assert all(x["status"] == 0 for x in results)
    delivered = np.array([1e3 * (x["done_s"] - x["submit_s"]) for x in results])
    rendered = np.array([1e3 * (x["rendered_s"] - x["submit_s"]) for x in results])
    return {"delivered": _pct(delivered), "rendered": _pct(rendered), "requests": len(results),
            "duration_s": duration, "served_frames_per_s": round(len(results) / wall, 1), "offered_rate": 2000,
            "delivered_bytes": int(sum(8 * v.w * v.h for (_, _, v) in stream_reqs))}


def e2e_run(r, torch, sids, timed, args):
    """Closed loop through the public API with every frame (colour + depth)
    copied to page-locked host memory: chunks of args.e2e_chunk requests of the
    stream, each chunk's frames into one half of a write-combined page-locked
    pool from sgl_host_alloc (chunk k + 2
    reuses chunk k's half once chunk k is delivered, so the GPU is never left
    idle between chunks); chunks are taken from the stream's timed requests in
    turn until at least args.e2e_seconds have passed (and at least 8 chunks).
    A chunk is queued with one sgl_server_submit_batch call and collected with
    one sgl_server_wait_batch call; its request descriptors (view, camera,
    host buffer pointers) are packed before the timed region."""
    from swegl_gb300.runtime import Server, host_buffer

    M = args.e2e_chunk
    chunks = [timed[i:i + M] for i in range(0, len(timed) - M + 1, M)][:32] or [timed[:M]]
    half = max(sum(2 * v.w * v.h for (_, _, v) in ch) for ch in chunks) + 16
    pool = host_buffer(2 * half)  # write-combined page-locked memory (sgl_host_alloc)
    srv = r.server(budget_bytes=args.budget, max_batch=args.max_batch, streams=args.streams, copy_out=True)

    def pack(ch, h):
        off, items = h * half, []
        for (_, k, v) in ch:
            px = v.w * v.h
            items.append((sids[k], v, pool[off:off + px], pool[off + px:off + 2 * px].view(np.float32)))
            off += 2 * px
        return Server.requests(items)

    packed = [(pack(ch, 0), pack(ch, 1)) for ch in chunks]

    def collect(tk):
        res = srv.wait_many(tk, 600.0)
        assert all(x.status == 0 for x in res)

    collect(srv.submit_many(packed[0][0]))  # warm-up
    inflight = []
    n = nbytes = 0
    t0 = time.perf_counter()
    k = 0
    while True:
        if len(inflight) == 2:
            collect(inflight.pop(0))
        if k >= 8 and time.perf_counter() - t0 >= args.e2e_seconds:
            break
        c = k % len(chunks)
        inflight.append(srv.submit_many(packed[c][k % 2]))
        n += len(chunks[c])
        nbytes += sum(8 * v.w * v.h for (_, _, v) in chunks[c])
        k += 1
    for tk in inflight:
        collect(tk)
    dt = time.perf_counter() - t0
    srv.close()
    from swegl_gb300 import abi

    return {"fps": n / dt, "h2d": C.sizeof(abi.Request) * M, "d2h": int(nbytes / k), "chunks": k, "seconds": dt,
            "requests": n}


def parity_of(gpu_frames, cpu_frames) -> dict:
    """Depth bit-exactness and the per-pixel |dRGB| histogram (max over the
    three channels) of GPU frames against the oracle's frames of the same
    requests."""
    hist = np.zeros(4, np.int64)
    depth_ok = True
    px = 0
    for (gp, gz), cf in zip(gpu_frames, cpu_frames):
        depth_ok &= bool(np.array_equal(gz.view(np.uint32), cf.zbuffer.view(np.uint32)))
        a = gp.view(np.uint8).reshape(gp.shape + (4,))[..., :3].astype(np.int16)
        b = cf.pixels.view(np.uint8).reshape(cf.pixels.shape + (4,))[..., :3].astype(np.int16)
        d = np.abs(a - b).max(axis=-1)
        hist += np.bincount(np.minimum(d, 3).ravel(), minlength=4)[:4]
        px += d.size
    return {"frames": len(gpu_frames), "pixels": int(px), "depth_bit_exact": depth_ok,
            "rgb_abs_diff_hist_0_1_2_3plus": hist.tolist(),
            "within_1lsb": round(float(hist[:2].sum()) / max(px, 1), 6), "max_lsb_le_2": bool(hist[3] == 0)}


def gpu_sample_frames(r, sids, sample) -> list:
    """The GPU frames (colour, depth) of a bounded request sample, through the
    serving loop with copy-out."""
    srv = r.server(copy_out=True)
    out = []
    for (_, k, v) in sample:
        pix = np.zeros((v.h, v.w), np.uint32)
        z = np.zeros((v.h, v.w), np.float32)
        srv.submit(sids[k], v, pix, z)
        out.append((pix, z))
    srv.drain(600.0)
    srv.close()
    return out


def cpu_serve_baseline(scenes, timed, args, gpu_frames=None) -> dict:
    """The oracle restatement on all host threads over a bounded prefix of the
    request stream, grouped by scene; with the GPU frames of the same requests
    it also checks them (depth bits, |dRGB| histogram)."""
    import oracle

    threads = cpu_threads()
    chunk = args.cpu_requests

    def render_chunk(sample, keep: bool):
        by_scene = {}
        for j, (_, k, v) in enumerate(sample):
            by_scene.setdefault(k, []).append((j, v))
        frames_out = [None] * len(sample) if keep else None
        for k, jv in by_scene.items():
            frames = oracle.render_parallel(scenes[k], [v for (_, v) in jv], threads)
            if keep:
                for (j, _), f in zip(jv, frames):
                    frames_out[j] = f
        return frames_out

    # the first chunk is also the parity sample; then about args.cpu_seconds of host work in all
    n, t0 = 0, time.perf_counter()
    cpu_frames = render_chunk(timed[:chunk], True)
    n += len(timed[:chunk])
    while n + chunk <= len(timed) and (time.perf_counter() - t0) < args.cpu_seconds:
        render_chunk(timed[n:n + chunk], False)
        n += chunk
    dt = time.perf_counter() - t0
    # single-thread latency: requests of the stream one at a time on one thread
    lat, t1 = [], time.perf_counter()
    for (_, k, v) in timed:
        ta = time.perf_counter()
        oracle.render(scenes[k], [v])
        lat.append(time.perf_counter() - ta)
        if len(lat) >= 64 or time.perf_counter() - t1 >= args.cpu_seconds / 2:
            break
    out = {"value": round(n / dt, 3), "unit": "frames/s", "cores": threads, "kind": "port",
           "sample": f"the first {n} requests of the stream on {threads} threads ({dt:.1f} s)",
           "single_thread_ms": {"mean": round(1e3 * float(np.mean(lat)), 2),
                                "p50": round(1e3 * float(np.median(lat)), 2),
                                "requests": len(lat)}}
    if gpu_frames is not None:
        out["parity"] = parity_of(gpu_frames, cpu_frames)
    return out


def run_reference(args, rank, world):
    """The reference's CPU algorithm (the oracle restatement) on the host cores,
    same workload and metric; each step renders a bounded slice of requests."""
    if rank != 0:
        return None
    import oracle
    from swegl_gb300 import scenes as S

    threads = cpu_threads()
    if args.workload == "batch64":
        scene = S.spheres_scene()
        views = S.batch_views(64)
        cfg = {"workload": "spheres200_64_viewports_batch", "triangles": scene.n_triangles, "views": 64}
        metric = "frames/s (64 viewports of uneven size in one graph-captured launch sequence)"
        oracle.render_parallel(scene, views[:threads], threads)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            oracle.render_parallel(scene, views, threads)
            times.append(time.perf_counter() - t0)
        n_per_step = len(views)
    elif args.workload == "frame":
        scene = S.spheres_scene()
        views = [S.spheres_view(1920, 1080)] * threads
        cfg = {"workload": "spheres200_1080p_frame", "triangles": scene.n_triangles, "viewport": "1920x1080"}
        metric = "frames/s (plain renderer, one 1080p frame per launch sequence)"
        oracle.render_parallel(scene, views, threads)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            oracle.render_parallel(scene, views, threads)
            times.append(time.perf_counter() - t0)
        n_per_step = len(views)
    else:
        scenes = S.serving_scenes()
        per_step = args.cpu_requests_per_step
        reqs = S.serving_requests((args.steps + 1) * per_step, seed=60)
        cfg = serve_config(args)
        metric = METRIC

        def step(chunk):
            by_scene = {}
            for (_, k, v) in chunk:
                by_scene.setdefault(k, []).append(v)
            for k, views in by_scene.items():
                oracle.render_parallel(scenes[k], views, threads)

        step(reqs[:per_step])
        times = []
        for s in range(args.steps):
            t0 = time.perf_counter()
            step(reqs[(s + 1) * per_step:(s + 2) * per_step])
            times.append(time.perf_counter() - t0)
        n_per_step = per_step
    fps = n_per_step * len(times) / sum(times)
    return {
        "impl": "reference", "metric": metric, "value": round(fps, 3), "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sum(times) / len(times), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded scenes and request stream, swegl_gb300/scenes.py)", "config": cfg,
        "cpu_baseline": {"value": round(fps, 3), "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": f"{n_per_step} requests per step on {threads} threads"},
        "e2e": {"value": round(fps, 3), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["serve", "frame", "dof", "layers", "batch64"], default="serve")
    ap.add_argument("--requests-per-step", type=int, default=4096)
    ap.add_argument("--seq-requests", type=int, default=512)
    ap.add_argument("--profile-requests", type=int, default=512, help="serving: requests of the per-kernel profile")
    ap.add_argument("--duration", type=float, default=60.0, help="open-loop latency run, seconds")
    ap.add_argument("--ring-bytes", type=int, default=4 << 30, help="latency run: pinned host frames in flight")
    ap.add_argument("--e2e-chunk", type=int, default=256, help="e2e: requests submitted together")
    ap.add_argument("--e2e-seconds", type=float, default=2.0, help="e2e: at least this long")
    ap.add_argument("--budget", type=int, default=40 << 30)
    ap.add_argument("--max-batch", type=int, default=64)
    ap.add_argument("--streams", type=int, default=3)
    ap.add_argument("--cpu-frames", type=int, default=4096, help="CPU baseline: at most this many frames")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline: about this much host work")
    ap.add_argument("--cpu-requests", type=int, default=48)
    ap.add_argument("--cpu-requests-per-step", type=int, default=32)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local_rank = env_rank()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload in FRAMES:
        out = run_frame(args, rank, world, local_rank)
    elif args.workload == "layers":
        out = run_layers(args, rank, world, local_rank)
    elif args.workload == "batch64":
        out = run_batch64(args, rank, world, local_rank)
    else:
        out = run_serve(args, rank, world, local_rank)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
