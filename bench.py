#!/usr/bin/env python
"""Benchmark of the GB300 swegl renderer; prints ONE JSON line (rank 0).

Workloads (synthetic, seeded; see swegl_gb300/scenes.py):
  frame  200 UV spheres (819,200 triangles, 8 value-noise 1024^2 textures,
         sun + 4 point lights, shininess in [8,128]) at 1920x1080, one frame
         per step, plain one-frame-per-launch renderer.

Timing: W warm-up steps, then K timed steps, each bracketed by CUDA events on
the launching stream.  Inputs are larger than L2: four resident copies of the
scene (about 4 x 100 MB against a 129 MB L2) are rendered in rotation, so each
step reads its scene cold.  `e2e` renders the same frames through the public
C ABI with host (pinned) buffers: the frame copy back to the host is inside
its timed region.  Under torchrun (N > 1) every rank renders its own frames
(replicas, no collective); rank 0 prints the max-over-ranks timing.

--impl reference times the reference's CPU algorithm (the oracle's C
restatement, built from oracle/sgl_oracle.c) on all host threads on the same
workload.
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


# ----------------------------------------------------------------- helpers --
def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_traffic(name: str):
    """Per-launch DRAM traffic from the committed ncu summary (profiles/)."""
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
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
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


def frame_alg_bytes(scene, w: int, h: int) -> int:
    """Algorithmic bytes of one frame: 32 B per vertex (position, normal, uv),
    4 B per index, 4 B per texel of every texture, 8 B per viewport pixel
    (BGRA8 colour + FP32 depth written once)."""
    texels = sum(int(t.size) for t in scene.textures)
    return 32 * len(scene.positions) + 4 * len(scene.indices) + 4 * texels + 8 * w * h


# ---------------------------------------------------------------- workloads --
def build_frame_workload():
    from swegl_gb300 import scenes as S

    scene = S.spheres_scene()
    view = S.spheres_view(1920, 1080)
    cfg = {"workload": "spheres200_1080p_frame", "spheres": 200, "triangles": scene.n_triangles,
           "vertices": int(len(scene.positions)), "viewport": "1920x1080", "textures": "8 x 1024^2 value noise",
           "lights": "sun + 4 point", "shininess": "U[8,128]",
           "l2": "inputs larger than L2: 4 resident scene copies rendered in rotation",
           "renderer": "one frame per launch sequence"}
    return scene, [view], cfg


def run_ours(args, rank, world, local_rank):
    import torch

    from swegl_gb300 import abi
    from swegl_gb300.runtime import Renderer

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    scene, views, cfg = build_frame_workload()
    r = Renderer(local_rank)
    copies = [r.upload(scene) for _ in range(4)]
    sid = copies[0]
    v = views[0]
    stream = torch.cuda.Stream()
    pix = torch.zeros((v.h, v.w), dtype=torch.int32, device="cuda")
    zb = torch.zeros((v.h, v.w), dtype=torch.float32, device="cuda")
    tgt = abi.Target()
    tgt.pixels = pix.data_ptr()
    tgt.pitch = 4 * v.w
    tgt.width, tgt.height = v.w, v.h
    tgt.zbuffer = C.cast(C.c_void_p(zb.data_ptr()), C.POINTER(C.c_float))
    def step(k):
        r.render_device(copies[k % len(copies)], views, [tgt], stream=stream.cuda_stream)

    with torch.cuda.stream(stream):
        for k in range(args.warmup):
            step(k)
    torch.cuda.synchronize()
    stats = r.render_device(sid, views, [tgt], stream=stream.cuda_stream, stats=True)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    r.profile(True)
    with ClockSampler(local_rank) as clocks:
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                starts[k].record(stream)
                step(k)
                ends[k].record(stream)
        torch.cuda.synchronize()
    prof = r.profile_read()
    r.profile(False)
    if dist:
        dist.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(step_ms)
    if dist:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    frames_per_s = world * args.steps / (total_ms / 1e3)

    # e2e through the public API with pinned host buffers (copy-out inside)
    host_pix = torch.zeros((v.h, v.w), dtype=torch.int32).pin_memory()
    host_z = torch.zeros((v.h, v.w), dtype=torch.float32).pin_memory()
    htgt = abi.Target()
    htgt.pixels = host_pix.data_ptr()
    htgt.pitch = 4 * v.w
    htgt.width, htgt.height = v.w, v.h
    htgt.zbuffer = C.cast(C.c_void_p(host_z.data_ptr()), C.POINTER(C.c_float))
    vd = (abi.ViewDesc * 1)(abi.view_desc(v))
    td = (abi.Target * 1)(htgt)

    def e2e_step(k):
        st = r.lib.sgl_render(r.ctx, copies[k % len(copies)], vd, td, 1, 0, None, None)
        if st != 0:
            raise RuntimeError(f"sgl_render failed: {st}")

    for k in range(args.warmup):
        e2e_step(k)
    e2e_times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        e2e_step(k)
        e2e_times.append(time.perf_counter() - t0)
    e2e_total = sum(e2e_times)
    if dist:
        t = torch.tensor([e2e_total], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_fps = world * args.steps / e2e_total

    alg = frame_alg_bytes(scene, v.w, v.h)
    frame_ms = total_ms / args.steps
    peaks = measured_peaks()
    achieved = alg / (frame_ms / 1e3) / 1e9
    kernels = {k: {"avg_us": round(1e3 * d["total_ms"] / max(1, d["launches"]), 2), "launches": d["launches"]}
               for k, d in prof.items()}
    dom = max(prof.items(), key=lambda kv: kv[1]["total_ms"])[0] if prof else None
    out = {
        "metric": "frames/s (single 1080p frame per launch sequence)",
        "value": round(frames_per_s, 2),
        "unit": "frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(frame_ms, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32",
        "data": "synthetic (seeded scenes, see swegl_gb300/scenes.py)",
        "config": cfg,
        "gfragments_per_s": round(stats["fragments"] * frames_per_s / 1e9, 3),
        "fragments_per_frame": stats["fragments"],
        "kernels": kernels,
        "dominant_kernel": dom,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4), "peak_source": peaks["source"],
                     "unit_of_work": "one frame (alg bytes %d)" % alg,
                     "traffic": profile_traffic("frame_1080p_traffic.md")},
        "e2e": {"value": round(e2e_fps, 2), "unit": "frames/s", "h2d_bytes_per_step": C.sizeof(abi.ViewDesc),
                "d2h_bytes_per_step": 8 * v.w * v.h},
        "gpu_launches": int(stats["kernel_launches"]) * args.steps,
        "clocks": clocks.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(scene, views, args)
    if dist:
        dist.destroy_process_group()
    r.close()
    return out if rank == 0 else None


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(scene, views, args) -> dict:
    """The oracle restatement on all host threads, a bounded sample of the workload."""
    import oracle

    threads = cpu_threads()
    n = max(threads, args.cpu_frames)
    frame_views = [views[i % len(views)] for i in range(n)]
    oracle.render_parallel(scene, frame_views[:threads], threads)  # warm-up
    t0 = time.perf_counter()
    oracle.render_parallel(scene, frame_views, threads)
    dt = time.perf_counter() - t0
    return {"value": round(n / dt, 3), "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"{n} frames of the same workload on {threads} threads ({dt:.1f} s)"}


def run_reference(args, rank, world):
    """The reference's CPU algorithm (oracle restatement) timed on the host cores."""
    if rank != 0:
        return None
    scene, views, cfg = build_frame_workload()
    import oracle

    threads = cpu_threads()
    per_step = threads
    frame_views = [views[0]] * per_step
    for _ in range(max(1, min(args.warmup, 1))):
        oracle.render_parallel(scene, frame_views, threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.render_parallel(scene, frame_views, threads)
        times.append(time.perf_counter() - t0)
    fps = per_step * len(times) / sum(times)
    return {
        "impl": "reference",
        "metric": "frames/s (single 1080p frame per launch sequence)",
        "value": round(fps, 3),
        "unit": "frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(1e3 * sum(times) / len(times), 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32",
        "data": "synthetic (seeded scenes, see swegl_gb300/scenes.py)",
        "config": cfg,
        "cpu_baseline": {"value": round(fps, 3), "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": f"{per_step} frames per step on {threads} threads"},
        "e2e": {"value": round(fps, 3), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-frames", type=int, default=32)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local_rank = env_rank()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_ours(args, rank, world, local_rank)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
