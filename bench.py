#!/usr/bin/env python3
"""Benchmark of the GB300 wavefront path tracer on the triangle-heavy traversal scene.

Workload (the configuration the headline metric is quoted on): displaced icosphere of
~100k triangles (rough gold conductor, GGX alpha 0.2) over a checkerboard ground quad,
2048x1024 HDR environment map with a sun lobe, 1024x1024 pixels, max depth 25, seeded
synthetic data. One step = one wavefront pass of `--spp-per-step` samples of every pixel
(4 by default, i.e. 4M paths); a full 1024-spp render is 256 such steps.

* value: rays traced (closest-hit queries, counted as the reference counts them) per
  second of device time, inputs resident in HBM, L2 flushed between timed steps.
* e2e: the same metric through the reference-facing C-ABI with host buffers: every step
  re-uploads the scene (what the reference's SceneRef does on every render) and reads
  the mean image and the tonemapped RGB8 image back.
* roofline: the trace kernel's algorithmic bytes (node fetches x node size + triangle
  tests x triangle record size + ray in / hit out, counted by an instrumented pass)
  over its measured time, against the measured HBM copy bandwidth.
* cpu_baseline: the CPU restatement of the reference integrator (oracle/), OpenMP on all
  host cores, on a bounded pixel subset of the same scene.

`--impl reference` times the reference's integrator on the host cores (the CPU
restatement in oracle/, pinned to the reference's own code in the build container):
one step = a bounded pixel subset of the same workload.
Multi-GPU (--gpus N under torchrun): independent replicas, each rank renders its own
samples of the same frame (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s at matched RMSE vs FP64 oracle (plain vs batched/served); p99 latency"
WORKLOAD = "triangle-heavy traversal: displaced icosphere 100k tris, GGX rough gold alpha 0.2, checkerboard ground, 2048x1024 env, 1024x1024, depth 25"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--bvh", default="binary", choices=["binary", "wide", "wide-persistent"])
    ap.add_argument("--spp-per-step", type=int, default=4)
    ap.add_argument("--trace-variant", type=int, default=0,
                    help="binary traversal: 0 compiler register choice, 1 at most 64 registers")
    ap.add_argument("--tris", type=int, default=100_000)
    ap.add_argument("--res", type=int, default=1024)
    ap.add_argument("--depth", type=int, default=25)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


def build_scene(args):
    from illume_gb300 import synth
    return synth.traversal_scene(tris=args.tris, seed=1, width=args.res, height=args.res)


def cpu_baseline(sd, args, seconds):
    """The oracle (reference integrator restated) on all host cores, on a strided pixel
    subset of the workload at 1 spp; returns (Mrays/s, threads, description)."""
    from oracle import pyoracle
    import numpy as np
    osc = pyoracle.OracleScene(sd)
    W = H = args.res
    stride = 7
    pixels = np.arange(0, W * H, stride, dtype=np.int32)
    chunk = 4096
    rays = 0
    t0 = time.perf_counter()
    done = 0
    k = 0
    while True:
        sel = pixels[(k * chunk) % len(pixels):(k * chunk) % len(pixels) + chunk]
        _, _, r = osc.render(W, H, 1, args.depth, pixels=sel, sample_begin=k, isect=1, precision=32)
        rays += r
        done += len(sel)
        k += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    desc = (f"{done} paths (1 spp on every {stride}th pixel of the {W}x{H} frame, depth {args.depth}), "
            f"{rays} rays, {dt:.1f} s, OpenMP {threads} threads, FP32 oracle")
    return rays / dt / 1e6, threads, desc


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from illume_gb300 import synth  # noqa: F401
    from oracle import pyoracle
    import numpy as np
    sd = build_scene(args)
    osc = pyoracle.OracleScene(sd)
    W = H = args.res
    pixels = np.arange(0, W * H, 97, dtype=np.int32)   # 10,810 paths per step
    def step(k):
        return osc.render(W, H, 1, args.depth, pixels=pixels, sample_begin=k, isect=1, precision=32)[2]
    for k in range(args.warmup):
        step(k)
    rays = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        rays += step(args.warmup + k)
    dt = time.perf_counter() - t0
    v = rays / dt / 1e6
    threads = os.cpu_count() or 1
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "mode": "reference integrator on host cores",
                   "pixels_per_step": int(len(pixels)), "spp_per_step": 1, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": round(v, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{len(pixels)} paths per step (every 97th pixel, 1 spp, depth {args.depth}), "
                                   f"CPU restatement of the reference integrator (oracle/), OpenMP {threads} threads"},
        "e2e": {"value": round(v, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import ctypes
    import numpy as np
    import torch
    from illume_gb300 import _capi as C
    from illume_gb300.api import Context, HostScene, Renderer

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = local
    torch.cuda.set_device(dev)
    sd = build_scene(args)
    ctx = Context(dev)
    scene = HostScene.from_data(ctx, sd)
    p = scene.default_params(args.spp_per_step, args.depth)
    p.width = p.height = args.res
    p.samples_per_pass = args.spp_per_step
    p.bvh_kind = {"binary": C.BVH_BINARY, "wide": C.BVH_WIDE8, "wide-persistent": C.BVH_WIDE8_PERSISTENT}[args.bvh]
    p.intersector = C.ISECT_WATERTIGHT
    p.accum_mode = C.ACCUM_FP32
    p.sample_begin = rank * 1_000_000
    p.reserved[0] = args.trace_variant
    r = Renderer(ctx, scene, params=p)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{dev}")   # > 129 MB L2

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for k in range(args.warmup):
        r.render_device(accumulate=k > 0)
    torch.cuda.synchronize()
    clocks = Clocks(dev)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    dev_ms, rays, launches = 0.0, 0, 0
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        torch.cuda.synchronize()
        st = r.render_device(accumulate=True)
        dev_ms += st.render_ms
        rays += st.rays
        launches += st.kernel_launches
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()

    # max over ranks of device time, sum of rays
    if world > 1:
        t = torch.tensor([dev_ms, float(rays)], dtype=torch.float64, device=f"cuda:{dev}")
        tmax = t.clone()
        torch.distributed.all_reduce(tmax[0:1], op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(tmax[1:2], op=torch.distributed.ReduceOp.SUM)
        dev_ms_max, rays_all = float(tmax[0]), int(tmax[1])
    else:
        dev_ms_max, rays_all = dev_ms, rays
    value = rays_all / (dev_ms_max * 1e-3) / 1e6

    # roofline of the trace kernel: counts from an instrumented pass, time from a plain pass
    prof_t = C.Profile()
    C.check(C.lib().illume_renderer_profile(r.handle, 0, ctypes.byref(prof_t)))
    prof_c = C.Profile()
    C.check(C.lib().illume_renderer_profile(r.handle, 1, ctypes.byref(prof_c)))
    bytes_per_ray = ((prof_c.node_fetches * prof_c.node_bytes + prof_c.tri_tests * prof_c.tri_bytes) / max(prof_c.rays, 1)
                     + 32 + 24)
    trace_bytes = bytes_per_ray * prof_t.rays
    achieved_gbs = trace_bytes / (prof_t.trace_ms * 1e-3) / 1e9
    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    traffic = None
    tf = os.path.join(ROOT, "profiles", "trace_traffic.txt")
    if os.path.exists(tf):
        for line in open(tf):
            if line.startswith("dram_bytes_per_launch_full_workload:"):
                traffic = float(line.split(":")[1])

    # end to end through the C-ABI with host buffers
    npix = args.res * args.res
    mean = np.zeros((npix, 3), np.float32)
    rgb8 = np.zeros((npix, 3), np.uint8)
    e2e_steps = max(1, min(args.steps, 4))
    up_bytes = ctypes.c_size_t()
    st = C.RenderStats()
    barrier()
    t0 = time.perf_counter()
    e2e_rays = 0
    for k in range(e2e_steps):
        C.check(C.lib().illume_scene_upload(scene.handle, ctypes.byref(up_bytes)))
        C.check(C.lib().illume_render(r.handle, C.fptr(mean), None, None, C.u8ptr(rgb8), ctypes.byref(st)))
        e2e_rays += st.rays
    e2e_s = time.perf_counter() - t0
    e2e_value = e2e_rays / e2e_s / 1e6
    if world > 1:
        t = torch.tensor([e2e_s, float(e2e_rays)], dtype=torch.float64, device=f"cuda:{dev}")
        torch.distributed.all_reduce(t[0:1], op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(t[1:2], op=torch.distributed.ReduceOp.SUM)
        e2e_value = float(t[1]) / float(t[0]) / 1e6

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, desc = cpu_baseline(sd, args, args.cpu_seconds)
        cpu = {"value": round(v, 4), "unit": "Mrays/s", "cores": cores, "kind": "port", "sample": desc}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dev_ms_max / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "mode": "plain wavefront", "bvh": args.bvh, "intersector": "watertight",
                       "spp_per_step": args.spp_per_step, "paths_per_step": npix * args.spp_per_step,
                       "triangles": sd.num_triangles(), "resolution": [args.res, args.res], "max_depth": args.depth,
                       "l2": "flushed between timed steps (256 MB write)", "parallelism": f"replicas x{world}",
                       "wall_s": round(wall, 3), "rays_per_step": rays_all // args.steps},
            "roofline": {"bound": "hbm", "achieved": round(achieved_gbs, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved_gbs / peak, 4), "traffic": traffic,
                         "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback",
                         "kernel": "k_trace", "bytes_per_ray": round(bytes_per_ray, 1),
                         "node_fetches_per_ray": round(prof_c.node_fetches / max(prof_c.rays, 1), 2),
                         "tri_tests_per_ray": round(prof_c.tri_tests / max(prof_c.rays, 1), 2),
                         "trace_ms_per_pass": round(prof_t.trace_ms, 3), "shade_ms_per_pass": round(prof_t.shade_ms, 3)},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s",
                    "h2d_bytes_per_step": int(up_bytes.value) + 16, "d2h_bytes_per_step": npix * (12 + 3) + 8},
            "gpu_launches": int(launches),
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    r.close()
    scene.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
