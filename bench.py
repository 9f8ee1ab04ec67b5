#!/usr/bin/env python3
"""Benchmark of the GB300 wavefront path tracer on the triangle-heavy traversal scene.

Workload (the configuration the headline metric is quoted on): displaced icosphere of
~100k triangles (rough gold conductor, GGX alpha 0.2) over a checkerboard ground quad,
2048x1024 HDR environment map with a sun lobe, 1024x1024 pixels, max depth 25, seeded
synthetic data. One step = `--spp-per-step` samples of every pixel (128 by default, 134M
paths), rendered as four passes of 32 samples on four engines that take turns, so that
one pass's last bounces overlap the next passes; a full 1024-spp render is 8 such steps.

* value: rays traced (closest-hit queries, counted as the reference counts them) per
  second of device time, inputs resident in HBM, L2 flushed between timed steps.
* e2e: the same metric through the reference-facing C-ABI with host buffers, over as
  many steps as the device leg, L2 flushed before each: every step
  re-uploads the scene geometry (what the reference's SceneRef does on every render;
  the library keeps a page-locked copy of it) and reads the mean image and the
  tonemapped RGB8 image back into pinned host arrays.
* roofline: the trace kernel's algorithmic bytes (node fetches x node size + triangle
  tests x triangle record size + ray in / hit out, counted by an instrumented pass)
  over its measured time, against the L2 read bandwidth measured in the same run (the
  scene's traversal data is L2-resident); the fraction of the measured HBM copy
  bandwidth is kept beside it.
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
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--bvh", default="wide4", choices=["wide4", "binary", "wide", "wide-persistent"])
    ap.add_argument("--spp-per-step", type=int, default=128)
    ap.add_argument("--trace-variant", type=int, default=0,
                    help="binary traversal: 0 64 registers + fused box tests + dynamic ray fetch + while-while "
                         "(default), 1 compiler register choice, 2 variant 1 held to 64 registers, 3 variant 0 with "
                         "leaves tested where met")
    ap.add_argument("--estimator", default="reference", choices=["reference", "nee"],
                    help="reference: BSDF sampling only (the reference's estimator); nee: next-event estimation "
                         "with MIS (shadow rays count as rays)")
    ap.add_argument("--shade-variant", type=int, default=0,
                    help="shade kernel: 0 measured best register bound (default), 1 compiler's choice, "
                         "2 / 3 / 4 at most 80 / 72 / 64 registers")
    ap.add_argument("--queue-slots", type=int, default=0,
                    help="path regeneration: rays in flight per engine (0: every path of a pass starts at once)")
    ap.add_argument("--regen-threshold", type=float, default=1.0,
                    help="path regeneration: refill when the next queue holds at most this share of the slots")
    ap.add_argument("--intersector", default="mt", choices=["mt", "watertight"],
                    help="triangle test of the traversal and Cornell workloads, their CPU baseline, reference "
                         "arm and oracle check: mt = the reference's Moller-Trumbore test "
                         "(src/primitives/mesh.cu:445-476; the default, as the reference measures its rays), "
                         "watertight = the library's default test")
    ap.add_argument("--bvh-builder", default="host", choices=["host", "device"],
                    help="traversal workload: BVHs built by binned SAH on the host cores (default) or by "
                         "locally-ordered clustering on the GPU")
    ap.add_argument("--engines", type=int, default=0,
                    help="engines taking turns on a step's passes (0: the library's choice)")
    ap.add_argument("--tris", type=int, default=100_000)
    ap.add_argument("--scene", default="traversal", choices=["traversal", "sss", "instanced"],
                    help="traversal workload's scene: the headline 100k-triangle scene (default), the "
                         "700k-triangle subsurface scene, or the 2M-triangle instanced scene (BVH layout "
                         "comparisons where the BVH outgrows the caches)")
    ap.add_argument("--res", type=int, default=1024)
    ap.add_argument("--depth", type=int, default=25)
    ap.add_argument("--sss-res", type=int, nargs=2, default=[96, 72],
                    help="sss: image size (the accumulation study needs the per-pixel spp, not the pixels)")
    ap.add_argument("--sss-spp", type=int, default=20000)
    ap.add_argument("--workload", default="traversal", choices=["traversal", "batched", "served", "sss", "cornell"],
                    help="traversal: the headline single-render workload; batched: 64 uneven jobs in one job "
                         "table vs one job at a time; served: Poisson request stream, continuous batching vs "
                         "one request at a time; sss: accumulation precision study; cornell: the small "
                         "Cornell-box case with the oracle beside it")
    ap.add_argument("--jobs", type=int, default=64)
    ap.add_argument("--requests", type=int, default=48)
    ap.add_argument("--plain-1spp", action="store_true",
                    help="batched: also time one job at a time with one sample per pass")
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--lanes", type=int, default=0,
                    help="served: job tables per kernel setting (0: the library's default)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def isect_of(args):
    from illume_gb300 import _capi as C
    return C.ISECT_MT if args.intersector == "mt" else C.ISECT_WATERTIGHT


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
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
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
    if args.scene == "sss":
        return synth.sss_scene(700_000, seed=3, width=args.res, height=args.res)
    if args.scene == "instanced":
        sd = synth.instanced_scene(16, 125_000, seed=5)
        sd.width = sd.height = args.res
        return sd
    return synth.traversal_scene(tris=args.tris, seed=1, width=args.res, height=args.res)


def workload_name(args):
    if args.scene == "sss":
        return (f"subsurface scene: 700k-tri displaced dielectric (ior 1.3) around a medium in the Cornell box, "
                f"{args.res}x{args.res}, depth {args.depth}")
    if args.scene == "instanced":
        return (f"instanced scene: 16 displaced 125k-tri meshes (2M tris), mixed materials, 2048x1024 env, "
                f"{args.res}x{args.res}, depth {args.depth}")
    return WORKLOAD


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
        _, _, r = osc.render(W, H, 1, args.depth, pixels=sel, sample_begin=k, isect=isect_of(args), precision=32)
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


def reference_integrator_line(args):
    """The reference arm on the reference's own integrator: its src/ built for the host
    (OpenMP) from the staged copy of the sources (oracle/build_ref.py), timed on the
    traversal workload's full frame at 1 spp per step. Returns (line, None), or (None,
    why) where that cannot run here (then the CPU restatement stands in)."""
    if args.scene != "traversal" or args.workload != "traversal":
        return None, "the reference's own integrator is timed on the traversal workload only"
    from oracle import build_ref
    if not (build_ref.available() or build_ref.staged_available()):
        return None, "no copy of the reference sources here (oracle/build_ref.py stage)"
    try:
        from illume_gb300 import synth
        from oracle import pyref
        from oracle.time_ref_vs_port import write_scene
        t0 = time.perf_counter()
        pyref.lib(staged=True)
        build_s = time.perf_counter() - t0
        # the reference keeps a BVH file beside each OBJ and reuses it by name: one folder
        # per mesh size
        work = os.path.join(build_ref.WORK_DIR, f"bench_{args.tris}")
        os.makedirs(work, exist_ok=True)
        name = write_scene(work, args.tris)
        t0 = time.perf_counter()
        rs = pyref.RefScene(name, work, staged=True)
        rs.set_env(synth.environment_map(1, 2048, 1024))
        load_s = time.perf_counter() - t0
    except Exception as e:  # a build or load failure: the restatement stands in
        return None, f"the reference's integrator could not be built or loaded here: {e!r}"[:300]
    W = H = args.res
    threads = os.cpu_count() or 1

    def step(k):
        return rs.render(W, H, 1, args.depth, sample_begin=k, nthreads=threads)[2]

    for k in range(args.warmup):
        step(k)
    rays = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        rays += step(args.warmup + k)
    dt = time.perf_counter() - t0
    rs.close()
    v = rays / dt / 1e6
    sample = (f"the {W}x{H} frame at 1 spp per step (depth {args.depth}; {rays} rays over {args.steps} steps), "
              f"the reference's own integrator (its src/ built for the host with OpenMP, {threads} threads)")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "mode": "the reference's own integrator on host cores",
                   "material": "the reference's rough conductor 'Au' (Beckmann, alpha 0.2) for the GGX gold: "
                               "the reference has no GGX",
                   "pixels_per_step": W * H, "spp_per_step": 1, "l2": "n/a (CPU)",
                   "reference_build_s": round(build_s, 1), "reference_scene_load_s": round(load_s, 1)},
        "cpu_baseline": {"value": round(v, 4), "unit": "Mrays/s", "cores": threads, "kind": "reference",
                         "sample": sample},
        "e2e": {"value": round(v, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line, None


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    line, why = reference_integrator_line(args)
    if line is not None:
        print(json.dumps(line), flush=True)
        return
    from illume_gb300 import synth  # noqa: F401
    from oracle import pyoracle
    import numpy as np
    sd = build_scene(args)
    osc = pyoracle.OracleScene(sd)
    W = H = args.res
    pixels = np.arange(0, W * H, 97, dtype=np.int32)   # 10,810 paths per step
    def step(k):
        return osc.render(W, H, 1, args.depth, pixels=pixels, sample_begin=k, isect=isect_of(args), precision=32)[2]
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
        "config": {"workload": WORKLOAD, "mode": "CPU restatement of the reference integrator on host cores",
                   "pixels_per_step": int(len(pixels)), "spp_per_step": 1, "l2": "n/a (CPU)",
                   "reference_integrator": why},
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
    ctx.set_bvh_builder(C.BVH_BUILD_DEVICE if args.bvh_builder == "device" else C.BVH_BUILD_HOST)
    scene = HostScene.from_data(ctx, sd)
    p = scene.default_params(args.spp_per_step, args.depth)
    p.width = p.height = args.res
    p.samples_per_pass = args.spp_per_step
    p.bvh_kind = {"binary": C.BVH_BINARY, "wide": C.BVH_WIDE8, "wide-persistent": C.BVH_WIDE8_PERSISTENT,
                  "wide4": C.BVH_WIDE4}[args.bvh]
    p.intersector = isect_of(args)
    p.accum_mode = C.ACCUM_FP32
    p.sample_begin = rank * 1_000_000
    p.estimator = C.ESTIMATOR_NEE if args.estimator == "nee" else C.ESTIMATOR_REFERENCE
    p.trace_variant = args.trace_variant
    p.shade_variant = args.shade_variant
    p.engines = args.engines
    p.queue_slots = args.queue_slots
    p.regen_threshold = args.regen_threshold
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

    # image quality of what was timed: every warm-up and timed step accumulated into one
    # image; the FP64 oracle renders the same samples (same Philox streams) of a pixel
    # subset, so the difference is the FP32 arithmetic of the GPU path
    acc_spp = (args.warmup + args.steps) * args.spp_per_step
    quality = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import pyoracle
        g = r.read(mean=False, sums=True)
        npix_q = args.res * args.res
        subset = np.arange(npix_q // 97, npix_q, npix_q // 48, dtype=np.int32)[:48]
        t0q = time.perf_counter()
        osum, _, _ = pyoracle.OracleScene(sd).render(args.res, args.res, acc_spp, args.depth, seed=p.seed, job=p.job,
                                                      isect=isect_of(args), precision=64, pixels=subset,
                                                      sample_begin=p.sample_begin)
        om = osum / acc_spp
        gm = g["sum"][subset] / acc_spp
        quality = {"pixels": int(len(subset)), "spp": int(acc_spp),
                   "rmse_vs_fp64_oracle": float(np.sqrt(np.mean((gm - om) ** 2))),
                   "rel_rmse_vs_fp64_oracle": float(np.sqrt(np.mean((gm - om) ** 2)) / max(float(np.mean(np.abs(om))), 1e-12)),
                   "max_rel_err": float(np.max(np.abs(gm - om) / np.maximum(np.abs(om), 1e-6))),
                   "oracle_s": round(time.perf_counter() - t0q, 1)}
    # the renderer splits a step over its engines (by default two when each half-pass
    # keeps >= 2M paths)
    npix_all = args.res * args.res
    step_paths = args.spp_per_step * npix_all
    n_eng = args.engines if args.engines > 0 else (max(2, min(4, step_paths >> 24)) if args.spp_per_step >= 2 and
                                                   step_paths >= (1 << 22) else 1)
    n_eng = max(1, min(n_eng, args.spp_per_step))
    pass_spp = (args.spp_per_step + n_eng - 1) // n_eng
    # roofline of the trace kernel: counts from an instrumented pass, time from a plain pass
    # (one pass of one engine, kernels launched one by one)
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
    l2_peak = ctypes.c_double(0.0)
    C.check(C.lib().illume_measure_l2_read(ctx.handle, 32 << 20, 200, ctypes.byref(l2_peak)))
    l2_peak = l2_peak.value
    algo_per_launch = round(trace_bytes / max(prof_t.trace_launches, 1))

    # end to end through the C-ABI with host buffers
    npix = args.res * args.res
    # the step's results land in pinned host memory (page-locked, DMA-able)
    mean = torch.zeros((npix, 3), dtype=torch.float32, pin_memory=True).numpy()
    rgb8 = torch.zeros((npix, 3), dtype=torch.uint8, pin_memory=True).numpy()
    # every step as in the device leg: the L2 flushed before it (outside the step's time),
    # then upload, render and read back, timed on the host clock
    e2e_steps = args.steps
    up_bytes = ctypes.c_size_t()
    st = C.RenderStats()
    barrier()
    e2e_s = 0.0
    e2e_rays = 0
    t_up = t_dev = 0.0
    for k in range(e2e_steps):
        flush.fill_((k + 1) & 0xFF)
        torch.cuda.synchronize()
        ta = time.perf_counter()
        C.check(C.lib().illume_scene_upload(scene.handle, ctypes.byref(up_bytes)))
        t_up += time.perf_counter() - ta
        C.check(C.lib().illume_render(r.handle, C.fptr(mean), None, None, C.u8ptr(rgb8), ctypes.byref(st)))
        e2e_s += time.perf_counter() - ta
        t_dev += st.render_ms * 1e-3
        e2e_rays += st.rays
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
            "config": {"workload": workload_name(args), "mode": "plain wavefront" + (", passes of %d samples on %d engines taking "
                       "turns" % (pass_spp, n_eng) if n_eng > 1 else "") + (
                           ", paths regenerated into %d queue slots per engine (threshold %.2f)" %
                           (args.queue_slots, args.regen_threshold) if args.queue_slots > 0 else ""),
                       "bvh": args.bvh, "intersector": args.intersector,
                       "bvh_builder": args.bvh_builder, "bvh_build_ms": round(scene.build_info()["build_ms"], 1),
                       "estimator": args.estimator, "trace_variant": args.trace_variant,
                       "spp_per_step": args.spp_per_step, "paths_per_step": npix * args.spp_per_step,
                       "triangles": sd.num_triangles(), "resolution": [args.res, args.res], "max_depth": args.depth,
                       "l2": "flushed between timed steps (256 MB write)", "parallelism": f"replicas x{world}",
                       "wall_s": round(wall, 3), "rays_per_step": rays_all // args.steps},
            # the scene's node and triangle bytes (~10 MB) fit in L2, so the traversal roofline
            # is the L2 read bandwidth, measured in this run (MEASURED_PEAKS.json has no L2
            # figure); the HBM copy bandwidth is kept beside it
            "roofline": {"bound": "l2", "achieved": round(achieved_gbs, 1), "peak": round(l2_peak, 1), "unit": "GB/s",
                         "frac": round(achieved_gbs / l2_peak, 4) if l2_peak else None, "traffic": None,
                         "peak_source": "measured in this run: L2 read bandwidth of a 32 MB buffer swept 200 times "
                                        "with 16-byte loads that bypass L1 (illume_measure_l2_read)",
                         "traffic_note": "DRAM bytes per trace launch come from ncu only (profiles/); not measured "
                                         "in this run",
                         "hbm_gbs": peak, "frac_of_hbm": round(achieved_gbs / peak, 4),
                         "hbm_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback",
                         "kernel": "k_trace", "bytes_per_ray": round(bytes_per_ray, 1),
                         "algorithmic_bytes_per_launch": algo_per_launch,
                         "node_fetches_per_ray": round(prof_c.node_fetches / max(prof_c.rays, 1), 2),
                         "tri_tests_per_ray": round(prof_c.tri_tests / max(prof_c.rays, 1), 2),
                         "node_fetch_lane_utilisation": round(prof_c.node_fetches / max(prof_c.lane_slots, 1), 3),
                         "profiled_pass_spp": pass_spp,
                         "trace_ms_per_pass": round(prof_t.trace_ms, 3), "shade_ms_per_pass": round(prof_t.shade_ms, 3),
                         "accumulate_ms_per_pass": round(prof_t.accumulate_ms, 3),
                         "raygen_ms_per_pass": round(prof_t.raygen_ms, 3)},
            "cpu_baseline": cpu,
            "quality": quality,
            "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s",
                    "h2d_bytes_per_step": int(up_bytes.value) + 16, "d2h_bytes_per_step": npix * (12 + 3) + 8,
                    "ms_per_step": round(e2e_s / e2e_steps * 1e3, 3),
                    "upload_ms_per_step": round(t_up / e2e_steps * 1e3, 3),
                    "device_render_ms_per_step": round(t_dev / e2e_steps * 1e3, 3)},
            "gpu_launches": int(launches),
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    r.close()
    scene.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def _job_params(scene, d, C, camera=None):
    p = scene.default_params(d["spp"], d["max_depth"])
    p.width, p.height = d["width"], d["height"]
    p.seed, p.job = d.get("seed", 0), d["job"]
    p.intersector = C.ISECT_WATERTIGHT
    p.bvh_kind = C.BVH_WIDE4
    p.accum_mode = C.ACCUM_FP32
    if camera is not None:
        p.camera = C.fptr(camera)
    return p


def _upload_all(ctx, datas):
    from illume_gb300.api import HostScene
    return [HostScene.from_data(ctx, sd) for sd in datas]


def run_batched(args):
    """64 uneven jobs: one job at a time through the plain renderer versus all jobs in one
    job table (illume_render_batch: continuous admission, slots shared between jobs,
    autotuned slot count and trace kernel). Scenes are resident before timing; each arm's
    images are compared bit for bit."""
    import torch
    import numpy as np
    from illume_gb300 import _capi as C
    from illume_gb300 import synth
    from illume_gb300.api import Context, Renderer, render_batch
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    t_gen = time.perf_counter()
    pool = synth.MeshPool(seed=2)
    jobs = synth.batch_jobs(args.jobs, seed=2, pool=pool)
    ctx = Context(local)
    scenes = _upload_all(ctx, [sd for sd, _ in jobs])
    params = [_job_params(sc, d, C) for sc, (_, d) in zip(scenes, jobs)]
    gen_s = time.perf_counter() - t_gen
    paths = sum(p.width * p.height * p.spp for p in params)
    tris = [sd.num_triangles() for sd, _ in jobs]

    def plain(spp_per_pass):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rays, dev_ms, launches, means = 0, 0.0, 0, []
        for sc, p in zip(scenes, params):
            q = C.RenderParams.from_buffer_copy(p)
            q.samples_per_pass = spp_per_pass
            r = Renderer(ctx, sc, params=q)
            st = r.render_device()
            means.append(r.read(mean=True)["mean"])
            r.close()
            rays += st.rays
            dev_ms += st.render_ms
            launches += st.kernel_launches
        wall = time.perf_counter() - t0
        return dict(rays=rays, device_ms=dev_ms, wall_s=wall, launches=launches, means=means)

    # warm-up: one small job through each path
    small = int(np.argmin([p.width * p.height * p.spp for p in params]))
    render_batch(ctx, [scenes[small]], [params[small]])
    clocks = Clocks(local)
    clocks.start()
    t0 = time.perf_counter()
    means_b, _, jstats, bs = render_batch(ctx, scenes, params, autotune=bool(args.autotune))
    torch.cuda.synchronize()
    wall_b = time.perf_counter() - t0
    clk = clocks.stop()
    rays_b = sum(j.rays for j in jstats)
    pl = plain(0)
    pl1 = plain(1) if args.plain_1spp else None
    same = all(np.array_equal(a, b, equal_nan=True) for a, b in zip(means_b, pl["means"]))
    if pl1 is not None:
        same = same and all(np.array_equal(a, b, equal_nan=True) for a, b in zip(means_b, pl1["means"]))
    nan_pixels = int(sum(np.isnan(m).any(1).sum() for m in means_b))
    batched_dev = rays_b / (bs.device_ms * 1e-3) / 1e6
    batched_wall = rays_b / wall_b / 1e6
    plain_dev = pl["rays"] / (pl["device_ms"] * 1e-3) / 1e6
    plain_wall = pl["rays"] / pl["wall_s"] / 1e6
    line = {
        "metric": METRIC, "value": round(batched_dev, 3), "unit": "Mrays/s", "n_gpus": 1, "steps": int(bs.passes),
        "warmup": 1, "ms_per_step": round(bs.device_ms / max(bs.passes, 1), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched uneven jobs: {args.jobs} jobs, resolution U{{128,256,512,1024}}^2, spp "
                               "U[64,1024], 1-8 displaced icospheres (5k-700k tris, 16-mesh pool) with random "
                               "affine transforms, mixed materials, 2048x1024 env, depth 15",
                   "mode": "one job table (continuous admission, shared path slots) vs one job at a time",
                   "paths": int(paths), "triangles_per_job_min_max": [min(tris), max(tris)],
                   "scene_gen_upload_s": round(gen_s, 1), "autotune": bool(args.autotune),
                   "chosen_path_slots": int(bs.path_capacity), "chosen_trace_variant": int(bs.trace_variant),
                   "l2": "inputs larger than L2 (scenes ~GBs)"},
        "batched": {"mrays_device": round(batched_dev, 2), "mrays_wall": round(batched_wall, 2), "rays": int(rays_b),
                    "device_s": round(bs.device_ms * 1e-3, 3), "wall_s": round(wall_b, 3), "passes": int(bs.passes)},
        "plain": {"mrays_device": round(plain_dev, 2), "mrays_wall": round(plain_wall, 2), "rays": int(pl["rays"]),
                  "device_s": round(pl["device_ms"] * 1e-3, 3), "wall_s": round(pl["wall_s"], 3),
                  "samples_per_pass": "auto (min(spp, 128M / pixels))"},
        "speedup_device": round(batched_dev / plain_dev, 3), "speedup_wall": round(batched_wall / plain_wall, 3),
        "images_identical_across_arms": bool(same), "nan_pixels": nan_pixels,
        "e2e": {"value": round(batched_wall, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(sum(p.width * p.height * 12 for p in params) / max(bs.passes, 1))},
        "gpu_launches": int(bs.kernel_launches),
        "clocks": clk,
    }
    if pl1 is not None:
        d1 = pl1["rays"] / (pl1["device_ms"] * 1e-3) / 1e6
        line["plain_1spp"] = {"mrays_device": round(d1, 2), "mrays_wall": round(pl1["rays"] / pl1["wall_s"] / 1e6, 2),
                              "device_s": round(pl1["device_ms"] * 1e-3, 3), "wall_s": round(pl1["wall_s"], 3)}
        line["speedup_vs_1spp_device"] = round(batched_dev / d1, 3)
    print(json.dumps(line), flush=True)


def run_served(args):
    """Poisson request stream over three resident scenes (the traversal scene, the
    subsurface scene, 16 instanced 125k-triangle meshes); each request has its own
    resolution, spp, depth and orbit camera. Served: continuous batching in one job table
    under a 150 GB budget, requests admitted as they arrive. Plain: one request at a time
    in arrival order. Latency = finish - arrival (wall)."""
    import torch
    import numpy as np
    from illume_gb300 import _capi as C
    from illume_gb300 import synth
    from illume_gb300.api import Context, Renderer, Server
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    t_gen = time.perf_counter()
    env = synth.environment_map(1)
    datas = [synth.traversal_scene(100_000, seed=1), synth.sss_scene(700_000, seed=3),
             synth.instanced_scene(16, 125_000, seed=5, env=env)]
    ctx = Context(local)
    scenes = _upload_all(ctx, datas)
    reqs = synth.request_stream(args.requests, len(scenes), seed=4)
    cams = [synth.orbit_camera(datas[r["scene"]], np.random.default_rng(r["pose_seed"])) for r in reqs]
    params = [_job_params(scenes[r["scene"]], r, C, cam) for r, cam in zip(reqs, cams)]
    gen_s = time.perf_counter() - t_gen
    paths = sum(p.width * p.height * p.spp for p in params)

    def pct(xs, q):
        return float(np.percentile(np.asarray(xs), q))

    # served arm
    opts = {"lanes": args.lanes} if args.lanes > 0 else {}
    srv = Server(ctx, hbm_budget_bytes=150 << 30, max_jobs_in_flight=64, autotune=int(args.autotune), **opts)
    warm = srv.submit(scenes[0], _job_params(scenes[0], dict(width=64, height=64, spp=4, max_depth=4, job=999), C))
    srv.run()
    srv.poll(warm)
    s0 = srv.stats()
    clocks = Clocks(local)
    clocks.start()
    t0 = time.perf_counter()
    nxt, ids, finish, means_s = 0, {}, {}, {}
    while nxt < len(reqs) or len(finish) < len(reqs):
        now = time.perf_counter() - t0
        while nxt < len(reqs) and reqs[nxt]["arrival"] <= now:
            ids[srv.submit(scenes[reqs[nxt]["scene"]], params[nxt])] = nxt
            nxt += 1
        if len(ids) == len(finish):
            time.sleep(max(0.0, min(0.002, reqs[nxt]["arrival"] - now)))
            continue
        srv.step()
        t = time.perf_counter() - t0
        for jid, k in ids.items():
            if k in finish:
                continue
            out = srv.poll(jid)
            if out is not None:
                finish[k] = t
                means_s[k] = out["mean"]
    wall_s = max(finish.values()) - reqs[0]["arrival"]
    clk = clocks.stop()
    s1 = srv.stats()
    rays_s = s1.rays - s0.rays
    lat_s = [finish[k] - reqs[k]["arrival"] for k in range(len(reqs))]
    srv.close()

    # plain arm: one request at a time, in arrival order
    t0 = time.perf_counter()
    finish_p, rays_p, dev_p, same = {}, 0, 0.0, True
    for k, (r, p) in enumerate(zip(reqs, params)):
        now = time.perf_counter() - t0
        if r["arrival"] > now:
            time.sleep(r["arrival"] - now)
        rr = Renderer(ctx, scenes[r["scene"]], params=p)
        st = rr.render_device()
        m = rr.read(mean=True)["mean"]
        rr.close()
        finish_p[k] = time.perf_counter() - t0
        rays_p += st.rays
        dev_p += st.render_ms
        same = same and np.array_equal(m, means_s[k], equal_nan=True)
    wall_p = max(finish_p.values()) - reqs[0]["arrival"]
    lat_p = [finish_p[k] - reqs[k]["arrival"] for k in range(len(reqs))]
    served = rays_s / wall_s / 1e6
    plain = rays_p / wall_p / 1e6
    line = {
        "metric": METRIC, "value": round(served, 3), "unit": "Mrays/s", "n_gpus": 1, "steps": int(s1.passes - s0.passes),
        "warmup": 1, "ms_per_step": round((s1.device_ms - s0.device_ms) / max(s1.passes - s0.passes, 1), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"served: {args.requests} Poisson requests (mean 40/s, seed 4) over 3 resident scenes "
                               "(traversal 100k, subsurface 700k, 16 x 125k instanced); resolution log-uniform "
                               "64^2-1920x1080, spp log-uniform 16-4096, depth U{10..25}, orbit cameras",
                   "mode": "continuous batching (150 GB budget) vs one request at a time",
                   "paths": int(paths), "scene_gen_upload_s": round(gen_s, 1),
                   "chosen_path_slots": int(s1.path_capacity), "chosen_trace_variant": int(s1.trace_variant)},
        "served": {"mrays_wall": round(served, 2), "mrays_device": round(rays_s / ((s1.device_ms - s0.device_ms) * 1e-3) / 1e6, 2),
                   "p50_latency_s": round(pct(lat_s, 50), 3), "p99_latency_s": round(pct(lat_s, 99), 3),
                   "wall_s": round(wall_s, 3), "rays": int(rays_s)},
        "plain": {"mrays_wall": round(plain, 2), "mrays_device": round(rays_p / (dev_p * 1e-3) / 1e6, 2),
                  "p50_latency_s": round(pct(lat_p, 50), 3), "p99_latency_s": round(pct(lat_p, 99), 3),
                  "wall_s": round(wall_p, 3), "rays": int(rays_p)},
        "speedup_wall": round(served / plain, 3),
        "images_identical_across_arms": bool(same),
        "e2e": {"value": round(served, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(sum(p.width * p.height * 12 for p in params) / max(s1.passes - s0.passes, 1))},
        "gpu_launches": int(s1.kernel_launches - s0.kernel_launches),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_sss(args):
    """Accumulation precision at high spp: the subsurface scene (700k-triangle dielectric
    boundary around a scattering medium in the Cornell box, depth 50) rendered with the
    FP32, compensated-FP32 and FP64 per-pixel accumulators, both Henyey-Greenstein
    samplers. Reported per mode: Mrays/s, the accumulation error against the FP64 sum of
    the same samples (every pixel), and the RMSE against the FP64 host oracle (same
    Philox streams) on a pixel subset."""
    import torch
    import numpy as np
    from illume_gb300 import _capi as C
    from illume_gb300 import synth
    from illume_gb300.api import Context, HostScene, Renderer
    from oracle import pyoracle
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    W, H = args.sss_res
    spp, depth = args.sss_spp, 50
    sd = synth.sss_scene(700_000, seed=3, width=W, height=H)
    ctx = Context(local)
    scene = HostScene.from_data(ctx, sd)
    # 24 pixels spread over the central part of the frame, where the box is (a stride that
    # is a multiple of the width would keep to one column, at 960 wide the left edge)
    subset = np.array([int(H * (0.1 + 0.8 * (k + 0.5) / 24)) * W + int(W * (0.2 + 0.6 * ((7 * k % 24) + 0.5) / 24))
                       for k in range(24)], dtype=np.int32)
    out = {"metric": METRIC, "unit": "Mrays/s", "n_gpus": 1, "steps": 1, "warmup": 0, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"subsurface accumulation: 700k-tri dielectric (ior 1.3) around a medium "
                                  f"(sigma_a 0.01/0.08/0.3, sigma_s 1, g 0.7) in the Cornell box, {W}x{H}, depth "
                                  f"{depth}, {spp} spp per pixel", "oracle_pixels": int(len(subset))},
           "modes": {}}
    mrays0 = None
    for hg in (0, 1):
        sums = {}
        for mode, name in ((C.ACCUM_FP64, "fp64"), (C.ACCUM_KAHAN, "kahan"), (C.ACCUM_FP32, "fp32")):
            p = scene.default_params(spp, depth)
            p.width, p.height, p.seed, p.job, p.exact_hg, p.accum_mode = W, H, 7, 0, hg, mode
            r = Renderer(ctx, scene, params=p)
            st = r.render_device()
            sums[name] = r.read(mean=False, sums=True)["sum"]
            r.close()
            mr = st.rays / (st.render_ms * 1e-3) / 1e6
            if mrays0 is None and name == "fp32":
                mrays0 = (mr, st.render_ms)
            out["modes"][f"{name}_hg{hg}"] = {"mrays": round(mr, 2), "render_s": round(st.render_ms * 1e-3, 3),
                                               "rays": int(st.rays)}
        t0 = time.perf_counter()
        osum, _, orays = pyoracle.OracleScene(sd).render(W, H, spp, depth, seed=7, job=0, isect=C.ISECT_WATERTIGHT,
                                                        exact_hg=hg, precision=64, pixels=subset)
        oracle_s = time.perf_counter() - t0
        ref = sums["fp64"]
        scale = np.maximum(np.abs(ref), 1e-6)
        omean = osum / spp
        for name in ("fp64", "kahan", "fp32"):
            m = out["modes"][f"{name}_hg{hg}"]
            rel = np.abs(sums[name] - ref) / scale
            m["accum_rel_err_max"] = float(rel.max())
            m["accum_rel_err_mean"] = float(rel.mean())
            gm = sums[name][subset] / spp
            m["rmse_vs_fp64_oracle"] = float(np.sqrt(np.mean((gm - omean) ** 2)))
            m["rel_rmse_vs_fp64_oracle"] = float(np.sqrt(np.mean((gm - omean) ** 2)) / max(np.mean(np.abs(omean)), 1e-12))
        out["config"][f"oracle_s_hg{hg}"] = round(oracle_s, 1)
        out["config"][f"oracle_rays_hg{hg}"] = int(orays)
    out["value"] = round(mrays0[0], 3)
    out["ms_per_step"] = round(mrays0[1], 3)
    print(json.dumps(out), flush=True)


def run_cornell(args):
    """The small plain-method case: the Cornell box (mirror and glass spheres, 256x256,
    64 spp, depth 8, FP32 accumulation, seed 0). One step = one full render on the GPU.
    Beside it, the same render by the oracle (the reference integrator restated) on all
    host cores in FP32 (timed) and in FP64 (the image the GPU's is compared with: same
    Philox streams, so the difference is arithmetic, not Monte Carlo noise)."""
    import torch
    import numpy as np
    from illume_gb300 import _capi as C
    from illume_gb300 import synth
    from illume_gb300.api import Context, HostScene, Renderer
    from oracle import pyoracle
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    W = H = 256
    spp, depth = 64, 8
    sd = synth.cornell_scene(W, H)
    ctx = Context(local)
    scene = HostScene.from_data(ctx, sd)
    p = scene.default_params(spp, depth)
    p.width, p.height, p.seed, p.job, p.accum_mode = W, H, 0, 0, C.ACCUM_FP32
    p.estimator = C.ESTIMATOR_NEE if args.estimator == "nee" else C.ESTIMATOR_REFERENCE
    p.intersector = isect_of(args)
    r = Renderer(ctx, scene, params=p)
    for _ in range(args.warmup):
        r.render_device()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    dev_ms, rays, launches = 0.0, 0, 0
    for _ in range(args.steps):
        st = r.render_device()
        dev_ms += st.render_ms
        rays += st.rays
        launches += st.kernel_launches
    torch.cuda.synchronize()
    clk = clocks.stop()
    g = r.read(mean=False, sums=True)
    r.close()
    gmean = g["sum"] / spp
    gvar = np.maximum(g["sumsq"] / spp - gmean * gmean, 0)
    value = rays / (dev_ms * 1e-3) / 1e6
    osc = pyoracle.OracleScene(sd)
    t0 = time.perf_counter()
    o32, _, crays = osc.render(W, H, spp, depth, seed=0, job=0, isect=isect_of(args), precision=32)
    cpu_s = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    osum, osq, _ = osc.render(W, H, spp, depth, seed=0, job=0, isect=isect_of(args), precision=64)
    om = osum / spp
    ovar = np.maximum(osq / spp - om * om, 0)
    rmse = float(np.sqrt(np.mean((gmean - om) ** 2)))
    rmse32 = float(np.sqrt(np.mean((gmean - o32 / spp) ** 2)))
    sigma = np.sqrt((gvar + ovar) / spp)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dev_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"Cornell box (5 wall quads, 130x105 light (17,12,4), mirror and glass spheres r=90), "
                               f"{W}x{H}, {spp} spp, depth {depth}, FP32 accumulation, seed 0",
                   "estimator": args.estimator, "intersector": args.intersector, "rays_per_render": rays // args.steps,
                   "l2": "scene and image fit in L2 (working set < 40 MB); not flushed"},
        # the reference estimator follows the oracle's Philox streams, so these differences
        # are arithmetic (FP32 paths that part from the FP64 ones); the next-event estimator
        # draws other samples, so for it they are Monte Carlo noise
        "rmse_vs_fp64_oracle": rmse,
        "rel_rmse_vs_fp64_oracle": rmse / max(float(np.mean(np.abs(om))), 1e-12),
        "rmse_vs_fp32_oracle": rmse32,
        # per-pixel 3-sigma with sample variances of 64 samples: pixels whose reference-
        # estimator samples never reached the light have a zero variance estimate, so for the
        # next-event estimator the image mean below is the unbiasedness figure at this spp
        "within_3sigma_of_fp64_oracle": float(np.mean(np.abs(gmean - om) <= 3 * sigma + 1e-6)),
        "image_mean_rel_diff_vs_fp64_oracle": float((gmean.mean() - om.mean()) / max(abs(om.mean()), 1e-12)),
        "variance_per_sample": {"gpu": float(gvar.mean()), "fp64_oracle": float(ovar.mean())},
        "cpu_baseline": {"value": round(crays / cpu_s / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"the full {W}x{H} {spp}-spp render, FP32 oracle, {crays} rays, {cpu_s:.1f} s, "
                                   f"OpenMP {threads} threads"},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    scene.close()
    ctx.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "served":
        run_served(args)
    elif args.workload == "sss":
        run_sss(args)
    elif args.workload == "cornell":
        run_cornell(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
