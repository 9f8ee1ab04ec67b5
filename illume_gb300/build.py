"""In-tree build of the native library (illume_gb300/_lib/libillume_gb300.so) and the CLI.

CUDA sources are compiled for sm_103a only; host C++ with g++. Floating-point contraction
is disabled on both sides (-fmad=false / -ffp-contract=off) so that FP32 results do not
depend on the compiler's choice of fused multiply-adds: the kernels write their fused
multiply-adds explicitly where they want them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB = os.path.join(LIB_DIR, "libillume_gb300.so")
CLI = os.path.join(LIB_DIR, "illume")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["kernels/trace_kernels.cu", "kernels/integrator.cu", "kernels/noalloc.cu", "kernels/bvh_device.cu"]
CPP_SOURCES = ["host/json.cpp", "host/mesh_io.cpp", "host/xform.cpp", "host/bvh_build.cpp", "host/runtime.cpp",
               "host/scene_json.cpp", "host/image_io.cpp", "host/deflate_encode.cpp", "host/png_decode.cpp", "host/engine.cpp", "host/lights.cpp", "host/renderer.cpp", "host/server.cpp",
               "host/capi.cpp"]


def _headers():
    hs = [os.path.join(ROOT, "include", "illume.h")]
    for d, _, files in os.walk(CSRC):
        hs += [os.path.join(d, f) for f in files if f.endswith((".h", ".cuh"))]
    return hs


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(h) > t for h in headers)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, os.path.basename(s) + ".o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, os.path.basename(s) + ".o")
        objs.append(obj)
        if force or _stale(obj, src, headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                         "-Wno-unused-function", "-I", os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj])
    outputs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                outputs.append(out)
    if jobs or not os.path.exists(LIB):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    cli_src = os.path.join(CSRC, "cli", "illume_main.cpp")
    if jobs or not os.path.exists(CLI) or os.path.getmtime(cli_src) > os.path.getmtime(CLI):
        _run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), cli_src, "-o", CLI, "-L", LIB_DIR,
              "-lillume_gb300", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        for o in outputs:
            if o.strip():
                print(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
