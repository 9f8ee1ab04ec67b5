"""The reference's own CUDA megakernel renderer, built for sm_103a as a second baseline.

TEST INFRASTRUCTURE (a baseline that is timed, never part of the product). Four steps:

    python oracle/build_megakernel.py prepare [--jobs N]  # build container: copy, patch,
                                                          # write the scenes, check trees
    python oracle/build_megakernel.py build               # GPU machine (or here): nvcc
    python oracle/build_megakernel.py run [dir]           # GPU machine: time every scene,
                                                          # frames and logs into dir
    python oracle/build_megakernel.py check dir           # build container: frame means
                                                          # against the host build

`prepare` copies the reference's src/ and include/ from the reference checkout (read from
ILLUME_REFERENCE_ROOT, else the build container's checkout path) into
baseline/_ref/megakernel/, which git ignores and which travels with the working tree to
the GPU machine, and applies the patches the sources need with this compiler, each a
one-line change that leaves the renderer's arithmetic alone:
  * jsonutils.h names a template parameter `default` (a C++ keyword): renamed `def`;
  * math/transform.h includes "rapidjson\\document.h" with a backslash: forward slash;
  * math/vector2.h's operators take non-const references (a temporary cannot bind):
    const references, const member functions;
  * transform_from_matrix(Matrix4&) is called with a temporary: takes a const reference;
  * main.cu calls the MSVC-only _snprintf: snprintf;
  * primitives/mesh.cu:345 starts the mesh bounds from an uninitialised AABB: zero, the
    start value the host build of the same sources uses (oracle/build_ref.py);
  * renderer.cu:571 prints the rays per second: the line after it also prints the ray
    count the rate divides (its own `total_rays`), so several renders can be summed;
  * bitmap.c writes PNG through libpng, which this image lacks: replaced by a writer of
    binary PPM with the same functions (bitmap.h unchanged), written here.

It then writes the scenes in the reference's JSON vocabulary into the copy's work folder:
  cornell    config 0: tests/golden/scenes/box.json, 256x256, 64 spp, depth 8;
  traversal  the 100k-triangle displaced icosphere in the reference's rough "Au"
             conductor (Beckmann alpha 0.2: the reference knows no GGX or custom complex
             indices) over the checkerboard ground, under the synthetic 2048x1024
             environment written as a Radiance .hdr file; 1024x1024, 128 spp, depth 25;
  subsurface the Cornell box without its spheres around the 700k-triangle displaced
             icosphere (seed 3, scaled 120, centred at (277.5, 140, 277.5)), a smooth
             dielectric of ior 1.3 enclosing the medium sigma_a (0.01, 0.08, 0.3),
             sigma_s 1, g 0.7; 960x720, depth 50, 256 spp (the 20,000-spp render would
             keep the megakernel busy for most of an hour; its rate does not depend on
             the sample count past the first few);
  batch      the 64 uneven jobs of the batched workload (seed 2, the same generator the
             bench uses), each its own scene file at its own resolution and spp, depth
             15; the job materials in the reference's names: lambert, plastic,
             roughrefractive (Beckmann in place of GGX, same alpha, ior 1.5) and
             roughconductor "Cu" (the reference's copper table in place of the job's
             copper indices); instance rotations as the reference's Euler angles
             (R = Rx Ry Rz, src/math/transform.cu), checked against the job's matrix.
Each distinct mesh is loaded once with the host build of the same sources (oracle/_ref,
several meshes in parallel processes), which writes the reference's BVH cache file next
to the OBJ (src/accel/bvh.cpp:399-417); the GPU build loads those files instead of
building its own trees. The traversal of src/primitives/mesh.cu:485-527 pushes both
children of a hit inner node before it compares the stack index with its 32 entries, so
an inner node reached with 31 or more right siblings pending would write one entry past
the stack. `prepare` walks every cached tree, stops unless the deepest inner node leaves
the push inside the stack (at most 30 pending) and every child index and leaf range lies
inside the file, and records the checked files' digests; `run` renders only while the
files still match them. Every frame holds a multiple of 256 pixels, which keeps the read
of src/renderer.cu:144 (made before the kernel's bounds test) inside the status buffer.

`build` compiles the copy with nvcc (-arch sm_103a, -rdc=true, --use_fast_math, as the
reference's Visual Studio project builds it). `run` renders every job with the
reference's own executable and command line (<save> <scene.json> <spp> <maxdepth>) and
reports, per scene group, the rays per second the reference prints
(src/renderer.cu:568-572: rays traced over its whole render call, scene upload, cuRAND
set-up and host compaction included; scene parsing and the BVH load are before it),
aggregated over a group's jobs as the summed rays over the summed timed seconds.
"""
from __future__ import annotations

import hashlib
import json
import math
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_ROOT = os.environ.get("ILLUME_REFERENCE_ROOT", "/root/reference")
DEST = os.path.join(ROOT, "baseline", "_ref", "megakernel")
WORK = os.path.join(DEST, "work")
EXE = os.path.join(DEST, "illume_ref")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
BVH_STACK_SIZE = 32   # src/accel/bvh.h:9

_BITMAP_PPM = r'''/* Bitmap functions of bitmap.h; images are written as binary PPM (no libpng here). */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>

#include "bitmap.h"

Bitmap* bitmap_new(size_t width, size_t height) {
  Bitmap* b = (Bitmap*)malloc(sizeof(Bitmap));
  b->width = width;
  b->height = height;
  b->pixels = (Pixel*)calloc(width * height, sizeof(Pixel));
  return b;
}

void bitmap_free(Bitmap* b) {
  if (!b) return;
  free(b->pixels);
  free(b);
}

void bitmap_set_pixel(Bitmap* b, int x, int y, int red, int green, int blue) {
  Pixel* p = &b->pixels[(size_t)y * b->width + (size_t)x];
  p->red = (size_t)red;
  p->green = (size_t)green;
  p->blue = (size_t)blue;
}

Pixel* bitmap_get_pixel(Bitmap* b, int x, int y) { return &b->pixels[(size_t)y * b->width + (size_t)x]; }

int bitmap_save_to_png(Bitmap* b, char* path) {
  FILE* f = fopen(path, "wb");
  if (!f) return -1;
  fprintf(f, "P6\n%lu %lu\n255\n", (unsigned long)b->width, (unsigned long)b->height);
  for (size_t i = 0; i < b->width * b->height; ++i) {
    unsigned char c[3] = {(unsigned char)b->pixels[i].red, (unsigned char)b->pixels[i].green,
                          (unsigned char)b->pixels[i].blue};
    fwrite(c, 1, 3, f);
  }
  fclose(f);
  return 0;
}
'''


# ---------------------------------------------------------------- copy and patches
def _patch(path, old, new):
    with open(path) as f:
        s = f.read()
    if old not in s:
        raise RuntimeError(f"patch target not found in {path}: {old!r}")
    with open(path, "w") as f:
        f.write(s.replace(old, new))


def _copy_and_patch():
    if os.path.isdir(DEST):
        shutil.rmtree(DEST)
    os.makedirs(DEST)
    shutil.copytree(os.path.join(REF_ROOT, "src"), os.path.join(DEST, "src"))
    shutil.copytree(os.path.join(REF_ROOT, "include"), os.path.join(DEST, "include"))
    src = os.path.join(DEST, "src")
    _patch(os.path.join(src, "jsonutils.h"), "T default)", "T def)")
    _patch(os.path.join(src, "jsonutils.h"), "object = default;", "object = def;")
    _patch(os.path.join(src, "math", "transform.h"), '#include "rapidjson\\document.h"', '#include "rapidjson/document.h"')
    v2 = os.path.join(src, "math", "vector2.h")
    _patch(v2, "Vec2f operator+(Vec2f& v)", "Vec2f operator+(const Vec2f& v) const")
    _patch(v2, "Vec2f operator*(float s)", "Vec2f operator*(float s) const")
    _patch(v2, "Vec2f operator*(Vec2f& v)", "Vec2f operator*(const Vec2f& v) const")
    _patch(os.path.join(src, "math", "transform.cu"), "transform_from_matrix(Matrix4&",
           "transform_from_matrix(const Matrix4&")
    _patch(os.path.join(src, "main.cu"), "_snprintf(", "snprintf(")
    _patch(os.path.join(src, "primitives", "mesh.cu"), "    AABB bounds;\n    for (int i = 0; i < tri_amount",
           "    AABB bounds = {};\n    for (int i = 0; i < tri_amount")
    _patch(os.path.join(src, "renderer.cu"), 'printf("Rays per sec: %f rays/s\\n", rays_per_sec);',
           'printf("Rays per sec: %f rays/s\\n", rays_per_sec); printf("Rays traced: %lld\\n", total_rays);')
    with open(os.path.join(src, "bitmap.c"), "w") as f:
        f.write(_BITMAP_PPM)


# ---------------------------------------------------------------- scene files
def _write_obj(path, P, T):
    with open(path, "w") as f:
        f.write("".join("v %.9g %.9g %.9g\n" % tuple(p) for p in P))
        f.write("".join("f %d %d %d\n" % (a + 1, b + 1, c + 1) for a, b, c in T))


def _write_rgbe(path, rgb):
    """Radiance .hdr of an (h, w, 3) float image: RGBE scanlines in the run-length form,
    each channel written as literal runs of at most 128 bytes."""
    import numpy as np
    h, w, _ = rgb.shape
    m = rgb.max(axis=2)
    mant, ex = np.frexp(m)
    ok = m > 1e-32
    scale = np.where(ok, mant * 256.0 / np.where(ok, m, 1.0), 0.0)
    px = np.zeros((h, w, 4), np.uint8)
    for c in range(3):
        px[:, :, c] = np.clip(rgb[:, :, c] * scale, 0, 255).astype(np.uint8)
    px[:, :, 3] = np.where(ok, ex + 128, 0).astype(np.uint8)
    out = bytearray(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {h} +X {w}\n".encode())
    for y in range(h):
        out += bytes((2, 2, w >> 8, w & 255))
        for c in range(4):
            row = px[y, :, c].tobytes()
            for x in range(0, w, 128):
                chunk = row[x:x + 128]
                out.append(len(chunk))
                out += chunk
    with open(path, "wb") as f:
        f.write(out)


def _camera(M34, fov=40.0):
    """The reference camera JSON of a lookat matrix of this project (columns: right, up,
    forward, position): translation and a look-at point one unit ahead."""
    pos = [float(v) for v in M34[:, 3]]
    ahead = [float(M34[i, 3] + M34[i, 2]) for i in range(3)]
    return {"transform": {"translation": pos, "lookat": ahead}, "fov": fov, "depth_of_field": 1.0,
            "aperture_radius": 0.0}


def _rot(axis, deg):
    import numpy as np
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    i, j = [(1, 2), (2, 0), (0, 1)][axis]
    R = np.eye(3)
    R[i, i], R[i, j], R[j, i], R[j, j] = c, -s, s, c
    return R


def _euler_xyz(R):
    """Angles (degrees) with R = Rx(a) Ry(b) Rz(c), the reference's order."""
    b = math.asin(max(-1.0, min(1.0, R[0, 2])))
    a = math.atan2(-R[1, 2], R[2, 2])
    c = math.atan2(-R[0, 1], R[0, 0])
    return [math.degrees(a), math.degrees(b), math.degrees(c)]


def _transform(M34):
    """Translation, uniform scale and Euler angles of a rotation-times-scale matrix,
    checked by rebuilding the matrix."""
    import numpy as np
    A = np.asarray(M34[:, :3], np.float64)
    s = float(np.cbrt(np.linalg.det(A)))
    ang = _euler_xyz(A / s)
    back = _rot(0, ang[0]) @ _rot(1, ang[1]) @ _rot(2, ang[2]) * s
    if np.abs(back - A).max() > 1e-4 * max(1.0, s):
        raise ValueError("instance transform is not a rotation times a uniform scale")
    return {"translation": [float(v) for v in M34[:, 3]], "scale": [s, s, s], "rotation": ang}


def _material(s, m, name, medium=None):
    from illume_gb300 import _capi as C
    alb = [float(v) for v in s.textures[m.albedo_tex].color]
    rough = float(s.textures[m.roughness_tex].color[0])
    if m.type == C.MAT_LAMBERT:
        d = {"type": "lambert", "albedo": alb}
    elif m.type == C.MAT_PLASTIC:
        d = {"type": "plastic", "albedo": alb, "ior": float(m.ior)}
    elif m.type == C.MAT_ROUGHREFRACTIVE:
        d = {"type": "roughrefractive", "albedo": alb, "roughness": rough, "ior": float(m.ior)}
    elif m.type == C.MAT_ROUGHCONDUCTOR:
        d = {"type": "roughconductor", "material": "Cu", "roughness": rough}
    elif m.type == C.MAT_REFRACTIVE:
        d = {"type": "refractive", "albedo": alb, "ior": float(m.ior)}
    else:
        raise ValueError(f"no reference material for type {m.type}")
    d["name"] = name
    if medium:
        d["medium"] = medium
    return d


def _mesh_file(P, T, files):
    key = hashlib.sha256(P.tobytes() + T.tobytes()).hexdigest()[:12]
    name = f"mesh_{key}.obj"
    if name not in files:
        _write_obj(os.path.join(WORK, name), P, T)
        files[name] = len(T)
    return name


def _cornell_jobs():
    for f in ("box.json", "quad.obj"):
        shutil.copyfile(os.path.join(ROOT, "tests", "golden", "scenes", f), os.path.join(WORK, f))
    return [{"scene": "box.json", "spp": 64, "depth": 8, "timeout": 600}]


def _traversal_jobs(files):
    from illume_gb300 import synth
    P, T = synth.displaced_icosphere(synth.freq_for_tris(100_000), 1)
    ico = _mesh_file(P, T, files)
    with open(os.path.join(WORK, "ground_c1.obj"), "w") as f:
        f.write("v -10 -1.2 -10\nv 10 -1.2 -10\nv 10 -1.2 10\nv -10 -1.2 10\n")
        f.write("vt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\nf 1/1 2/2 3/3\nf 1/1 3/3 4/4\n")
    identity = {"translation": [0, 0, 0], "scale": [1, 1, 1], "rotation": [0, 0, 0]}
    scene = {
        "environment_map": {"type": "bitmap", "file": "env.hdr"},
        "materials": [
            {"name": "gold", "type": "roughconductor", "material": "Au", "roughness": 0.2},
            {"name": "ground", "type": "lambert",
             "albedo": {"type": "checkerboard", "on_color": [0.8, 0.8, 0.8], "off_color": [0.2, 0.2, 0.2],
                        "scale": [16.0, 16.0]}},
        ],
        "meshes": [{"file": ico, "name": "ico", "bvh_items_per_node": 4},
                   {"file": "ground_c1.obj", "name": "ground", "has_texcoords": True}],
        "primitives": [{"type": "mesh_instance", "mesh": "ico", "material": "gold", "transform": identity},
                       {"type": "mesh_instance", "mesh": "ground", "material": "ground", "transform": identity}],
        "camera": _camera(synth.lookat((0.0, 0.8, -4.2), (0.0, -0.15, 0.0))),
        "render_settings": {"resolution": [1024, 1024], "ray_bias": 0.0001},
    }
    with open(os.path.join(WORK, "c1.json"), "w") as f:
        json.dump(scene, f)
    return [{"scene": "c1.json", "spp": 128, "depth": 25, "timeout": 900}]


def _subsurface_jobs(files):
    from illume_gb300 import synth
    with open(os.path.join(ROOT, "tests", "golden", "scenes", "box.json")) as f:
        scene = json.load(f)
    P, T = synth.displaced_icosphere(synth.freq_for_tris(700_000), 3)
    scene["meshes"].append({"file": _mesh_file(P, T, files), "name": "ico", "bvh_items_per_node": 4})
    scene["mediums"] = [{"name": "sss", "absorption": [1 - 0.01, 1 - 0.08, 1 - 0.3], "scattering": 1.0, "g": 0.7}]
    scene["materials"].append({"name": "sss_glass", "type": "refractive", "ior": 1.3, "albedo": [1.0, 1.0, 1.0],
                               "medium": "sss"})
    scene["primitives"] = [p for p in scene["primitives"] if p["type"] != "sphere"]
    scene["primitives"].append({"type": "mesh_instance", "mesh": "ico", "material": "sss_glass",
                                "transform": {"translation": [277.5, 140.0, 277.5], "scale": [120.0] * 3,
                                              "rotation": [0.0, 0.0, 0.0]}})
    scene["render_settings"]["resolution"] = [960, 720]
    with open(os.path.join(WORK, "sss.json"), "w") as f:
        json.dump(scene, f)
    return [{"scene": "sss.json", "spp": 256, "depth": 50, "timeout": 900}]


def _batch_jobs(files, n):
    from illume_gb300 import synth
    pool = synth.MeshPool(seed=2)
    out = []
    for sd, d in synth.batch_jobs(n, seed=2, pool=pool):
        j = d["job"]
        meshes, prims = [], []
        for mi, mesh in enumerate(sd.meshes):
            meshes.append({"file": _mesh_file(mesh.positions, mesh.tris, files), "name": f"m{mi}",
                           "bvh_items_per_node": 4})
        mats = [_material(sd, m, f"mat{k}") for k, m in enumerate(sd.materials)]
        for (mi, mat, M, _, _) in sd.instances:
            prims.append({"type": "mesh_instance", "mesh": f"m{mi}", "material": f"mat{mat}", "transform": _transform(M)})
        scene = {"environment_map": {"type": "bitmap", "file": "env.hdr"}, "materials": mats, "meshes": meshes,
                 "primitives": prims, "camera": _camera(sd.camera_transform, sd.camera_fov),
                 "render_settings": {"resolution": [d["width"], d["height"]], "ray_bias": float(sd.ray_bias)}}
        name = f"batch_{j:02d}.json"
        with open(os.path.join(WORK, name), "w") as f:
            json.dump(scene, f)
        out.append({"scene": name, "spp": d["spp"], "depth": d["max_depth"], "timeout": 600})
    return out


def _build_tree(obj):
    """One mesh loaded by the host build of the reference (writes its BVH cache file)."""
    sys.path.insert(0, ROOT)
    from oracle import pyref
    name = f"_tree_{os.path.splitext(obj)[0]}.json"
    with open(os.path.join(WORK, name), "w") as f:
        json.dump({"meshes": [{"file": obj, "name": "m", "bvh_items_per_node": 4}], "primitives": [],
                   "render_settings": {"resolution": [256, 256]}}, f)
    pyref.RefScene(name, WORK).close()
    os.remove(os.path.join(WORK, name))
    return obj


def max_pending_at_push(path):
    """Most right siblings on the stack of src/primitives/mesh.cu:485-527 when an inner
    node of this cached tree is popped, every box test taken as a hit (the worst case).

    The file holds node_amount, tri_index_amount (int32) and node_amount GPUNodes of 32
    bytes (AABB of six floats, then two uint32: left/right child, or for a leaf the
    triangle count with bit 31 set and the first index; src/accel/bvh.h:11-28). The
    traversal pops a node, and for an inner node pushes right then left, so when it pops
    a node every ancestor whose left child lies on the path still has its right child
    pending; the push then raises the stack to that count plus two. Every child index and
    leaf range is checked against the file's counts first."""
    import numpy as np
    raw = np.fromfile(path, dtype=np.uint32)
    n, ntri = int(raw[0]), int(raw[1])
    if raw.size != 2 + 8 * n + ntri:
        raise ValueError(f"{path}: size does not match its counts")
    nodes = raw[2:2 + 8 * n].reshape(n, 8)
    first, second = nodes[:, 6], nodes[:, 7]
    leaf = (first & 0x80000000) != 0
    count = (first & 0x7FFFFFFF).astype(np.int64)
    if np.any(~leaf & ((first >= n) | (second >= n))) or np.any(leaf & (second.astype(np.int64) + count > ntri)):
        raise ValueError(f"{path}: a child or a leaf range lies outside the tree")
    worst, todo = 0, [(0, 0)]
    while todo:
        i, pending = todo.pop()
        if first[i] & 0x80000000:
            continue
        worst = max(worst, pending)
        todo.append((int(second[i]), pending))
        todo.append((int(first[i]), pending + 1))
    return worst, n


def _digest(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def prepare(njobs=64):
    if not os.path.isdir(os.path.join(REF_ROOT, "src")):
        print("reference sources not available")
        return False
    sys.path.insert(0, ROOT)
    from illume_gb300 import synth
    from oracle import build_ref
    _copy_and_patch()
    os.makedirs(WORK)
    _write_rgbe(os.path.join(WORK, "env.hdr"), synth.environment_map(1, 2048, 1024)[:, :, :3])
    files = {}
    groups = {"cornell": _cornell_jobs(), "traversal": _traversal_jobs(files), "subsurface": _subsurface_jobs(files),
              "batch": _batch_jobs(files, njobs)}
    build_ref.build()
    objs = ["quad.obj", "ground_c1.obj"] + sorted(files, key=lambda k: -files[k])
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(min(len(objs), os.cpu_count() or 1)) as p:
        for obj in p.imap_unordered(_build_tree, objs):
            print("tree built:", obj, flush=True)
    checked = {}
    for f in sorted(os.listdir(WORK)):
        if f.endswith(".bvh"):
            pending, nodes = max_pending_at_push(os.path.join(WORK, f))
            print(f"{f}: {nodes} nodes, at most {pending} right siblings pending at an inner node")
            if pending > BVH_STACK_SIZE - 2:
                print("a push could pass the reference's traversal stack; not prepared")
                return False
            checked[f] = _digest(os.path.join(WORK, f))
    with open(os.path.join(WORK, "checked_bvh.json"), "w") as fh:
        json.dump(checked, fh)
    with open(os.path.join(WORK, "jobs.json"), "w") as fh:
        json.dump(groups, fh, indent=1)
    print("prepared", DEST)
    return True


# ---------------------------------------------------------------- build, run, check
def build():
    src = os.path.join(DEST, "src")
    if not os.path.isdir(src):
        print("no prepared copy at", DEST)
        return False
    units = []
    for d, _, files in os.walk(src):
        units += [os.path.join(d, f) for f in files if f.endswith((".cu", ".cpp"))]
    nvcc = os.path.join(CUDA_HOME, "bin", "nvcc")
    os.makedirs(os.path.join(DEST, "obj"), exist_ok=True)
    objs, jobs = [], []
    for u in sorted(units):
        o = os.path.join(DEST, "obj", os.path.relpath(u, src).replace(os.sep, "_") + ".o")
        objs.append(o)
        lang = ["-x", "cu"] if u.endswith(".cpp") else []
        jobs.append([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-rdc=true", "--use_fast_math", "-O3",
                     "-std=c++17", "-w", *lang, "-I", src, "-I", os.path.join(DEST, "include"), "-c", u, "-o", o])
    for c in ("arraylist.c", "bitmap.c"):
        o = os.path.join(DEST, "obj", c + ".o")
        objs.append(o)
        jobs.append(["gcc", "-O2", "-c", os.path.join(src, c), "-o", o])
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True) for j in jobs]
    ok = True
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        if p.returncode != 0:
            ok = False
            print("failed:", " ".join(j), "\n", out[-3000:])
    if not ok:
        return False
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-rdc=true", *objs, "-o", EXE, "-lcurand"],
                   check=True)
    print("built", EXE)
    return True


def _image_name(scene, spp, depth):
    """The file main.cu:12 names the saved frame (PPM content here)."""
    with open(os.path.join(WORK, scene)) as f:
        w, h = json.load(f)["render_settings"]["resolution"]
    return f"out-{w}x{h}-{spp}spp-{depth}md.png"


def _render(job, out_dir=None, keep_frame=False):
    scene, spp, depth = job["scene"], job["spp"], job["depth"]
    r = subprocess.run([EXE, "out", scene, str(spp), str(depth)], cwd=WORK, capture_output=True, text=True,
                       timeout=job["timeout"])
    text = r.stdout + r.stderr
    img = os.path.join(WORK, _image_name(scene, spp, depth))
    if out_dir:
        base = os.path.splitext(scene)[0]
        with open(os.path.join(out_dir, f"megakernel_{base}.log"), "w") as f:
            f.write(text)
        if keep_frame and os.path.exists(img):
            shutil.copyfile(img, os.path.join(out_dir, f"megakernel_{base}.ppm"))
    if os.path.exists(img):
        os.remove(img)
    rate = re.search(r"Rays per sec: ([0-9.eE+]+)", text)
    rays = re.search(r"Rays traced: ([0-9]+)", text)
    secs = re.search(r"Render time: ([0-9.eE+]+) seconds", text)
    if r.returncode != 0 or not rate or not rays:
        raise RuntimeError(f"{scene}: exit {r.returncode}: {text[-400:]}")
    return {"rays": int(rays.group(1)), "rays_per_s": float(rate.group(1)),
            "render_s": float(secs.group(1)) if secs else None}


def run(out_dir=None, groups=None):
    if not os.path.exists(EXE):
        print(json.dumps({"megakernel": "unavailable", "why": "not built"}))
        return
    if out_dir:
        os.makedirs(out_dir, exist_ok=True)
    with open(os.path.join(WORK, "checked_bvh.json")) as fh:
        checked = json.load(fh)
    for f, d in checked.items():
        if _digest(os.path.join(WORK, f)) != d:
            print(json.dumps({"megakernel": "unavailable", "why": f"{f} differs from the checked tree"}))
            return
    with open(os.path.join(WORK, "jobs.json")) as fh:
        all_groups = json.load(fh)
    out = {}
    for name, jobs in all_groups.items():
        if groups and name not in groups:
            continue
        res = [_render(j, out_dir, keep_frame=name in ("cornell", "traversal")) for j in jobs]
        rays = sum(r["rays"] for r in res)
        timed = sum(r["rays"] / r["rays_per_s"] for r in res)
        paths = sum(j["spp"] * _pixels(j["scene"]) for j in jobs)
        out[name] = {"jobs": len(jobs), "rays": rays, "timed_s": round(timed, 4),
                     "mrays_s": round(rays / timed / 1e6, 2), "rays_per_path": round(rays / paths, 4),
                     "render_s": round(sum(r["render_s"] or 0 for r in res), 4)}
        print(json.dumps({name: out[name]}), flush=True)
    print(json.dumps(out))


def _pixels(scene):
    with open(os.path.join(WORK, scene)) as f:
        w, h = json.load(f)["render_settings"]["resolution"]
    return w * h


def _read_ppm(path):
    import numpy as np
    with open(path, "rb") as f:
        data = f.read()
    head = data.split(b"\n", 3)
    w, h = (int(v) for v in head[1].split())
    return np.frombuffer(head[3], np.uint8)[:w * h * 3].reshape(h, w, 3)


def check(out_dir):
    """Build container: the mean 8-bit value of each saved frame against the host build
    of the same sources rendering the same scene, spp and depth."""
    import numpy as np
    sys.path.insert(0, ROOT)
    from oracle import build_ref, pyref
    build_ref.build()
    with open(os.path.join(WORK, "jobs.json")) as fh:
        all_groups = json.load(fh)
    res = {}
    for name in ("cornell", "traversal"):
        job = all_groups[name][0]
        path = os.path.join(out_dir, f"megakernel_{os.path.splitext(job['scene'])[0]}.ppm")
        if not os.path.exists(path):
            continue
        gpu = _read_ppm(path).astype(np.float64)
        rs = pyref.RefScene(job["scene"], WORK)
        s, _, rays = rs.render(rs.width, rs.height, job["spp"], job["depth"], nthreads=os.cpu_count())
        host = rs.tonemap(s, job["spp"]).reshape(rs.height, rs.width, 3).astype(np.float64)
        rs.close()
        res[name] = {"gpu_mean": [round(v, 3) for v in gpu.mean(axis=(0, 1))],
                     "host_mean": [round(v, 3) for v in host.mean(axis=(0, 1))],
                     "host_rays_per_path": round(rays / (rs.width * rs.height * job["spp"]), 4)}
    print(json.dumps(res))
    return res


if __name__ == "__main__":
    step = sys.argv[1] if len(sys.argv) > 1 else ""
    if step == "prepare":
        n = int(sys.argv[sys.argv.index("--jobs") + 1]) if "--jobs" in sys.argv else 64
        sys.exit(0 if prepare(n) else 1)
    elif step == "build":
        sys.exit(0 if build() else 1)
    elif step == "run":
        run(sys.argv[2] if len(sys.argv) > 2 else None, sys.argv[3].split(",") if len(sys.argv) > 3 else None)
    elif step == "check":
        check(sys.argv[2])
    else:
        print(__doc__)
