"""Generates the golden fixtures of tests/golden/ from the reference renderer itself.

Run in the build container, where the reference sources exist:
    PYTHONPATH=. python tests/golden/make_golden.py [scene names]
(with only "textured", only that scene's fixture is written; the others stay as they are)

1. Writes the test scenes of tests/golden/scenes/ (JSON in the reference's scene format,
   OBJ meshes, and .hdr / .png bitmap textures; all authored here, none copied from the
   reference).
2. Runs the reference's own code, built for the host by oracle/build_ref.py, on seeded
   inputs and on those scenes, and stores its outputs:
     ref_components.npz   sampling, Fresnel, microfacet, intersection and tonemap functions
     ref_json.npz         transform / material / medium / texture parsing
     ref_scene_<name>.npz the parsed scene (HostScene + SceneRef export), camera rays,
                          closest hits of a seeded ray set, a small render and its tonemap
The fixtures are small and committed; the tests read them on machines without the
reference.
"""
from __future__ import annotations

import json
import math
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

SCENE_DIR = os.path.join(HERE, "scenes")


# ---------------------------------------------------------------- scene files
def write_obj_files():
    os.makedirs(SCENE_DIR, exist_ok=True)
    with open(os.path.join(SCENE_DIR, "quad.obj"), "w") as f:
        f.write("# unit quad in the xy plane\n")
        for v in [(-0.5, -0.5, 0), (0.5, -0.5, 0), (0.5, 0.5, 0), (-0.5, 0.5, 0)]:
            f.write("v %.6f %.6f %.6f\n" % v)
        for t in [(0, 0), (1, 0), (1, 1), (0, 1)]:
            f.write("vt %.6f %.6f\n" % t)
        f.write("f 1/1 2/2 3/3\nf 1/1 3/3 4/4\n")
    # unit cube with per-face normals and texcoords
    with open(os.path.join(SCENE_DIR, "box.obj"), "w") as f:
        f.write("# unit cube\n")
        corners = [(x, y, z) for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)]
        for c in corners:
            f.write("v %.6f %.6f %.6f\n" % c)
        for t in [(0, 0), (1, 0), (1, 1), (0, 1)]:
            f.write("vt %.6f %.6f\n" % t)
        normals = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
        for n in normals:
            f.write("vn %.6f %.6f %.6f\n" % n)
        idx = lambda x, y, z: 1 + (x * 4 + y * 2 + z)
        faces = [
            (0, [idx(1, 0, 0), idx(1, 1, 0), idx(1, 1, 1), idx(1, 0, 1)]),
            (1, [idx(0, 0, 1), idx(0, 1, 1), idx(0, 1, 0), idx(0, 0, 0)]),
            (2, [idx(0, 1, 0), idx(0, 1, 1), idx(1, 1, 1), idx(1, 1, 0)]),
            (3, [idx(0, 0, 1), idx(0, 0, 0), idx(1, 0, 0), idx(1, 0, 1)]),
            (4, [idx(1, 0, 1), idx(1, 1, 1), idx(0, 1, 1), idx(0, 0, 1)]),
            (5, [idx(0, 0, 0), idx(0, 1, 0), idx(1, 1, 0), idx(1, 0, 0)]),
        ]
        for n, q in faces:
            a, b, c, d = q
            f.write(f"f {a}/1/{n + 1} {b}/2/{n + 1} {c}/3/{n + 1}\n")
            f.write(f"f {a}/1/{n + 1} {c}/3/{n + 1} {d}/4/{n + 1}\n")
    # icosphere, 2 subdivisions (320 triangles), vertex normals and spherical texcoords
    t = (1 + 5 ** 0.5) / 2
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [tuple(np.array(v) / np.linalg.norm(v)) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(2):
        cache = {}
        nf = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                p = (np.array(verts[a]) + np.array(verts[b])) / 2
                verts.append(tuple(p / np.linalg.norm(p)))
                cache[key] = len(verts) - 1
            return cache[key]
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    with open(os.path.join(SCENE_DIR, "ico.obj"), "w") as f:
        f.write("# icosphere, 2 subdivisions\n")
        for v in verts:
            f.write("v %.6f %.6f %.6f\n" % v)
        for v in verts:
            u = 0.5 + math.atan2(v[2], v[0]) / (2 * math.pi)
            w = 0.5 - math.asin(max(-1.0, min(1.0, v[1]))) / math.pi
            f.write("vt %.6f %.6f\n" % (u, w))
        for v in verts:
            f.write("vn %.6f %.6f %.6f\n" % v)
        for a, b, c in faces:
            f.write(f"f {a + 1}/{a + 1}/{a + 1} {b + 1}/{b + 1}/{b + 1} {c + 1}/{c + 1}/{c + 1}\n")


def write_rgbe(path, rgb):
    """Radiance .hdr, flat (not run-length encoded) RGBE scanlines, top row first."""
    h, w, _ = rgb.shape
    out = bytearray(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {h} +X {w}\n".encode())
    for y in range(h):
        for x in range(w):
            r, g, b = (float(v) for v in rgb[y, x])
            m = max(r, g, b)
            if m < 1e-32:
                out += bytes(4)
                continue
            f, e = math.frexp(m)
            sc = f * 256.0 / m
            out += bytes([int(r * sc), int(g * sc), int(b * sc), e + 128])
    with open(path, "wb") as f:
        f.write(bytes(out))


def write_png(path, pix, color_type):
    """8-bit PNG (color type 0 gray, 2 RGB or 6 RGBA), filter 0 on every row."""
    import struct
    import zlib
    h, w = pix.shape[:2]
    raw = b"".join(b"\x00" + pix[y].astype(np.uint8).tobytes() for y in range(h))

    def chunk(tag, data):
        c = struct.pack(">I", len(data)) + tag + data
        return c + struct.pack(">I", zlib.crc32(tag + data) & 0xffffffff)
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, color_type, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 9)) + chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(png)


def write_texture_files():
    """Bitmap textures of the textured scene, seeded: an equirectangular sky with texel
    noise and a sharp sun lobe (a wrong uv or filter weight changes every escaped ray),
    an HDR albedo, and LDR albedo / roughness images in three PNG colour types."""
    rng = np.random.default_rng(77)
    W, H = 64, 32
    y = (np.arange(H) + 0.5) / H
    base = 0.25 + 0.9 * (1.0 - y)[:, None, None] * np.array([0.6, 0.75, 1.0])
    sky = base * (0.6 + 0.8 * rng.random((H, W, 3)))
    sun_x, sun_y = 41.3, 9.6
    xx, yy = np.meshgrid(np.arange(W) + 0.5, np.arange(H) + 0.5)
    lobe = 40.0 * np.exp(-((xx - sun_x) ** 2 + (yy - sun_y) ** 2) / (2 * 1.2 ** 2))
    sky = sky + lobe[:, :, None] * np.array([1.0, 0.9, 0.7])
    write_rgbe(os.path.join(SCENE_DIR, "sky.hdr"), sky)
    write_rgbe(os.path.join(SCENE_DIR, "tiles.hdr"), 0.05 + 0.9 * rng.random((16, 16, 3)))
    write_png(os.path.join(SCENE_DIR, "grid.png"), rng.integers(0, 256, size=(8, 8, 3)), 2)
    write_png(os.path.join(SCENE_DIR, "dots.png"), rng.integers(0, 256, size=(6, 10, 4)), 6)
    write_png(os.path.join(SCENE_DIR, "rough.png"), rng.integers(10, 120, size=(4, 8)), 0)


def tf(translation=(0, 0, 0), scale=(1, 1, 1), rotation=(0, 0, 0)):
    return {"translation": list(translation), "scale": list(scale), "rotation": list(rotation)}


def write_scene_files():
    # Config-0 Cornell box: five wall quads, ceiling light, mirror and glass spheres.
    box = {
        "materials": [
            {"name": "white", "type": "lambert", "albedo": [0.725, 0.71, 0.68]},
            {"name": "red", "type": "lambert", "albedo": [0.63, 0.065, 0.05]},
            {"name": "green", "type": "lambert", "albedo": [0.14, 0.45, 0.091]},
            {"name": "light", "type": "emissive", "albedo": [17.0, 12.0, 4.0]},
            {"name": "mirror", "type": "reflective", "albedo": [1.0, 1.0, 1.0]},
            {"name": "glass", "type": "refractive", "ior": 1.5, "albedo": [1.0, 1.0, 1.0]},
        ],
        "meshes": [{"file": "quad.obj", "name": "quad", "bvh_items_per_node": 4}],
        "primitives": [
            {"type": "mesh_instance", "mesh": "quad", "material": "white",
             "transform": tf((277.5, 0, 277.5), (555, 555, 555), (90, 0, 0))},
            {"type": "mesh_instance", "mesh": "quad", "material": "white",
             "transform": tf((277.5, 555, 277.5), (555, 555, 555), (90, 0, 0))},
            {"type": "mesh_instance", "mesh": "quad", "material": "white",
             "transform": tf((277.5, 277.5, 555), (555, 555, 555), (0, 0, 0))},
            {"type": "mesh_instance", "mesh": "quad", "material": "red",
             "transform": tf((0, 277.5, 277.5), (555, 555, 555), (0, 90, 0))},
            {"type": "mesh_instance", "mesh": "quad", "material": "green",
             "transform": tf((555, 277.5, 277.5), (555, 555, 555), (0, 90, 0))},
            {"type": "mesh_instance", "mesh": "quad", "material": "light",
             "transform": tf((277.5, 554.99, 277.5), (130, 105, 1), (90, 0, 0))},
            {"type": "sphere", "center": [185.0, 90.0, 370.0], "radius": 90.0, "material": "mirror"},
            {"type": "sphere", "center": [370.0, 90.0, 185.0], "radius": 90.0, "material": "glass"},
        ],
        "camera": {"transform": {"translation": [278.0, 273.0, -800.0], "rotation": [0.0, 0.0, 0.0]},
                   "fov": 40.0, "depth_of_field": 1.0, "aperture_radius": 0.0},
        "render_settings": {"resolution": [256, 256], "ray_bias": 0.01},
    }
    materials = {
        "environment_map": [0.5, 0.6, 0.8],
        "mediums": [{"name": "smoke", "absorption": [0.5, 0.6, 0.7], "scattering": 0.8, "g": 0.3}],
        "materials": [
            {"name": "floor", "type": "lambert",
             "albedo": {"type": "checkerboard", "on_color": [0.8, 0.8, 0.8], "off_color": [0.2, 0.2, 0.2],
                        "scale": [8.0, 8.0]}},
            {"name": "clay", "type": "lambert", "albedo": [0.7, 0.3, 0.2]},
            {"name": "mirror", "type": "reflective", "albedo": [0.9, 0.9, 0.9]},
            {"name": "glass", "type": "refractive", "ior": 1.5, "albedo": [0.98, 0.98, 0.98], "medium": "smoke"},
            {"name": "roughmirror", "type": "roughreflective", "ior": 1.4, "roughness": 0.1, "albedo": [0.8, 0.8, 0.8]},
            {"name": "roughglass", "type": "roughrefractive", "ior": 1.5, "roughness": 0.15,
             "albedo": [0.95, 0.95, 0.95]},
            {"name": "gold", "type": "conductor", "material": "Au"},
            {"name": "roughcopper", "type": "roughconductor", "material": "Cu", "roughness": 0.2},
            {"name": "plastic", "type": "plastic", "ior": 1.5, "albedo": [0.1, 0.4, 0.8]},
            {"name": "lamp", "type": "emissive", "albedo": [4.0, 4.0, 4.0]},
            {"name": "patchy", "type": "roughconductor", "material": "Ag",
             "roughness": {"type": "checkerboard", "on_color": [0.05, 0.05, 0.05], "off_color": [0.3, 0.3, 0.3],
                           "scale": [4.0, 2.0]}},
        ],
        "meshes": [{"file": "quad.obj", "name": "quad", "has_texcoords": True}],
        "primitives": [
            {"type": "mesh_instance", "mesh": "quad", "material": "floor",
             "transform": tf((0, 0, 0), (20, 20, 20), (90, 0, 0))},
            {"type": "sphere", "center": [-6.0, 1.0, 0.0], "radius": 1.0, "material": "clay"},
            {"type": "sphere", "center": [-3.6, 1.0, 0.0], "radius": 1.0, "material": "mirror"},
            {"type": "sphere", "center": [-1.2, 1.0, 0.0], "radius": 1.0, "material": "glass"},
            {"type": "sphere", "center": [1.2, 1.0, 0.0], "radius": 1.0, "material": "roughmirror"},
            {"type": "sphere", "center": [3.6, 1.0, 0.0], "radius": 1.0, "material": "roughglass"},
            {"type": "sphere", "center": [6.0, 1.0, 0.0], "radius": 1.0, "material": "gold"},
            {"type": "sphere", "center": [-3.6, 1.0, 3.0], "radius": 1.0, "material": "roughcopper"},
            {"type": "sphere", "center": [0.0, 1.0, 3.0], "radius": 1.0, "material": "plastic"},
            {"type": "sphere", "center": [3.6, 3.0, 3.0], "radius": 0.5, "material": "lamp"},
            {"type": "sphere", "center": [3.6, 1.0, 3.0], "radius": 1.0, "material": "patchy"},
        ],
        "camera": {"transform": {"translation": [0.0, 4.0, -12.0], "lookat": [0.0, 1.0, 1.0]},
                   "fov": 45.0, "depth_of_field": 1.0, "aperture_radius": 0.0},
        "render_settings": {"resolution": [64, 48], "ray_bias": 0.001, "tonemapper": "Filmic"},
    }
    mesh = {
        "environment_map": [0.2, 0.2, 0.25],
        "materials": [
            {"name": "floor", "type": "lambert",
             "albedo": {"type": "checkerboard", "on_color": [0.7, 0.7, 0.7], "off_color": [0.3, 0.3, 0.3],
                        "scale": [10.0, 10.0]}},
            {"name": "clay", "type": "lambert", "albedo": [0.6, 0.6, 0.5]},
            {"name": "gold", "type": "roughconductor", "material": "Au", "roughness": 0.1},
            {"name": "water", "type": "refractive", "ior": 1.33, "albedo": [0.95, 0.97, 1.0]},
            {"name": "crate", "type": "lambert",
             "albedo": {"type": "checkerboard", "on_color": [0.8, 0.5, 0.2], "off_color": [0.4, 0.2, 0.1],
                        "scale": [3.0, 3.0]}},
            {"name": "plastic", "type": "plastic", "ior": 1.45, "albedo": [0.8, 0.1, 0.1]},
            {"name": "light", "type": "emissive", "albedo": [10.0, 10.0, 10.0]},
        ],
        "meshes": [
            {"file": "ico.obj", "name": "ico"},
            {"file": "ico.obj", "name": "ico_smooth", "face_normals": False, "bvh_items_per_node": 8},
            {"file": "ico.obj", "name": "ico_flip", "flip_normals": True, "has_texcoords": True},
            {"file": "box.obj", "name": "box", "has_texcoords": True, "bvh_items_per_node": 2},
            {"file": "quad.obj", "name": "quad", "has_texcoords": True},
            {"file": "box.obj", "name": "zbox", "z_up": True, "face_normals": False},
        ],
        "primitives": [
            {"type": "mesh_instance", "mesh": "quad", "material": "floor",
             "transform": tf((0, 0, 0), (16, 16, 16), (90, 0, 0))},
            {"type": "mesh_instance", "mesh": "ico", "material": "clay", "transform": tf((-2.2, 1, 0))},
            {"type": "mesh_instance", "mesh": "ico_smooth", "material": "gold",
             "transform": tf((0, 1, 0), (1, 1, 1), (30, 45, 0))},
            {"type": "mesh_instance", "mesh": "ico_flip", "material": "water",
             "transform": tf((2.2, 1.5, 0), (1, 1.5, 1), (0, 0, 0))},
            {"type": "mesh_instance", "mesh": "box", "material": "crate",
             "transform": tf((0, 0.5, 3), (1, 1, 2), (0, 30, 0))},
            {"type": "mesh_instance", "mesh": "zbox", "material": "plastic",
             "transform": tf((3, 0.5, 3), (1, 1, 1), (10, 20, 30))},
            {"type": "sphere", "center": [0.0, 6.0, 0.0], "radius": 1.0, "material": "light"},
        ],
        "camera": {"transform": {"translation": [0.0, 3.0, -8.0], "rotation": [15.0, 0.0, 0.0]},
                   "fov": 50.0, "depth_of_field": 8.0, "aperture_radius": 0.05},
        "render_settings": {"resolution": [48, 40], "ray_bias": 0.001, "tonemapper": "Reinhard"},
    }
    textured = {
        "environment_map": {"type": "bitmap", "file": "sky.hdr"},
        "materials": [
            {"name": "floor", "type": "lambert", "albedo": {"type": "bitmap", "file": "tiles.hdr", "scale": [3.0, 3.0]}},
            {"name": "crate", "type": "lambert", "albedo": {"type": "bitmap", "file": "grid.png", "scale": [2.0, 2.0]}},
            {"name": "dotted", "type": "lambert", "albedo": {"type": "bitmap", "file": "dots.png"}},
            {"name": "brushed", "type": "roughconductor", "material": "Au",
             "roughness": {"type": "bitmap", "file": "rough.png", "scale": [2.0, 1.0]}},
            {"name": "mirror", "type": "reflective", "albedo": [0.95, 0.95, 0.95]},
            {"name": "tiledplastic", "type": "plastic", "ior": 1.5,
             "albedo": {"type": "bitmap", "file": "tiles.hdr", "scale": [1.5, 0.75]}},
        ],
        "meshes": [{"file": "quad.obj", "name": "quad", "has_texcoords": True},
                   {"file": "box.obj", "name": "box", "has_texcoords": True}],
        "primitives": [
            {"type": "mesh_instance", "mesh": "quad", "material": "floor",
             "transform": tf((0, 0, 0), (14, 14, 14), (90, 0, 0))},
            {"type": "mesh_instance", "mesh": "box", "material": "crate",
             "transform": tf((-3.2, 0.75, 1.0), (1.5, 1.5, 1.5), (0, 25, 0))},
            {"type": "sphere", "center": [-1.0, 1.0, -0.5], "radius": 1.0, "material": "dotted"},
            {"type": "sphere", "center": [1.3, 1.0, 0.5], "radius": 1.0, "material": "brushed"},
            {"type": "sphere", "center": [3.6, 1.2, 1.5], "radius": 1.2, "material": "mirror"},
            {"type": "sphere", "center": [0.4, 0.6, -2.4], "radius": 0.6, "material": "tiledplastic"},
        ],
        "camera": {"transform": {"translation": [0.0, 2.2, -9.0], "lookat": [0.0, 1.4, 0.0]},
                   "fov": 60.0, "depth_of_field": 1.0, "aperture_radius": 0.0},
        "render_settings": {"resolution": [64, 48], "ray_bias": 0.001},
    }
    for name, sc in (("box", box), ("materials", materials), ("mesh", mesh), ("textured", textured)):
        with open(os.path.join(SCENE_DIR, name + ".json"), "w") as f:
            json.dump(sc, f, indent=1)


# ---------------------------------------------------------------- reference outputs
def scene_aabb(sd):
    pts = []
    for (m, mat, M, inv, ti) in sd.instances:
        P = sd.meshes[m].positions
        pts.append(P @ M[:, :3].T + M[:, 3])
    for (c, r, mat) in sd.spheres:
        pts.append(np.array([c]) - r)
        pts.append(np.array([c]) + r)
    P = np.concatenate(pts)
    return P.min(0), P.max(0)


def seeded_rays(sd, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = scene_aabb(sd)
    ext = hi - lo
    lo, hi = lo - 0.1 * ext, hi + 0.1 * ext
    o = lo + rng.random((n, 3)) * (hi - lo)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], axis=1).astype(np.float32)


def gen_scene(name, pyref, golden_io, work):
    from oracle import build_ref
    for f in os.listdir(SCENE_DIR):
        if f.endswith((".obj", ".json", ".hdr", ".png")):
            shutil.copyfile(os.path.join(SCENE_DIR, f), os.path.join(work, f))
    rs = pyref.RefScene(name + ".json", work)
    sd = rs.export()
    out = golden_io.scene_to_arrays(sd)
    W, H = min(sd.width, 64), min(sd.height, 64)
    out["camera_size"] = np.array([W, H], np.int32)
    out["camera_rays"] = rs.camera_rays(W, H, sample=5, seed=0)
    rays = seeded_rays(sd, 4096, seed=11)
    t, prim, nrm = rs.closest_hit(rays)
    out["hit_rays"], out["hit_t"], out["hit_prim"], out["hit_normal"] = rays, t, prim, nrm
    spp, depth = (4, 8) if name == "box" else (4, 12)
    w, h = (32, 32) if name == "box" else (W, H)
    s, s2, nrays = rs.render(w, h, spp, depth, seed=0)
    out["render_size"] = np.array([w, h, spp, depth], np.int32)
    out["render_sum"], out["render_sumsq"], out["render_rays"] = s, s2, np.int64(nrays)
    out["render_rgb8"] = rs.tonemap(s, float(spp))
    rs.close()
    np.savez_compressed(os.path.join(HERE, f"ref_scene_{name}.npz"), **out)
    print(name, "rays", nrays, "mean", (s / spp).mean(0))


def gen_components(pyref):
    import ctypes
    L = pyref.lib()
    rng = np.random.default_rng(1234)
    n = 2048
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    out = {}
    # Fresnel dielectric over cosI in [-1, 1], ior in [1, 2.5]
    cosI = (rng.random(n) * 2 - 1).astype(np.float32)
    ior = (1 + rng.random(n) * 1.5).astype(np.float32)
    F = np.zeros(n, np.float32); cT = np.zeros(n, np.float32)
    for i in range(n):
        c = np.zeros(1, np.float32)
        F[i] = L.ref_fresnel_dielectric(float(cosI[i]), float(ior[i]), fp(c)); cT[i] = c[0]
    out.update(fres_cosI=cosI, fres_ior=ior, fres_F=F, fres_cosT=cT)
    eta = (0.1 + rng.random(n) * 2).astype(np.float32)
    k = (rng.random(n) * 5).astype(np.float32)
    cc = rng.random(n).astype(np.float32)
    out.update(cond_eta=eta, cond_k=k, cond_cos=cc,
               cond_F=np.array([L.ref_fresnel_conductor1(float(a), float(b), float(c)) for a, b, c in zip(eta, k, cc)],
                               np.float32))
    iors = np.array([1.3, 1.45, 1.5, 2.0], np.float32)
    out.update(dfres_ior=iors, dfres_val=np.array([L.ref_diffuse_fresnel(float(1.0 / x), 1000000) for x in iors],
                                                  np.float32))
    # samplers: u in (0, 1]
    u = ((np.floor(rng.random((n, 3)) * 16777216) + 1) / 16777216).astype(np.float32)
    out["u"] = u
    a = (0.01 + rng.random(n) * 0.8).astype(np.float32)
    g = (rng.random(n) * 1.8 - 0.9).astype(np.float32)
    g[:64] = 0.0
    out["alpha"], out["g"] = a, g
    res = {k2: np.zeros((n, 3), np.float32) for k2 in ("hemi", "circle", "sphere", "hg", "beck")}
    for i in range(n):
        L.ref_sample_hemisphere_cosine(float(u[i, 0]), float(u[i, 1]), fp(res["hemi"][i]))
        L.ref_sample_circle(float(u[i, 0]), float(u[i, 1]), fp(res["circle"][i]))
        L.ref_sample_sphere(float(u[i, 0]), float(u[i, 1]), fp(res["sphere"][i]))
        L.ref_sample_hg(float(g[i]), float(u[i, 0]), float(u[i, 1]), fp(res["hg"][i]))
        L.ref_sample_beckmann(float(a[i]), float(u[i, 0]), float(u[i, 1]), fp(res["beck"][i]))
    out.update({"s_" + k2: v for k2, v in res.items()})
    # basis, D, G
    nv = rng.normal(size=(n, 3)).astype(np.float32)
    nv /= np.linalg.norm(nv, axis=1, keepdims=True)
    vv = res["hemi"].copy()
    basis = np.zeros((n, 3), np.float32)
    for i in range(n):
        L.ref_to_basis(fp(np.ascontiguousarray(vv[i])), fp(np.ascontiguousarray(nv[i])), fp(basis[i]))
    out.update(basis_v=vv, basis_n=nv, basis_out=basis)
    m = basis
    D = np.array([L.ref_D_beckmann(fp(np.ascontiguousarray(m[i])), fp(np.ascontiguousarray(nv[i])), float(a[i]))
                  for i in range(n)], np.float32)
    wi = rng.normal(size=(n, 3)).astype(np.float32)
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3)).astype(np.float32)
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    G = np.array([L.ref_G_beckmann(fp(np.ascontiguousarray(wi[i])), fp(np.ascontiguousarray(wo[i])),
                                   fp(np.ascontiguousarray(m[i])), float(a[i])) for i in range(n)], np.float32)
    out.update(D_beck=D, G_wi=wi, G_wo=wo, G_beck=G)
    # triangle (Moller-Trumbore), AABB, sphere tests
    v = rng.normal(size=(n, 3, 3)).astype(np.float32)
    o = (rng.normal(size=(n, 3)) * 3).astype(np.float32)
    tgt = (v.mean(1) + rng.normal(size=(n, 3)) * 0.5).astype(np.float32)
    d = (tgt - o).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tt = np.zeros(n, np.float32); tu = np.zeros(n, np.float32); tv = np.zeros(n, np.float32)
    for i in range(n):
        uu = np.zeros(1, np.float32); vw = np.zeros(1, np.float32)
        tt[i] = L.ref_triangle_intersect(fp(np.ascontiguousarray(v[i, 0])), fp(np.ascontiguousarray(v[i, 1])),
                                         fp(np.ascontiguousarray(v[i, 2])), fp(np.ascontiguousarray(o[i])),
                                         fp(np.ascontiguousarray(d[i])), fp(uu), fp(vw))
        tu[i], tv[i] = uu[0], vw[0]
    out.update(tri_v=v, tri_o=o, tri_d=d, tri_t=tt, tri_u=tu, tri_v_out=tv)
    bl = np.minimum(v[:, 0], v[:, 1]); bh = np.maximum(v[:, 0], v[:, 1])
    out.update(box_lo=bl, box_hi=bh, box_t=np.array([L.ref_aabb_intersect(
        fp(np.ascontiguousarray(bl[i])), fp(np.ascontiguousarray(bh[i])), fp(np.ascontiguousarray(o[i])),
        fp(np.ascontiguousarray(d[i]))) for i in range(n)], np.float32))
    cen = v[:, 0]
    rad = (0.3 + rng.random(n)).astype(np.float32)
    st = np.zeros(n, np.float32); sn = np.zeros((n, 3), np.float32); suv = np.zeros((n, 2), np.float32)
    shit = np.zeros(n, np.int32)
    for i in range(n):
        t1 = np.zeros(1, np.float32)
        shit[i] = L.ref_sphere_intersect(fp(np.ascontiguousarray(cen[i])), float(rad[i]), fp(np.ascontiguousarray(o[i])),
                                         fp(np.ascontiguousarray(d[i])), fp(t1), fp(sn[i]), fp(suv[i]))
        st[i] = t1[0]
    out.update(sph_c=cen, sph_r=rad, sph_hit=shit, sph_t=st, sph_n=sn, sph_uv=suv)
    # tonemap operators
    rad_in = (np.abs(rng.normal(size=(n, 3))) * 2).astype(np.float32)
    for op in range(4):
        r = np.zeros((n, 3), np.float32)
        for i in range(n):
            L.ref_tonemap_eval(op, fp(np.ascontiguousarray(rad_in[i])), fp(r[i]))
        out[f"tone{op}"] = r
    out["tone_in"] = rad_in
    np.savez_compressed(os.path.join(HERE, "ref_components.npz"), **out)


def gen_json(pyref):
    import ctypes
    L = pyref.lib()
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    transforms = [
        {"translation": [1, 2, 3]},
        {"translation": [278, 273, -800], "rotation": [0, 0, 0]},
        {"translation": [277.5, 0, 277.5], "scale": [555, 555, 555], "rotation": [90, 0, 0]},
        {"translation": [-2.5, 1.25, 4], "scale": [0.5, 2, 1.5], "rotation": [10, 20, 30]},
        {"translation": [0, 4, -12], "lookat": [0, 1, 1]},
        {"translation": [3, -1, 2], "lookat": [-2, 5, 7], "scale": [2, 2, 2]},
        {"scale": [3, 1, 0.25], "rotation": [-45, 135, 270]},
    ]
    out = {"transforms_json": np.array([json.dumps(t) for t in transforms])}
    mats = np.zeros((len(transforms), 3, 16), np.float32)
    for i, t in enumerate(transforms):
        L.ref_transform_from_json(json.dumps(t).encode(), fp(mats[i, 0]), fp(mats[i, 1]), fp(mats[i, 2]))
    out["transforms"] = mats
    materials = [
        {"type": "lambert", "albedo": [0.1, 0.2, 0.3]},
        {"type": "emissive", "albedo": 2.5},
        {"type": "reflective"},
        {"type": "refractive", "ior": 1.33, "albedo": [0.9, 0.9, 0.9]},
        {"type": "roughreflective", "ior": 1.4, "roughness": 0.05, "albedo": [0.8, 0.8, 0.8]},
        {"type": "roughrefractive", "ior": 1.5, "roughness": 0.1},
        {"type": "conductor", "material": "Ag"},
        {"type": "conductor", "material": "Al"},
        {"type": "roughconductor", "material": "Au", "roughness": 0.08},
        {"type": "roughconductor", "material": "Pb", "roughness": 0.3},
        {"type": "conductor", "material": "unobtainium"},
        {"type": "plastic", "ior": 1.5, "albedo": [1.0, 0.37, 0.01]},
        {"type": "diffuse", "color": [0.5, 0.5, 0.5]},
    ]
    rows = []
    for m in materials:
        ior = np.zeros(1, np.float32); df = np.zeros(1, np.float32)
        eta = np.zeros(3, np.float32); k = np.zeros(3, np.float32)
        alb = np.zeros(3, np.float32); rough = np.zeros(3, np.float32)
        with pyref.quiet():
            typ = L.ref_material_from_json(json.dumps(m).encode(), fp(ior), fp(df), fp(eta), fp(k), fp(alb), fp(rough))
        rows.append(np.concatenate([[typ, ior[0], df[0]], eta, k, alb, rough]))
    out["materials_json"] = np.array([json.dumps(m) for m in materials])
    out["materials"] = np.array(rows, np.float32)
    mediums = [{"absorption": [0.5, 0.6, 0.7], "scattering": 0.8, "g": 0.3},
               {"absorption": [0.99, 0.92, 0.7], "scattering": 1.0},
               {"absorption": [1.0, 1.0, 1.0], "scattering": 0.0, "g": 0.1}]
    mrows = []
    for m in mediums:
        ab = np.zeros(3, np.float32); sc = np.zeros(1, np.float32); g = np.zeros(1, np.float32)
        act = ctypes.c_int()
        with pyref.quiet():
            L.ref_medium_from_json(json.dumps(m).encode(), fp(ab), fp(sc), fp(g), ctypes.byref(act))
        mrows.append(np.concatenate([ab, sc, g, [act.value]]))
    out["mediums_json"] = np.array([json.dumps(m) for m in mediums])
    out["mediums"] = np.array(mrows, np.float32)
    textures = [[0.25, 0.5, 0.75], {"type": "constant", "color": [0.3, 0.2, 0.1]},
                {"type": "checkerboard", "on_color": [1, 1, 1], "off_color": [0, 0, 0], "scale": [8, 8]},
                {"type": "checkerboard", "on_color": [0.9, 0.1, 0.1], "off_color": [0.1, 0.1, 0.9], "scale": [3.7, 5.2]}]
    rng = np.random.default_rng(7)
    uvs = (rng.random((256, 2)) * 1.4 - 0.2).astype(np.float32)
    tex_out = np.zeros((len(textures), 256, 3), np.float32)
    for i, t in enumerate(textures):
        for j in range(256):
            with pyref.quiet():
                L.ref_texture_eval(json.dumps(t).encode(), float(uvs[j, 0]), float(uvs[j, 1]), fp(tex_out[i, j]))
    out["textures_json"] = np.array([json.dumps(t) for t in textures])
    out["texture_uv"] = uvs
    out["textures"] = tex_out
    np.savez_compressed(os.path.join(HERE, "ref_json.npz"), **out)


def main():
    write_obj_files()
    write_texture_files()
    write_scene_files()
    from oracle import build_ref, pyref
    import golden_io
    if not pyref.available():
        print("reference sources not available: scene files written, fixtures left as they are")
        return
    build_ref.build()
    work = os.path.join(build_ref.WORK_DIR, "golden")
    os.makedirs(work, exist_ok=True)
    names = sys.argv[1:] or ["box", "materials", "mesh", "textured"]
    if names == ["textured"]:
        gen_scene("textured", pyref, golden_io, work)
        return
    gen_components(pyref)
    gen_json(pyref)
    for name in names:
        gen_scene(name, pyref, golden_io, work)


if __name__ == "__main__":
    main()
