"""CPU baseline check: the reference's own integrator built for the host (oracle/_ref)
against the oracle port, timed on the same scene, frame and thread count.

TEST INFRASTRUCTURE (the reference checkout, or its staged copy, is needed to build
oracle/_ref). The bench's reference arm runs the reference's own integrator where it
can be built (bench.py reference_integrator_line) and the port elsewhere; the CPU
baseline inside the bench's own line runs the port. This script measures how the
port's speed compares with the reference's own code on the triangle-heavy traversal
scene, so the ratio can be stated beside either baseline.

The scene: the 100k-triangle displaced icosphere over the checkerboard ground with the
synthetic 2048x1024 environment, written as reference JSON + OBJ. The reference knows
only the Beckmann distribution and its named conductors, so the mesh is the reference's
rough "Au" conductor (Beckmann, alpha 0.2) in both runs; the port renders the scene the
reference's loader produced (its exported SceneData), so both trace the same geometry.

    PYTHONPATH=. python oracle/time_ref_vs_port.py [--res 256] [--spp 1] [--threads 0]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def write_scene(work: str, tris: int) -> str:
    from illume_gb300 import synth
    P, T = synth.displaced_icosphere(synth.freq_for_tris(tris), 1)
    with open(os.path.join(work, "ico_c1.obj"), "w") as f:
        f.write("".join("v %.9g %.9g %.9g\n" % tuple(p) for p in P))
        f.write("".join("f %d %d %d\n" % (a + 1, b + 1, c + 1) for a, b, c in T))
    with open(os.path.join(work, "ground_c1.obj"), "w") as f:
        f.write("v -10 -1.2 -10\nv 10 -1.2 -10\nv 10 -1.2 10\nv -10 -1.2 10\n")
        f.write("vt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\nf 1/1 2/2 3/3\nf 1/1 3/3 4/4\n")
    cam = synth.lookat((0.0, 0.8, -4.2), (0.0, -0.15, 0.0))
    identity = {"translation": [0, 0, 0], "scale": [1, 1, 1], "rotation": [0, 0, 0]}
    scene = {
        "environment_map": [1.0, 1.0, 1.0],
        "materials": [
            {"name": "gold", "type": "roughconductor", "material": "Au", "roughness": 0.2},
            {"name": "ground", "type": "lambert",
             "albedo": {"type": "checkerboard", "on_color": [0.8, 0.8, 0.8], "off_color": [0.2, 0.2, 0.2],
                        "scale": [16.0, 16.0]}},
        ],
        "meshes": [{"file": "ico_c1.obj", "name": "ico", "bvh_items_per_node": 4},
                   {"file": "ground_c1.obj", "name": "ground", "has_texcoords": True}],
        "primitives": [{"type": "mesh_instance", "mesh": "ico", "material": "gold", "transform": identity},
                       {"type": "mesh_instance", "mesh": "ground", "material": "ground", "transform": identity}],
        "camera": {"transform": {"translation": [float(v) for v in cam[:, 3]],
                                 "lookat": [0.0, -0.15, 0.0]},
                   "fov": 40.0, "depth_of_field": 1.0, "aperture_radius": 0.0},
        "render_settings": {"resolution": [1024, 1024], "ray_bias": 0.0001},
    }
    with open(os.path.join(work, "c1.json"), "w") as f:
        json.dump(scene, f)
    return "c1.json"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--res", type=int, default=256)
    ap.add_argument("--spp", type=int, default=1)
    ap.add_argument("--depth", type=int, default=25)
    ap.add_argument("--tris", type=int, default=100_000)
    ap.add_argument("--threads", type=int, default=0)
    args = ap.parse_args()
    from illume_gb300 import _capi as C, synth
    from illume_gb300.scenedata import Texture
    from oracle import build_ref, pyoracle, pyref
    if not pyref.available():
        print("reference sources not available")
        return
    build_ref.build()
    work = os.path.join(build_ref.WORK_DIR, f"timing_{args.tris}")   # BVH files are reused by name
    os.makedirs(work, exist_ok=True)
    name = write_scene(work, args.tris)
    env = synth.environment_map(1, 2048, 1024)
    t0 = time.perf_counter()
    rs = pyref.RefScene(name, work)
    rs.set_env(env)
    load_s = time.perf_counter() - t0
    sd = rs.export()
    sd.textures[sd.env_tex] = Texture(C.TEX_BITMAP, texels=env, hdr=1)
    threads = args.threads or os.cpu_count()
    W = H = args.res
    # one untimed warm-up frame each, then the timed frame
    rs.render(32, 32, 1, args.depth, nthreads=threads)
    t0 = time.perf_counter()
    _, _, ref_rays = rs.render(W, H, args.spp, args.depth, nthreads=threads)
    ref_s = time.perf_counter() - t0
    o = pyoracle.OracleScene(sd)
    o.render(32, 32, 1, args.depth, isect=C.ISECT_MT, nthreads=threads)
    t0 = time.perf_counter()
    _, _, port_rays = o.render(W, H, args.spp, args.depth, isect=C.ISECT_MT, precision=32, nthreads=threads)
    port_s = time.perf_counter() - t0
    rs.close()
    ref_v, port_v = ref_rays / ref_s / 1e6, port_rays / port_s / 1e6
    print(json.dumps({"frame": [W, H], "spp": args.spp, "depth": args.depth, "threads": threads,
                      "reference_load_s": round(load_s, 1),
                      "reference": {"rays": ref_rays, "s": round(ref_s, 2), "mrays_s": round(ref_v, 3)},
                      "port": {"rays": port_rays, "s": round(port_s, 2), "mrays_s": round(port_v, 3)},
                      "port_over_reference": round(port_v / ref_v, 3)}))


if __name__ == "__main__":
    main()
