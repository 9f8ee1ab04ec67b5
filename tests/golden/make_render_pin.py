"""Generates tests/golden/ref_render_pin_cornell.npz: the reference's one shipped render as
a loose integration pin.

Run in the build container, where the reference checkout exists:
    PYTHONPATH=. python tests/golden/make_render_pin.py

The reference ships one render of a scene whose assets it also ships:
renders/cornell-1024x1024-100000spp-100md.png, of res/scenes/cornell_box.json (1024x1024,
100,000 samples per pixel, depth 100, linear tonemap). It came from an older revision
(cuRAND XORWOW streams, fast math), so it pins the integrator statistically, not pixel
by pixel. This script stores
  * the scene as the reference's own loader parses it (HostScene + SceneRef export, the
    same export the other golden scenes use);
  * the render's 16 x 16 regions of 64 x 64 pixels as linear radiance bounds: the
    linear tonemap is (clamp(x) ^ (1 / 2.2)) x 255 truncated (src/tonemapper.cu), so a
    byte v < 255 means x lies in [(v / 255) ^ 2.2, ((v + 1) / 255) ^ 2.2); a region's
    radiance mean lies between the means of those bounds. Regions holding a clipped byte
    (255) bound nothing and are marked unusable;
  * the regions where the reference's present code (built for the host, oracle/_ref)
    itself lies more than 4 standard errors outside those bounds in a 128 x 128 render
    at 2048 spp (seed 0): where the shipped render and today's reference code differ.
    The oracle and the GPU renderer draw the same per-path streams as that build, so
    they differ from the shipped render in the same regions and nowhere else.
"""
from __future__ import annotations

import os
import shutil
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

OUT = os.path.join(HERE, "ref_render_pin_cornell.npz")
RENDER = os.path.join("renders", "cornell-1024x1024-100000spp-100md.png")
GRID = 16
PIN_RES, PIN_SPP = 128, 2048   # the reference code's own render against the pin


def read_png_rgb8(path: str) -> np.ndarray:
    """8-bit RGB, non-interlaced PNG (ISO 15948 filters 0-4) as an (h, w, 3) array."""
    d = open(path, "rb").read()
    assert d[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, [], 0, 0
    while pos < len(d):
        n, = struct.unpack(">I", d[pos:pos + 4])
        typ, body = d[pos + 4:pos + 8], d[pos + 8:pos + 8 + n]
        pos += 12 + n
        if typ == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
            assert depth == 8 and ctype == 2 and interlace == 0, (depth, ctype, interlace)
        elif typ == b"IDAT":
            idat.append(body)
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8).reshape(h, 3 * w + 1)
    out = np.zeros((h, 3 * w), np.int32)
    prev = np.zeros(3 * w, np.int32)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros(3 * w, np.int32)
            for x in range(3 * w):
                a = cur[x - 3] if x >= 3 else 0
                b = prev[x]
                c = prev[x - 3] if x >= 3 else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, 3).astype(np.uint8)


def main():
    from oracle import build_ref, pyref
    import golden_io
    if not pyref.available():
        print("reference sources not available: fixture left as it is")
        return
    build_ref.build()
    img = read_png_rgb8(os.path.join(build_ref.REF_ROOT, RENDER))
    h, w, _ = img.shape
    k = h // GRID
    v = img.astype(np.float64)
    lo = (v / 255.0) ** 2.2
    hi = ((v + 1.0) / 255.0) ** 2.2
    blocks = lambda a: a.reshape(GRID, k, GRID, k, 3).mean(axis=(1, 3))
    usable = (img.reshape(GRID, k, GRID, k, 3) < 255).all(axis=(1, 3, 4))
    work = os.path.join(build_ref.WORK_DIR, "render_pin")
    os.makedirs(os.path.join(work, "res"), exist_ok=True)
    for f in ("cube.obj", "quad.obj"):
        shutil.copyfile(os.path.join(build_ref.REF_ROOT, "res", f), os.path.join(work, "res", f))
    shutil.copyfile(os.path.join(build_ref.REF_ROOT, "res", "scenes", "cornell_box.json"),
                    os.path.join(work, "cornell_box.json"))
    rs = pyref.RefScene("cornell_box.json", work)
    sd = rs.export()
    pin = dict(region_lo=blocks(lo).astype(np.float64), region_hi=blocks(hi).astype(np.float64),
               region_usable=usable)
    sys.path.insert(0, os.path.dirname(HERE))
    from conftest import render_pin_check
    s, s2, _ = rs.render(PIN_RES, PIN_RES, PIN_SPP, 100)
    rs.close()
    far, usable_n, image_z = render_pin_check(s.astype(np.float64), s2.astype(np.float64), PIN_SPP, PIN_RES, pin,
                                              return_mask=True)
    out = golden_io.scene_to_arrays(sd)
    out.update(pin, render_size=np.array([w, h], np.int32), render_spp=np.int32(100000), render_depth=np.int32(100),
               mean_rgb8=img.reshape(-1, 3).mean(axis=0), ref_code_far=far, ref_code_res=np.int32(PIN_RES),
               ref_code_spp=np.int32(PIN_SPP), ref_code_image_z=image_z)
    np.savez_compressed(OUT, **out)
    print(OUT, "usable regions", int(usable.sum()), "of", GRID * GRID, "mean rgb8", img.reshape(-1, 3).mean(axis=0),
          "regions where the reference code differs", int(far.sum()), "image z", image_z)


if __name__ == "__main__":
    main()
