"""Generates tests/golden/ref_image_formats.npz: small BMP, TGA and PGM files (written here,
covering the header variants, bit depths, palettes, run-length coding and row orders the
library reads) and the texels the reference's own loader gives for each (stb_image behind
src/texture.cu:36-65, through the reference built for the host: a bitmap texture
evaluated at every texel centre, point sampled, divided by 255).

Run in the build container, where the reference checkout exists:
    PYTHONPATH=. python tests/golden/make_image_formats.py
"""
from __future__ import annotations

import ctypes
import json
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "ref_image_formats.npz")


def bmp(img, bpp, top_down=False, header=40, palette=None, masks=None):
    """img: (h, w, 3) uint8 RGB, or (h, w) palette indices when bpp <= 8."""
    h, w = img.shape[:2]
    stride = ((w * bpp + 31) // 32) * 4
    rows = []
    for y in range(h):
        r = bytearray(stride)
        if bpp <= 8:
            per = 8 // bpp
            for x in range(w):
                r[x // per] |= int(img[y, x]) << (8 - bpp * (x % per + 1))
        elif bpp == 24:
            for x in range(w):
                r[3 * x:3 * x + 3] = bytes([img[y, x, 2], img[y, x, 1], img[y, x, 0]])
        else:
            for x in range(w):
                rr, gg, bb = (int(v) for v in img[y, x])
                a = (x * 37 + y * 11) & 255
                if masks is None:
                    v = bb | gg << 8 | rr << 16 | a << 24
                else:
                    v = 0
                    for val, m in zip((rr, gg, bb, a), masks):
                        sh = (m & -m).bit_length() - 1
                        v |= val << sh
                r[4 * x:4 * x + 4] = struct.pack("<I", v)
        rows.append(bytes(r))
    data = b"".join(rows if top_down else rows[::-1])
    pal = b""
    if palette is not None:
        entry = 3 if header == 12 else 4
        pal = b"".join(bytes([c[2], c[1], c[0]] + ([0] if entry == 4 else [])) for c in palette)
    if header == 12:
        dib = struct.pack("<IhhHH", 12, w, -h if top_down else h, 1, bpp)
    else:
        comp = 3 if masks is not None else 0
        dib = struct.pack("<IiiHHIIiiII", header, w, -h if top_down else h, 1, bpp, comp, len(data), 2835, 2835,
                          len(palette) if palette is not None else 0, 0)
        if header > 40:
            m = masks or (0x00ff0000, 0x0000ff00, 0x000000ff, 0xff000000)
            dib += struct.pack("<IIII", *m) + bytes(header - 56)
        elif masks is not None:
            dib += struct.pack("<III", *masks[:3])
    offset = 14 + len(dib) + len(pal)
    return b"BM" + struct.pack("<IHHI", offset + len(data), 0, 0, offset) + dib + pal + data


def tga(pixels, w, h, itype, bpp, top_down=False, cmap=None, cm_first=0):
    """pixels: list of per-pixel byte strings in file order (row 0 first as stored)."""
    cm_bits = 24 if cmap is not None else 0
    hdr = struct.pack("<BBBHHBHHHHBB", 0, 1 if cmap is not None else 0, itype, cm_first,
                      len(cmap) if cmap is not None else 0, cm_bits, 0, 0, w, h, bpp, 0x20 if top_down else 0)
    body = b""
    if cmap is not None:
        body += b"".join(bytes([c[2], c[1], c[0]]) for c in cmap)
    if itype & 8:   # run-length packets: runs of equal pixels, raw packets otherwise
        i = 0
        while i < len(pixels):
            j = i
            while j + 1 < len(pixels) and pixels[j + 1] == pixels[i] and j + 1 - i < 127:
                j += 1
            if j > i:
                body += bytes([0x80 | (j - i)]) + pixels[i]
                i = j + 1
            else:
                k = i
                while k + 1 < len(pixels) and pixels[k + 1] != pixels[k] and k + 1 - i < 127:
                    k += 1
                body += bytes([k - i]) + b"".join(pixels[i:k + 1])
                i = k + 1
    else:
        body += b"".join(pixels)
    return hdr + body


def cases():
    rng = np.random.default_rng(17)
    rgb = lambda h, w: rng.integers(0, 256, (h, w, 3)).astype(np.uint8)
    pal256 = rng.integers(0, 256, (256, 3)).astype(np.uint8)
    out = {}
    out["bmp24.bmp"] = bmp(rgb(3, 5), 24)
    out["bmp24_top_down.bmp"] = bmp(rgb(3, 4), 24, top_down=True)
    out["bmp24_core_header.bmp"] = bmp(rgb(2, 3), 24, header=12)
    out["bmp32.bmp"] = bmp(rgb(2, 3), 32)
    out["bmp32_v4_bitfields.bmp"] = bmp(rgb(3, 3), 32, header=108, masks=(0x000000ff, 0x0000ff00, 0x00ff0000, 0xff000000))
    out["bmp8.bmp"] = bmp(rng.integers(0, 256, (3, 7)), 8, palette=pal256)
    out["bmp4.bmp"] = bmp(rng.integers(0, 16, (2, 9)), 4, palette=pal256[:16])
    out["bmp1.bmp"] = bmp(rng.integers(0, 2, (2, 17)), 1, palette=pal256[:2], top_down=True)
    img = rgb(3, 5)
    px24 = [bytes([img[y, x, 2], img[y, x, 1], img[y, x, 0]]) for y in range(3) for x in range(5)]
    out["tga24.tga"] = tga(px24, 5, 3, 2, 24)
    px32 = [p + bytes([200]) for p in px24]
    out["tga32_top_down.tga"] = tga(px32, 5, 3, 2, 32, top_down=True)
    px16 = [struct.pack("<H", int(v)) for v in rng.integers(0, 1 << 15, 12)]
    out["tga16.tga"] = tga(px16, 4, 3, 2, 16)
    runs = [px24[0]] * 5 + px24[5:9] + [px24[9]] * 6
    out["tga24_rle.tga"] = tga(runs, 5, 3, 10, 24)
    grey = [bytes([int(v)]) for v in rng.integers(0, 256, 12)]
    out["tga_grey.tga"] = tga(grey, 6, 2, 3, 8)
    out["tga_grey_rle.tga"] = tga([grey[0]] * 7 + grey[7:], 6, 2, 11, 8, top_down=True)
    # colour maps from entry 0: stb_image 2.14 skips a map's first-entry index as a byte
    # count and does not subtract it from the pixel indices, so maps that start later
    # decode differently there (this library follows the format: index - first entry)
    cm = rng.integers(0, 256, (20, 3)).astype(np.uint8)
    idx = [bytes([int(v)]) for v in rng.integers(0, 20, 15)]
    out["tga_colormap.tga"] = tga(idx, 5, 3, 1, 8, cmap=cm)
    out["tga_colormap_rle.tga"] = tga([idx[0]] * 4 + idx[4:], 5, 3, 9, 8, cmap=cm)
    g = rng.integers(0, 256, (4, 6)).astype(np.uint8)
    out["grey.pgm"] = b"P5\n# comment\n6 4\n255\n" + g.tobytes()
    return out


def main():
    from oracle import build_ref, pyref
    if not pyref.available():
        print("reference sources not available: fixture left as it is")
        return
    build_ref.build()
    L = pyref.lib()
    work = os.path.join(build_ref.WORK_DIR, "formats")
    os.makedirs(work, exist_ok=True)
    out = {}
    for name, data in cases().items():
        path = os.path.join(work, name)
        with open(path, "wb") as f:
            f.write(data)
        # the size from the file itself, then every texel centre
        w, h = (struct.unpack("<ii", data[18:26]) if name.endswith(".bmp") and data[14] != 12 else
                struct.unpack("<hh", data[18:22]) if name.endswith(".bmp") else
                struct.unpack("<HH", data[12:16]) if name.endswith(".tga") else
                tuple(int(v) for v in data.split(b"\n")[2].split()))
        h = abs(h)
        tex = np.zeros((h, w, 3), np.float32)
        for y in range(h):
            for x in range(w):
                o = (ctypes.c_float * 3)()
                with pyref.quiet():
                    L.ref_texture_eval(json.dumps({"type": "bitmap", "file": path}).encode(), (x + 0.5) / w,
                                       (y + 0.5) / h, o)
                tex[y, x] = list(o)
        key = name.replace(".", "_")
        out["file_" + key] = np.frombuffer(data, np.uint8)
        out["name_" + key] = np.array(name)
        out["texels_" + key] = tex
    np.savez_compressed(OUT, **out)
    print(OUT, len(cases()), "files")


if __name__ == "__main__":
    main()
