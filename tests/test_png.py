"""PNG bitmap textures on CPU: files written here by an independent encoder (Python's zlib
for the deflate stream at several compression levels, every scanline filter, every
colour type and bit depth, Adam7 interlace) must decode to the texels stb_image gives
the reference (8-bit RGBA: grey replicated, alpha 255 unless given, palettes expanded,
16-bit samples reduced to their high byte, sub-byte grey scaled to 0..255)."""
import json
import struct
import zlib

import numpy as np
import pytest

from illume_gb300 import _capi as C
from test_ingest import CAM, host_scene_from_json

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def chunk(t, data):
    return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xFFFFFFFF)


def paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def filter_rows(rows, bpp, rng):
    out, prev = b"", bytes(len(rows[0])) if rows else b""
    for r in rows:
        f = int(rng.integers(5))
        enc = bytearray(len(r))
        for i in range(len(r)):
            a = r[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, paeth(a, b, c)][f]
            enc[i] = (r[i] - pred) & 0xFF
        out += bytes([f]) + bytes(enc)
        prev = r
    return out


def pack_row(samples, depth):
    """samples: 1-D int array of one row (all channels interleaved)."""
    if depth == 16:
        return b"".join(struct.pack(">H", int(v)) for v in samples)
    if depth == 8:
        return bytes(int(v) for v in samples)
    out, acc, nbits = bytearray(), 0, 0
    for v in samples:
        acc = (acc << depth) | int(v)
        nbits += depth
        if nbits == 8:
            out.append(acc)
            acc, nbits = 0, 0
    if nbits:
        out.append(acc << (8 - nbits))
    return bytes(out)


def encode_png(img, depth, ctype, interlace, rng, level, plte=None, trns=None):
    """img: (H, W, C) integer samples at `depth` bits."""
    H, W, ch = img.shape
    bpp = max(1, ch * depth // 8)
    raw = b""
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    for (x0, y0, dx, dy) in passes:
        sub = img[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        rows = [pack_row(sub[y].reshape(-1), depth) for y in range(sub.shape[0])]
        raw += filter_rows(rows, bpp, rng)
    ihdr = struct.pack(">IIBBBBB", W, H, depth, ctype, 0, 0, interlace)
    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr)
    if plte is not None:
        out += chunk(b"PLTE", bytes(plte.reshape(-1).astype(np.uint8)))
    if trns is not None:
        out += chunk(b"tRNS", trns)
    z = zlib.compress(raw, level)
    # split the stream over several IDAT chunks
    cut = len(z) // 2
    out += chunk(b"IDAT", z[:cut]) + chunk(b"IDAT", z[cut:]) + chunk(b"IEND", b"")
    return out


def expected_rgba(img, depth, ctype, plte=None, trns_idx=None, key=None):
    H, W, _ = img.shape
    out = np.zeros((H, W, 4), np.float32)
    out[..., 3] = 255
    if ctype == 3:
        out[..., :3] = plte[img[..., 0]]
        if trns_idx is not None:
            a = np.full(256, 255.0)
            a[:len(trns_idx)] = trns_idx
            out[..., 3] = a[img[..., 0]]
        return out
    hi = img >> 8 if depth == 16 else img
    if ctype in (0, 4):
        g = hi[..., 0] * (255 // ((1 << depth) - 1)) if depth < 8 else hi[..., 0]
        out[..., 0] = out[..., 1] = out[..., 2] = g
        if ctype == 4:
            out[..., 3] = hi[..., 1]
        elif key is not None:
            out[..., 3][img[..., 0] == key[0]] = 0
    else:
        out[..., :3] = hi[..., :3]
        if ctype == 6:
            out[..., 3] = hi[..., 3]
        elif key is not None:
            out[..., 3][np.all(img[..., :3] == np.array(key), axis=-1)] = 0
    return out


def load(tmp_path, name):
    sc = {"materials": [{"name": "m", "type": "lambert", "albedo": {"type": "bitmap", "file": name}}],
          "primitives": [{"type": "sphere", "center": [0, 0, 0], "radius": 1, "material": "m"}], "camera": CAM}
    sd = host_scene_from_json(json.dumps(sc), str(tmp_path))
    return sd.textures[sd.materials[0].albedo_tex]


CASES = [(ct, d) for ct, ds in ((0, (1, 2, 4, 8, 16)), (2, (8, 16)), (3, (1, 2, 4, 8)), (4, (8, 16)), (6, (8, 16)))
         for d in ds]


@pytest.mark.parametrize("interlace", [0, 1])
@pytest.mark.parametrize("ctype,depth", CASES)
def test_png_decodes_like_stb(native_lib, tmp_path, ctype, depth, interlace):
    rng = np.random.default_rng(depth * 10 + ctype + 100 * interlace)
    H, W = int(rng.integers(1, 23)), int(rng.integers(1, 29))
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    plte = trns = None
    trns_idx = key = None
    if ctype == 3:
        n = 1 << depth
        img = rng.integers(0, n, size=(H, W, 1))
        plte = rng.integers(0, 256, size=(n, 3))
        trns_idx = rng.integers(0, 256, size=max(1, n // 2))
        trns = bytes(trns_idx.astype(np.uint8))
    else:
        img = rng.integers(0, 1 << depth, size=(H, W, ch))
        if ctype in (0, 2):
            key = [int(v) for v in img[0, 0, :ch]]   # make the key occur
            trns = b"".join(struct.pack(">H", v) for v in key)
    data = encode_png(img, depth, ctype, interlace, rng, level=int(rng.integers(0, 10)), plte=plte, trns=trns)
    (tmp_path / "t.png").write_bytes(data)
    t = load(tmp_path, "t.png")
    assert t.type == C.TEX_BITMAP and t.hdr == 0
    want = expected_rgba(img, depth, ctype, plte, trns_idx, key)
    assert t.texels.shape == want.shape
    assert np.array_equal(t.texels, want)


def test_png_large_dynamic_huffman(native_lib, tmp_path):
    """A photo-like image large enough for multi-block dynamic-Huffman streams."""
    rng = np.random.default_rng(7)
    H, W = 300, 257
    yy, xx = np.mgrid[0:H, 0:W]
    base = (np.stack([xx * 255 // W, yy * 255 // H, (xx + yy) % 256], -1) + rng.integers(0, 8, (H, W, 3))) % 256
    data = encode_png(base, 8, 2, 0, rng, level=9)
    (tmp_path / "big.png").write_bytes(data)
    t = load(tmp_path, "big.png")
    assert np.array_equal(t.texels[..., :3], base.astype(np.float32))


def test_corrupt_png_becomes_black(native_lib, tmp_path):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, size=(8, 8, 3))
    data = bytearray(encode_png(img, 8, 2, 0, rng, level=6))
    data[60:70] = b"\x00" * 10       # damage the deflate stream
    (tmp_path / "bad.png").write_bytes(bytes(data))
    t = load(tmp_path, "bad.png")
    assert t.type == C.TEX_CONSTANT


def _format_cases():
    from conftest import golden
    z = golden("ref_image_formats.npz")
    return z, sorted(k[len("file_"):] for k in z.files if k.startswith("file_"))


@pytest.mark.parametrize("key", _format_cases()[1])
def test_bmp_tga_pgm_decode_like_the_reference(native_lib, tmp_path, key):
    """BMP (1/4/8/24/32 bits, core / info / V4 headers, bit fields, both row orders), TGA
    (colour-mapped, true-colour and grey, raw and run-length, 8/16/24/32 bits, both row
    orders) and PGM files: the texels equal the ones the reference's own loader gives
    (tests/golden/make_image_formats.py); a file it cannot read is black for both."""
    z, _ = _format_cases()
    name = str(z["name_" + key])
    (tmp_path / name).write_bytes(z["file_" + key].tobytes())
    want = z["texels_" + key]
    tex = load(tmp_path, name)
    if tex.type == C.TEX_CONSTANT:     # the loader refused the file: a black constant
        assert not want.any(), name
        return
    got = np.asarray(tex.texels, np.float32).reshape(want.shape[0], want.shape[1], 4)[..., :3] / np.float32(255)
    assert np.array_equal(got, want), (name, np.argwhere(got != want)[:5])


def test_mutated_bmp_tga_pgm_files_load_or_turn_black(native_lib, tmp_path):
    """Byte flips, overwritten words and truncations of the format fixtures: every file
    loads as some texture or is refused (a black constant); none crashes the loader."""
    z, keys = _format_cases()
    rng = np.random.default_rng(0)
    for key in keys:
        name = str(z["name_" + key])
        data = bytearray(z["file_" + key].tobytes())
        for trial in range(40):
            d = bytearray(data)
            if trial % 3 == 0:
                for _ in range(int(rng.integers(1, 6))):
                    d[int(rng.integers(0, len(d)))] = int(rng.integers(0, 256))
            elif trial % 3 == 1:
                d = d[:int(rng.integers(0, len(d)))]
            else:
                i = int(rng.integers(0, max(1, len(d) - 4)))
                d[i:i + 4] = bytes(int(v) for v in rng.integers(0, 256, 4))
            (tmp_path / name).write_bytes(bytes(d))
            tex = load(tmp_path, name)
            assert tex.type in (C.TEX_CONSTANT, C.TEX_BITMAP)
