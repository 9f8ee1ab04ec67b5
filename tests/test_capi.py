"""The C-ABI library: loads, exports every entry point of include/illume.h, reports
errors through status codes (never exits), and builds host-only scenes on CPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, SCENES
from illume_gb300 import _capi as C


def header_functions():
    text = open(os.path.join(ROOT, "include", "illume.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[a-z_][a-z_0-9 \*]*?\b(illume_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(native_lib):
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(native_lib, n)]
    assert not missing, missing
    assert set(names) == set(C.PROTOTYPES), set(names) ^ set(C.PROTOTYPES)


def test_abi_version(native_lib):
    assert native_lib.illume_abi_version() == 4


def load_host(path, base=SCENES):
    h = ctypes.c_void_p()
    st = C.lib().illume_scene_load_json(None, path.encode(), base.encode() if base else None, ctypes.byref(h))
    return st, h


@pytest.mark.parametrize("name", ["box", "materials", "mesh", "textured"])
def test_host_only_scene_and_bvh_invariants(native_lib, name):
    st, h = load_host(os.path.join(SCENES, name + ".json"))
    assert st == C.OK, native_lib.illume_last_error()
    buf = ctypes.create_string_buffer(8192)
    assert native_lib.illume_scene_check_bvh(h, buf, 8192) == C.OK, native_lib.illume_last_error()
    assert b"mesh 0" in buf.value
    native_lib.illume_scene_destroy(h)


def test_bvh_invariants_on_a_large_irregular_mesh(native_lib):
    from illume_gb300 import synth
    from illume_gb300.scenedata import Mesh, SceneData, Material
    P, T = synth.displaced_icosphere(23, seed=5)          # 10,580 triangles
    rng = np.random.default_rng(0)
    P2 = (rng.normal(size=(300, 3)) * [5, 0.01, 5]).astype(np.float32)   # thin slab of random triangles
    T2 = rng.integers(0, 300, size=(400, 3)).astype(np.int32)
    s = SceneData()
    a = s.add_mesh(Mesh(P, T))
    b = s.add_mesh(Mesh(P2, T2))
    m = s.add_material(Material(C.MAT_LAMBERT, s.constant((0.5, 0.5, 0.5)), s.constant((0, 0, 0))))
    s.add_instance(a, m)
    s.add_instance(b, m)
    desc, keep = s.to_desc()
    h = ctypes.c_void_p()
    assert native_lib.illume_scene_create(None, ctypes.byref(desc), ctypes.byref(h)) == C.OK
    buf = ctypes.create_string_buffer(8192)
    assert native_lib.illume_scene_check_bvh(h, buf, 8192) == C.OK, native_lib.illume_last_error()
    native_lib.illume_scene_destroy(h)


def test_malformed_json_is_a_parse_error(native_lib):
    h = ctypes.c_void_p()
    st = native_lib.illume_scene_load_json_string(None, b'{"materials": [', None, ctypes.byref(h))
    assert st == C.ERR_PARSE
    assert b"JSON" in native_lib.illume_last_error()
    assert not h


def test_missing_obj_is_an_io_error(native_lib, tmp_path):
    j = '{"meshes": [{"file": "nope.obj", "name": "m"}], "primitives": []}'
    h = ctypes.c_void_p()
    st = native_lib.illume_scene_load_json_string(None, j.encode(), str(tmp_path).encode(), ctypes.byref(h))
    assert st == C.ERR_IO
    assert b"nope.obj" in native_lib.illume_last_error()


def test_missing_scene_file(native_lib):
    st, h = load_host("/nonexistent/scene.json")
    assert st == C.ERR_IO


def test_unknown_material_name_is_a_black_absorber(native_lib):
    j = ('{"materials": [{"name": "a", "type": "lambert", "albedo": [1,1,1]}],'
         ' "primitives": [{"type": "sphere", "center": [0,0,0], "radius": 1, "material": "zzz"}],'
         ' "camera": {"transform": {"translation": [0,0,-5]}, "fov": 40, "depth_of_field": 1, "aperture_radius": 0}}')
    h = ctypes.c_void_p()
    assert native_lib.illume_scene_load_json_string(None, j.encode(), None, ctypes.byref(h)) == C.OK
    d = C.SceneDesc()
    native_lib.illume_scene_describe(h, ctypes.byref(d))
    m = d.sphere_material[0]
    assert d.mat_type[m] == C.MAT_EMISSIVE
    t = d.mat_albedo_tex[m]
    assert [d.tex_color[3 * t + c] for c in range(3)] == [0, 0, 0]
    native_lib.illume_scene_destroy(h)


def test_invalid_descriptions_are_rejected(native_lib):
    from illume_gb300.scenedata import Mesh, SceneData, Material
    s = SceneData()
    mi = s.add_mesh(Mesh(np.zeros((3, 3), np.float32), np.array([[0, 1, 5]], np.int32)))   # index 5 out of range
    m = s.add_material(Material(C.MAT_LAMBERT, s.constant((1, 1, 1)), s.constant((0, 0, 0))))
    s.add_instance(mi, m)
    desc, keep = s.to_desc()
    h = ctypes.c_void_p()
    assert native_lib.illume_scene_create(None, ctypes.byref(desc), ctypes.byref(h)) == C.ERR_INVALID
    s.meshes[0].tris[:] = [[0, 1, 2]]
    s.instances[0] = (0, 7) + s.instances[0][2:]                                          # material 7 missing
    desc, keep = s.to_desc()
    assert native_lib.illume_scene_create(None, ctypes.byref(desc), ctypes.byref(h)) == C.ERR_INVALID


def test_null_arguments(native_lib):
    assert native_lib.illume_scene_create(None, None, None) == C.ERR_INVALID
    assert native_lib.illume_renderer_create(None, None, None, None) == C.ERR_INVALID
    assert native_lib.illume_render(None, None, None, None, None, None) == C.ERR_INVALID
    assert native_lib.illume_trace_closest(None, None, None, 0, 0, 0, None) == C.ERR_INVALID


def test_bitmap_roundtrip_png(native_lib, tmp_path):
    import struct
    import zlib
    b = native_lib.illume_bitmap_new(5, 3)
    px = np.ctypeslib.as_array(b.contents.pixels, shape=(15,))
    vals = np.arange(45).reshape(15, 3) * 5
    px["red"], px["green"], px["blue"] = vals[:, 0], vals[:, 1], vals[:, 2]
    path = str(tmp_path / "x.png")
    assert native_lib.illume_bitmap_save_png(b, path.encode()) == C.OK
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
            assert (w, h) == (5, 3)
        if typ == b"IDAT":
            idat += body
        pos += 12 + n
    got = unfilter_rgb8(zlib.decompress(idat), 5, 3).reshape(15, 3)
    assert np.array_equal(got, vals.astype(np.uint8))
    native_lib.illume_bitmap_free(b)


def unfilter_rgb8(raw, w, h):
    """Scanlines of an 8-bit RGB PNG (a filter byte, then 3w bytes) back to pixels
    (ISO 15948 9.2: none, sub, up, average, Paeth)."""
    stride = 3 * w
    assert len(raw) == h * (stride + 1)
    out = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        cur = np.zeros(stride, np.int32)
        if f in (0, 2):
            cur = (line + (prev if f == 2 else 0)) & 255
        else:
            for i in range(stride):
                a = cur[i - 3] if i >= 3 else 0
                b = prev[i]
                c = prev[i - 3] if i >= 3 else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) >> 1
                else:
                    q = a + b - c
                    pa, pb, pc = abs(q - a), abs(q - b), abs(q - c)
                    p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                cur[i] = (line[i] + p) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, 3).astype(np.uint8)


def _save_png(native_lib, img, path):
    h, w, _ = img.shape
    b = native_lib.illume_bitmap_new(w, h)
    px = np.ctypeslib.as_array(b.contents.pixels, shape=(w * h,))
    px["red"], px["green"], px["blue"] = img[..., 0].reshape(-1), img[..., 1].reshape(-1), img[..., 2].reshape(-1)
    assert native_lib.illume_bitmap_save_png(b, path.encode()) == C.OK
    native_lib.illume_bitmap_free(b)
    return open(path, "rb").read()


def _idat(data):
    import struct
    pos, idat = 8, b""
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        if data[pos + 4:pos + 8] == b"IDAT":
            idat += data[pos + 8:pos + 8 + n]
        pos += 12 + n
    return idat


@pytest.mark.parametrize("case", ["1x1", "odd", "flat", "noise", "gradient", "multi_segment"])
def test_png_writer_compresses_and_round_trips(native_lib, tmp_path, case):
    """The PNG writer's own deflate encoder (dynamic Huffman blocks, LZ77 over a 32 KB
    window, images over 512 KB of scanlines cut into segments joined by empty stored
    blocks) and adaptive row filters: Python's zlib and the library's own PNG decoder give
    back the pixels; smooth images shrink; the same image gives the same bytes."""
    import zlib
    from test_png import load
    rng = np.random.default_rng(5)
    img = {"1x1": rng.integers(0, 256, (1, 1, 3)),
           "odd": rng.integers(0, 256, (7, 13, 3)),
           "flat": np.full((64, 80, 3), 77),
           "noise": rng.integers(0, 256, (100, 77, 3)),
           "gradient": np.stack(np.meshgrid(np.arange(300) % 256, np.arange(200) % 256), -1)[..., [0, 1, 0]],
           "multi_segment": np.concatenate([np.full((250, 700, 3), 9), rng.integers(0, 256, (250, 700, 3))])}[case]
    img = np.asarray(img, np.uint8)
    h, w, _ = img.shape
    data = _save_png(native_lib, img, str(tmp_path / "a.png"))
    assert data == _save_png(native_lib, img, str(tmp_path / "b.png"))
    assert np.array_equal(unfilter_rgb8(zlib.decompress(_idat(data)), w, h), img)
    tex = load(tmp_path, "a.png")
    assert np.array_equal(np.asarray(tex.texels)[..., :3].reshape(h, w, 3), img.astype(np.float32))
    if case in ("flat", "gradient"):
        assert len(data) < 0.05 * img.size, len(data)
    if case == "noise":
        assert len(data) < 1.02 * img.size + 200, len(data)


def test_context_without_gpu_fails_cleanly(native_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    st = native_lib.illume_context_create(0, 0, ctypes.byref(h))
    assert st in (C.ERR_CUDA, C.ERR_INVALID)
    assert not h
