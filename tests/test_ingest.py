"""Scene ingest on CPU (host-only scenes, no GPU): the product's JSON/OBJ loader against
the reference's own parse of the same files (tests/golden/ref_*.npz)."""
import ctypes
import json
import re
import os
import struct

import numpy as np
import pytest

from conftest import SCENES, golden, golden_scene
from illume_gb300 import _capi as C
from illume_gb300.scenedata import SceneData


def host_scene_from_json(text, base=None):
    h = ctypes.c_void_p()
    st = C.lib().illume_scene_load_json_string(None, text.encode(), base.encode() if base else None, ctypes.byref(h))
    assert st == C.OK, C.lib().illume_last_error()
    d = C.SceneDesc()
    C.lib().illume_scene_describe(h, ctypes.byref(d))
    sd = SceneData.from_desc(d)
    C.lib().illume_scene_destroy(h)
    return sd


CAM = {"transform": {"translation": [0, 0, -5]}, "fov": 40, "depth_of_field": 1, "aperture_radius": 0}


@pytest.mark.parametrize("name", ["box", "materials", "mesh", "textured"])
def test_scene_files_parse_like_the_reference(native_lib, name):
    sd = host_scene_from_json(open(os.path.join(SCENES, name + ".json")).read(), SCENES)
    ref = golden_scene(name)
    assert len(sd.meshes) == len(ref.meshes)
    for a, b in zip(sd.meshes, ref.meshes):
        assert np.array_equal(a.positions, b.positions)
        assert np.array_equal(a.tris, b.tris)
        assert (a.normals is None) == (b.normals is None)
        if a.normals is not None:
            assert np.array_equal(a.normals, b.normals)
        assert (a.texcoords is None) == (b.texcoords is None)
        if a.texcoords is not None:
            assert np.array_equal(a.texcoords, b.texcoords)
    assert len(sd.instances) == len(ref.instances)
    for a, b in zip(sd.instances, ref.instances):
        assert a[0] == b[0]
        for k in (2, 3, 4):
            assert np.array_equal(a[k], b[k])
    assert len(sd.spheres) == len(ref.spheres)
    for a, b in zip(sd.spheres, ref.spheres):
        assert a[0] == b[0] and a[1] == b[1]
    # materials are compared through what they resolve to (textures are shared or not)
    from oracle import pyoracle
    osa, osb = pyoracle.OracleScene(sd), pyoracle.OracleScene(ref)
    prims_a = [x[1] for x in sd.spheres] + [x[1] for x in sd.instances]
    prims_b = [x[2] for x in ref.spheres] + [x[1] for x in ref.instances]
    prims_a = [x[2] for x in sd.spheres] + [x[1] for x in sd.instances]
    rng = np.random.default_rng(0)
    uvs = rng.random((16, 2)).astype(np.float32)
    for ma, mb in zip(prims_a, prims_b):
        A, B = sd.materials[ma], ref.materials[mb]
        assert A.type == B.type
        if A.type not in (C.MAT_CONDUCTOR, C.MAT_ROUGHCONDUCTOR):
            for u, v in uvs:
                assert np.array_equal(osa.texture_eval(A.albedo_tex, u, v), osb.texture_eval(B.albedo_tex, u, v))
        if A.type in (C.MAT_ROUGHREFLECTIVE, C.MAT_ROUGHREFRACTIVE, C.MAT_ROUGHCONDUCTOR):
            for u, v in uvs:
                assert np.array_equal(osa.texture_eval(A.roughness_tex, u, v), osb.texture_eval(B.roughness_tex, u, v))
        assert A.ior == B.ior or A.type in (C.MAT_EMISSIVE, C.MAT_LAMBERT, C.MAT_REFLECTIVE, C.MAT_CONDUCTOR,
                                            C.MAT_ROUGHCONDUCTOR)
        assert np.float32(A.diffuse_fresnel) == np.float32(B.diffuse_fresnel)
        assert A.eta == B.eta and A.k == B.k
        if A.medium >= 0 or B.medium >= 0:
            assert sd.mediums[A.medium] == ref.mediums[B.medium]
    assert np.array_equal(sd.camera_transform, ref.camera_transform)
    assert (sd.camera_fov, sd.camera_dof, sd.camera_aperture) == (ref.camera_fov, ref.camera_dof, ref.camera_aperture)
    assert (sd.width, sd.height, sd.ray_bias, sd.tonemapper) == (ref.width, ref.height, ref.ray_bias, ref.tonemapper)
    if ref.env_tex >= 0:
        assert np.array_equal(osa.texture_eval(sd.env_tex, 0.3, 0.6), osb.texture_eval(ref.env_tex, 0.3, 0.6))


def test_transforms(native_lib):
    z = golden("ref_json.npz")
    for js, want in zip(z["transforms_json"], z["transforms"]):
        sc = {"meshes": [{"file": "quad.obj", "name": "q"}],
              "materials": [{"name": "m", "type": "lambert", "albedo": [1, 1, 1]}],
              "primitives": [{"type": "mesh_instance", "mesh": "q", "material": "m", "transform": json.loads(str(js))}],
              "camera": {"transform": json.loads(str(js)), "fov": 40, "depth_of_field": 1, "aperture_radius": 0}}
        sd = host_scene_from_json(json.dumps(sc), SCENES)
        mat, inv, tinv = (want[k].reshape(4, 4)[:3] for k in range(3))
        assert np.array_equal(sd.instances[0][2], mat), js
        assert np.array_equal(sd.instances[0][3], inv), js
        assert np.array_equal(sd.instances[0][4], tinv), js
        assert np.array_equal(sd.camera_transform, mat), js


def test_materials_and_mediums(native_lib):
    z = golden("ref_json.npz")
    for js, row in zip(z["materials_json"], z["materials"]):
        m = json.loads(str(js))
        m["name"] = "m"
        sc = {"materials": [m], "primitives": [{"type": "sphere", "center": [0, 0, 0], "radius": 1, "material": "m"}],
              "camera": CAM}
        sd = host_scene_from_json(json.dumps(sc))
        mat = sd.materials[sd.spheres[0][2]]
        typ, ior, dfr = int(row[0]), row[1], row[2]
        want_type = typ if m["type"] != "diffuse" else C.MAT_LAMBERT
        assert mat.type == want_type, js
        if typ in (C.MAT_REFRACTIVE, C.MAT_ROUGHREFLECTIVE, C.MAT_ROUGHREFRACTIVE, C.MAT_PLASTIC):
            assert np.float32(mat.ior) == ior
        assert np.float32(mat.diffuse_fresnel) == dfr, js
        assert np.array_equal(np.float32(mat.eta), row[3:6]) and np.array_equal(np.float32(mat.k), row[6:9]), js
        albedo = np.float32(sd.textures[mat.albedo_tex].color)
        assert np.array_equal(albedo, row[9:12]), js
        if typ in (C.MAT_ROUGHREFLECTIVE, C.MAT_ROUGHREFRACTIVE, C.MAT_ROUGHCONDUCTOR):
            assert np.array_equal(np.float32(sd.textures[mat.roughness_tex].color), row[12:15]), js
    for js, row in zip(z["mediums_json"], z["mediums"]):
        m = json.loads(str(js))
        m["name"] = "med"
        sc = {"mediums": [m], "materials": [{"name": "g", "type": "refractive", "ior": 1.3, "medium": "med"}],
              "primitives": [{"type": "sphere", "center": [0, 0, 0], "radius": 1, "material": "g"}], "camera": CAM}
        sd = host_scene_from_json(json.dumps(sc))
        mat = sd.materials[sd.spheres[0][2]]
        absorption, scattering, g, active = sd.mediums[mat.medium]
        assert np.array_equal(np.float32(absorption), row[:3])
        assert np.float32(scattering) == row[3] and np.float32(g) == row[4] and active == int(row[5])


def test_textures(native_lib):
    from oracle import pyoracle
    z = golden("ref_json.npz")
    for k, js in enumerate(z["textures_json"]):
        sc = {"materials": [{"name": "m", "type": "lambert", "albedo": json.loads(str(js))}],
              "primitives": [{"type": "sphere", "center": [0, 0, 0], "radius": 1, "material": "m"}], "camera": CAM}
        sd = host_scene_from_json(json.dumps(sc))
        os_ = pyoracle.OracleScene(sd)
        tex = sd.materials[sd.spheres[0][2]].albedo_tex
        got = np.array([os_.texture_eval(tex, u, v) for u, v in z["texture_uv"]])
        assert np.array_equal(got, z["textures"][k]), js


def test_bitmap_texture_files(native_lib, tmp_path):
    rng = np.random.default_rng(1)
    img = rng.random((5, 7, 3)).astype(np.float32) * 4
    # PFM (bottom-up rows)
    with open(tmp_path / "t.pfm", "wb") as f:
        f.write(b"PF\n7 5\n-1.0\n")
        f.write(img[::-1].astype("<f4").tobytes())
    # PPM
    rgb8 = (rng.random((4, 6, 3)) * 255).astype(np.uint8)
    with open(tmp_path / "t.ppm", "wb") as f:
        f.write(b"P6\n# comment\n6 4\n255\n" + rgb8.tobytes())
    # Radiance HDR, flat scanlines
    e = np.array([[[128, 64, 32, 129], [255, 0, 1, 120]]], np.uint8)
    with open(tmp_path / "t.hdr", "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 1 +X 2\n" + e.tobytes())
    for name in ("t.pfm", "t.ppm", "t.hdr"):
        sc = {"materials": [{"name": "m", "type": "lambert", "albedo": {"type": "bitmap", "file": name}}],
              "primitives": [{"type": "sphere", "center": [0, 0, 0], "radius": 1, "material": "m"}], "camera": CAM}
        sd = host_scene_from_json(json.dumps(sc), str(tmp_path))
        t = sd.textures[sd.materials[0].albedo_tex]
        assert t.type == C.TEX_BITMAP, name
        if name == "t.pfm":
            assert t.hdr == 1 and np.array_equal(t.texels[..., :3], img)
        elif name == "t.ppm":
            assert t.hdr == 0 and np.array_equal(t.texels[..., :3], rgb8.astype(np.float32))
        else:
            want = e[0, :, :3].astype(np.float64) * np.ldexp(1.0, e[0, :, 3].astype(int) - 136)[:, None]
            assert np.allclose(t.texels[0, :, :3], want)


def test_missing_bitmap_becomes_black_like_the_reference(native_lib):
    sc = {"materials": [{"name": "m", "type": "lambert", "albedo": {"type": "bitmap", "file": "none.png"}}],
          "primitives": [{"type": "sphere", "center": [0, 0, 0], "radius": 1, "material": "m"}], "camera": CAM}
    sd = host_scene_from_json(json.dumps(sc))
    t = sd.textures[sd.materials[0].albedo_tex]
    assert t.type == C.TEX_CONSTANT and t.color == (0.0, 0.0, 0.0)


def test_obj_variants(native_lib, tmp_path):
    obj = ("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\nvt 0 0\nvt 1 0\nvt 0 1\nvn 0 0 2\nvn 0 3 0\n"
           "f 1/1/1 2/2/1 3/3/1\nf 1//2 2//2 4//2\nf 1 3 4 2\n")
    (tmp_path / "m.obj").write_text(obj)
    for opts, ntri in (({}, 3), ({"z_up": True}, 3)):
        sc = {"meshes": [dict(file="m.obj", name="m", **opts)],
              "materials": [{"name": "a", "type": "lambert", "albedo": [1, 1, 1]}],
              "primitives": [{"type": "mesh_instance", "mesh": "m", "material": "a", "transform": {}}], "camera": CAM}
        sd = host_scene_from_json(json.dumps(sc), str(tmp_path))
        m = sd.meshes[0]
        assert len(m.tris) == ntri
        if opts.get("z_up"):
            assert np.array_equal(m.positions[3], [0, 1, 0])
    # vertex normals requested but a face has none: an error, not an out-of-range read
    sc["meshes"] = [{"file": "m.obj", "name": "m", "face_normals": False}]
    h = ctypes.c_void_p()
    st = C.lib().illume_scene_load_json_string(None, json.dumps(sc).encode(), str(tmp_path).encode(), ctypes.byref(h))
    assert st != C.OK and b"normal index" in C.lib().illume_last_error()
    (tmp_path / "n.obj").write_text(obj.rsplit("f 1 3 4 2", 1)[0])
    sc["meshes"] = [{"file": "n.obj", "name": "m", "face_normals": False}]
    sd = host_scene_from_json(json.dumps(sc), str(tmp_path))
    assert sd.meshes[0].normals is not None
    assert np.allclose(np.linalg.norm(sd.meshes[0].normals, axis=1), 1.0)


_FLOAT_PREFIX = re.compile(r"^\s*[+-]?(\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?)")
_INT_PREFIX = re.compile(r"^\s*[+-]?\d+")


def _strtof(tok):
    m = _FLOAT_PREFIX.match(tok)
    return np.float32(float(m.group(0))) if m else np.float32(0.0)


def _strtol(tok):
    m = _INT_PREFIX.match(tok)
    return int(m.group(0)) if m else 0


def _obj_expected(text, face_normals=True, has_texcoords=False):
    """The loader's rules restated (mesh.cu:159-340 via load_obj_mesh): lines split on
    newlines with one trailing CR dropped, fields on single spaces with empty ones dropped
    (a tab stays inside its field), numbers read as strtof / strtol read a field's prefix,
    the first three corners of a face, corners p, p/t, p//n or p/t/n with empty fields
    dropped, vertices merged by value (+0 equal to -0) in first-use order, each taking the
    values of its first corner. Normals in these cases are unit length already."""
    v, vt, vn, corners = [], [], [], []
    for line in text.split("\n"):
        if line.endswith("\r"):
            line = line[:-1]
        tok = [t for t in line.split(" ") if t]
        if not tok:
            continue
        fl = lambda k: _strtof(tok[k]) if k < len(tok) else np.float32(0.0)
        if tok[0] == "v":
            v.append((fl(1), fl(2), fl(3)))
        elif tok[0] == "vt":
            vt.append((fl(1), fl(2)))
        elif tok[0] == "vn":
            vn.append((fl(1), fl(2), fl(3)))
        elif tok[0] == "f":
            for t in tok[1:4]:
                parts = [x for x in t.split("/") if x]
                num = lambda k: _strtol(parts[k]) - 1 if k < len(parts) else -1
                slashes = t.count("/")
                c = [-1, -1, -1]
                if slashes == 0:
                    c = [num(0), -1, -1]
                elif slashes == 1:
                    c = [num(0), num(1), -1]
                elif slashes == 2:
                    c = [num(0), -1, num(1)] if "//" in t else [num(0), num(1), num(2)]
                corners.append(c)
    ids, pos, nrm, tex, tris = {}, [], [], [], []
    for p, t, n in corners:
        key = (v[p], vn[n] if not face_normals else None, vt[t] if has_texcoords else None)
        if key not in ids:
            ids[key] = len(ids)
            pos.append(v[p])
            if not face_normals:
                nrm.append(vn[n])
            if has_texcoords:
                tex.append(vt[t])
        tris.append(ids[key])
    as32 = lambda a, k: np.array(a, np.float32).reshape(-1, k)
    return as32(pos, 3), np.array(tris, np.int32).reshape(-1, 3), as32(nrm, 3), as32(tex, 2)


def test_obj_parser_rules(native_lib, tmp_path):
    text = ("# a comment\nv 0 0 0\nv -0 0 0\nv 1 0 0\r\nv  0   1  0\nv 0\t1 0\nv 2.5 -0 1e1\n"
            "vt 0.5 0.25\nvt 0.5 0.25\nvt 1 1\nvn 0 0 1\nvn 0 1 0\nvn 0 0 1\n"
            "f 2/1/1 3/2/3 4/3/1\nf 1/2/3 3/1/1 6/3/2\nf 5/1/1 6/2/2 4/3/3 2/1/1\n"
            "f 6//2 1//1 3//3\nf +1/1/1 3/2/1 4/3/1\n")
    (tmp_path / "r.obj").write_text(text)
    for opts in ({}, {"face_normals": False}, {"has_texcoords": True}, {"face_normals": False, "has_texcoords": True}):
        if opts.get("has_texcoords"):    # the "p//n" face has no texcoord: an error, checked below
            body = text.replace("f 6//2 1//1 3//3\n", "")
        else:
            body = text
        (tmp_path / "s.obj").write_text(body)
        sc = {"meshes": [dict(file="s.obj", name="m", **opts)],
              "materials": [{"name": "a", "type": "lambert", "albedo": [1, 1, 1]}],
              "primitives": [{"type": "mesh_instance", "mesh": "m", "material": "a", "transform": {}}], "camera": CAM}
        sd = host_scene_from_json(json.dumps(sc), str(tmp_path))
        m = sd.meshes[0]
        pos, tris, nrm, tex = _obj_expected(body, opts.get("face_normals", True), opts.get("has_texcoords", False))
        assert np.array_equal(m.tris, tris), opts
        assert np.array_equal(m.positions.view(np.uint32), pos.view(np.uint32)), opts   # signs of zeros too
        if not opts.get("face_normals", True):
            assert np.array_equal(m.normals, nrm), opts
        if opts.get("has_texcoords"):
            assert np.array_equal(m.texcoords, tex), opts
    sc["meshes"] = [{"file": "r.obj", "name": "m", "has_texcoords": True}]
    h = ctypes.c_void_p()
    st = C.lib().illume_scene_load_json_string(None, json.dumps(sc).encode(), str(tmp_path).encode(), ctypes.byref(h))
    assert st != C.OK and b"texcoord index" in C.lib().illume_last_error()


def test_bitmap_texels_and_environment_like_the_reference(native_lib):
    """The textured scene's .hdr (flat RGBE) and .png (gray, RGB, RGBA) bitmaps decode to
    the texels the reference's stb_image path gives (src/imageio.cpp, 4 channels), and
    the equirectangular environment evaluates identically over the whole uv square
    (bilinear HDR filtering with wrap addressing, src/texture.cu:146-152)."""
    from oracle import pyoracle
    sd = host_scene_from_json(open(os.path.join(SCENES, "textured.json")).read(), SCENES)
    ref = golden_scene("textured")
    bitmaps = lambda s: [t for t in s.textures if t.texels is not None]
    A, B = bitmaps(sd), bitmaps(ref)
    assert len(A) >= 4 and len(B) >= 4
    key = lambda t: (t.texels.shape, t.hdr, t.texels.tobytes())
    assert sorted(map(key, A)) == sorted(map(key, B))
    osa, osb = pyoracle.OracleScene(sd), pyoracle.OracleScene(ref)
    rng = np.random.default_rng(5)
    uvs = (rng.random((512, 2)) * 1.6 - 0.3).astype(np.float32)
    for u, v in uvs:
        assert np.array_equal(osa.texture_eval(sd.env_tex, u, v), osb.texture_eval(ref.env_tex, u, v))
