"""Python binding of the reference renderer built for the host (oracle/_ref/libillume_ref.so).

TEST INFRASTRUCTURE: used to pin the oracle and to generate tests/golden/ fixtures in the
build container, where the reference sources exist, and by the bench's reference arm
(built there from the staged copy of the sources, build_ref.stage()). available() is
False where there is no checkout; the product never uses it.
"""
from __future__ import annotations

import contextlib
import ctypes
import os
import sys
from ctypes import POINTER, c_char_p, c_float, c_int, c_longlong, c_uint32, c_void_p

import numpy as np

from illume_gb300 import _capi as C
from illume_gb300.scenedata import SceneData
from . import build_ref

_LIB = None


def available() -> bool:
    return build_ref.available()


@contextlib.contextmanager
def quiet():
    """Silence the reference's printf output (fd 1) during a call."""
    sys.stdout.flush()
    libc = ctypes.CDLL(None)
    libc.fflush(None)
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    try:
        yield
    finally:
        libc.fflush(None)   # the reference's printf output still in the C library's buffer
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)


def lib(staged: bool = False):
    """The loaded library; staged=True lets it be built from the staged copy of the
    reference sources where there is no checkout (the bench's reference arm)."""
    global _LIB
    if _LIB is None:
        path = build_ref.build(staged=staged)
        if path is None:
            raise RuntimeError("reference sources are not available here")
        L = ctypes.CDLL(path)
        fp = POINTER(c_float)
        L.ref_scene_load.restype = c_void_p
        L.ref_scene_load.argtypes = [c_char_p, c_char_p]
        L.ref_scene_set_env.argtypes = [c_void_p, fp, c_int, c_int]
        L.ref_scene_info.argtypes = [c_void_p, POINTER(c_int), POINTER(c_int), fp]
        L.ref_scene_free.argtypes = [c_void_p]
        L.ref_scene_export.argtypes = [c_void_p, POINTER(C.SceneDesc)]
        L.ref_render.restype = c_longlong
        L.ref_render.argtypes = [c_void_p, c_int, c_int, c_int, c_int, c_int, c_uint32, c_uint32, c_float, c_int,
                                 fp, fp, c_int]
        L.ref_tonemap_image.argtypes = [c_void_p, fp, c_int, c_float, c_int, POINTER(ctypes.c_uint8)]
        L.ref_closest_hit.argtypes = [c_void_p, fp, c_int, fp, POINTER(ctypes.c_int), fp]
        L.ref_camera_rays.argtypes = [c_void_p, c_int, c_int, c_uint32, c_uint32, c_uint32, fp]
        L.ref_fresnel_dielectric.restype = c_float
        L.ref_fresnel_dielectric.argtypes = [c_float, c_float, fp]
        L.ref_fresnel_conductor1.restype = c_float
        L.ref_fresnel_conductor1.argtypes = [c_float, c_float, c_float]
        L.ref_diffuse_fresnel.restype = c_float
        L.ref_diffuse_fresnel.argtypes = [c_float, c_int]
        L.ref_D_beckmann.restype = c_float
        L.ref_D_beckmann.argtypes = [fp, fp, c_float]
        L.ref_G_beckmann.restype = c_float
        L.ref_G_beckmann.argtypes = [fp, fp, fp, c_float]
        L.ref_sample_beckmann.argtypes = [c_float, c_float, c_float, fp]
        for n in ("ref_sample_hemisphere_cosine", "ref_sample_circle", "ref_sample_sphere"):
            getattr(L, n).argtypes = [c_float, c_float, fp]
        L.ref_sample_hg.argtypes = [c_float, c_float, c_float, fp]
        L.ref_to_basis.argtypes = [fp, fp, fp]
        L.ref_triangle_intersect.restype = c_float
        L.ref_triangle_intersect.argtypes = [fp, fp, fp, fp, fp, fp, fp]
        L.ref_aabb_intersect.restype = c_float
        L.ref_aabb_intersect.argtypes = [fp, fp, fp, fp]
        L.ref_sphere_intersect.restype = c_int
        L.ref_sphere_intersect.argtypes = [fp, c_float, fp, fp, fp, fp, fp]
        L.ref_tonemap_eval.argtypes = [c_int, fp, fp]
        L.ref_transform_from_json.argtypes = [c_char_p, fp, fp, fp]
        L.ref_texture_eval.restype = c_int
        L.ref_texture_eval.argtypes = [c_char_p, c_float, c_float, fp]
        L.ref_medium_from_json.argtypes = [c_char_p, fp, fp, fp, POINTER(c_int)]
        L.ref_material_from_json.restype = c_int
        L.ref_material_from_json.argtypes = [c_char_p, fp, fp, fp, fp, fp, fp]
        _LIB = L
    return _LIB


def _fp(a):
    return a.ctypes.data_as(POINTER(c_float))


class RefScene:
    """A scene loaded by the reference's HostScene + SceneRef on the host."""

    def __init__(self, json_name: str, work_dir: str | None = None, staged: bool = False):
        work = work_dir or build_ref.prepare_work_dir()
        L = lib(staged)
        with quiet():
            self.handle = L.ref_scene_load(json_name.encode(), work.encode())
        if not self.handle:
            raise RuntimeError(f"reference could not load {json_name}")
        w, h, b = c_int(), c_int(), c_float()
        lib().ref_scene_info(self.handle, ctypes.byref(w), ctypes.byref(h), ctypes.byref(b))
        self.width, self.height, self.ray_bias = w.value, h.value, b.value

    def close(self):
        if self.handle:
            lib().ref_scene_free(self.handle)
            self.handle = None

    def set_env(self, rgba: np.ndarray):
        rgba = np.ascontiguousarray(rgba, dtype=np.float32)
        lib().ref_scene_set_env(self.handle, _fp(rgba), rgba.shape[1], rgba.shape[0])

    def export(self) -> SceneData:
        d = C.SceneDesc()
        lib().ref_scene_export(self.handle, ctypes.byref(d))
        return SceneData.from_desc(d)

    def render(self, width, height, spp, max_depth, sample_begin=0, seed=0, job=0, ray_bias=None, nthreads=0):
        n = width * height
        s = np.zeros(n * 3, np.float32)
        s2 = np.zeros(n * 3, np.float32)
        use = ray_bias is not None
        with quiet():
            rays = lib().ref_render(self.handle, width, height, spp, sample_begin, max_depth, seed, job,
                                    float(ray_bias or 0.0), int(use), _fp(s), _fp(s2), nthreads)
        return s.reshape(n, 3), s2.reshape(n, 3), int(rays)

    def tonemap(self, sum_rgb, samples, op=-1):
        s = np.ascontiguousarray(sum_rgb, dtype=np.float32).reshape(-1, 3)
        out = np.zeros(s.shape, np.uint8)
        lib().ref_tonemap_image(self.handle, _fp(s), s.shape[0], samples, op, out.ctypes.data_as(POINTER(ctypes.c_uint8)))
        return out

    def closest_hit(self, rays6):
        rays6 = np.ascontiguousarray(rays6, dtype=np.float32)
        n = rays6.shape[0]
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        nrm = np.zeros((n, 3), np.float32)
        lib().ref_closest_hit(self.handle, _fp(rays6), n, _fp(t), prim.ctypes.data_as(POINTER(ctypes.c_int)), _fp(nrm))
        return t, prim, nrm

    def camera_rays(self, W, H, sample=0, seed=0, job=0):
        out = np.zeros((W * H, 6), np.float32)
        lib().ref_camera_rays(self.handle, W, H, sample, seed, job, _fp(out))
        return out
