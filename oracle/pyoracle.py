"""Python binding of the oracle (CPU restatement of illume's path tracer, oracle/oracle.h).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, as the checker. The product package never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_int32, c_int64, c_uint32, c_void_p

import numpy as np

from illume_gb300 import _capi as C
from illume_gb300.scenedata import SceneData

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
SOURCES = [os.path.join(HERE, f) for f in ("oracle_capi.cpp", "oracle.h", "philox.h")]


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (IEEE float semantics: no contraction, no fast-math)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "..", "include", "illume.h")])
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", LIB_PATH, os.path.join(HERE, "oracle_capi.cpp")]
    subprocess.run(cmd, check=True)
    return LIB_PATH


class RenderArgs(ctypes.Structure):
    _fields_ = [("width", c_int32), ("height", c_int32), ("max_depth", c_int32), ("ray_bias", c_float),
                ("seed", c_uint32), ("job", c_uint32), ("isect", c_int32), ("exact_hg", c_int32),
                ("spp", c_int32), ("sample_begin", c_int32), ("precision", c_int32), ("num_pixels", c_int32),
                ("pixels", POINTER(c_int32)), ("nthreads", c_int32), ("nee", c_int32)]


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        fp = POINTER(c_float)
        L.oracle_scene_create.restype = c_void_p
        L.oracle_scene_create.argtypes = [POINTER(C.SceneDesc)]
        L.oracle_scene_destroy.argtypes = [c_void_p]
        L.oracle_closest_hit.argtypes = [c_void_p, fp, c_int, c_int, POINTER(C.Hit), c_int]
        L.oracle_closest_hit_brute.argtypes = [c_void_p, fp, c_int, c_int, POINTER(C.Hit), c_int]
        L.oracle_camera_rays.argtypes = [c_void_p, c_int, c_int, c_uint32, c_uint32, c_uint32, fp]
        L.oracle_render.restype = c_int64
        L.oracle_render.argtypes = [c_void_p, POINTER(RenderArgs), POINTER(c_double), POINTER(c_double)]
        L.oracle_tonemap_image.argtypes = [fp, c_int, c_float, c_int, POINTER(ctypes.c_uint8)]
        L.oracle_philox.argtypes = [POINTER(c_uint32), POINTER(c_uint32), POINTER(c_uint32)]
        L.oracle_bsdf_batch.argtypes = [c_int, c_int, fp, c_int, fp, c_int]
        L.oracle_texture_eval.argtypes = [c_void_p, c_int, c_float, c_float, fp]
        for name in ("oracle_fresnel_dielectric",):
            getattr(L, name).restype = c_float
            getattr(L, name).argtypes = [c_float, c_float, fp]
        L.oracle_fresnel_dielectric_d.restype = c_double
        L.oracle_fresnel_dielectric_d.argtypes = [c_double, c_double, POINTER(c_double)]
        L.oracle_fresnel_conductor1.restype = c_float
        L.oracle_fresnel_conductor1.argtypes = [c_float, c_float, c_float]
        L.oracle_diffuse_fresnel.restype = c_float
        L.oracle_diffuse_fresnel.argtypes = [c_float, c_int]
        L.oracle_D_beckmann.restype = c_float
        L.oracle_D_beckmann.argtypes = [fp, fp, c_float]
        L.oracle_G_beckmann.restype = c_float
        L.oracle_G_beckmann.argtypes = [fp, fp, fp, c_float]
        for name in ("oracle_sample_beckmann",):
            getattr(L, name).argtypes = [c_float, c_float, c_float, fp]
        for name in ("oracle_sample_hemisphere_cosine", "oracle_sample_circle", "oracle_sample_sphere"):
            getattr(L, name).argtypes = [c_float, c_float, fp]
        L.oracle_sample_hg.argtypes = [c_float, c_float, c_float, c_int, fp]
        L.oracle_to_basis.argtypes = [fp, fp, fp]
        for name in ("oracle_triangle_mt", "oracle_triangle_watertight"):
            getattr(L, name).restype = c_float
            getattr(L, name).argtypes = [fp, fp, fp, fp, fp, fp, fp]
        L.oracle_aabb_intersect.restype = c_float
        L.oracle_aabb_intersect.argtypes = [fp, fp, fp, fp]
        L.oracle_sphere_intersect.restype = c_int
        L.oracle_sphere_intersect.argtypes = [fp, c_float, fp, fp, fp, fp, fp]
        L.oracle_tonemap_eval.argtypes = [c_int, fp, fp]
        L.oracle_alias_build.argtypes = [POINTER(c_double), c_int, fp, POINTER(c_int32)]
        L.oracle_light_info.argtypes = [c_void_p, POINTER(c_int32), fp, POINTER(c_int32)]
        _LIB = L
    return _LIB


def _fp(a):
    return a.ctypes.data_as(POINTER(c_float))


class OracleScene:
    """Oracle-side copy of a SceneData (builds the oracle's own BVHs)."""

    def __init__(self, scene: SceneData):
        self.scene = scene
        self._desc, self._keep = scene.to_desc()
        self.handle = lib().oracle_scene_create(ctypes.byref(self._desc))

    def __del__(self):
        if getattr(self, "handle", None) and _LIB is not None:
            _LIB.oracle_scene_destroy(self.handle)
            self.handle = None

    def closest_hit(self, rays8: np.ndarray, isect: int = C.ISECT_WATERTIGHT, brute: bool = False, nthreads: int = 0):
        rays8 = np.ascontiguousarray(rays8, dtype=np.float32)
        n = rays8.shape[0]
        hits = (C.Hit * n)()
        fn = lib().oracle_closest_hit_brute if brute else lib().oracle_closest_hit
        fn(self.handle, _fp(rays8), n, isect, hits, nthreads)
        return hits_to_numpy(hits)

    def camera_rays(self, W, H, sample=0, seed=0, job=0):
        out = np.zeros((W * H, 6), np.float32)
        lib().oracle_camera_rays(self.handle, W, H, sample, seed, job, _fp(out))
        return out

    def render(self, width, height, spp, max_depth, ray_bias=None, seed=0, job=0, isect=C.ISECT_WATERTIGHT,
               exact_hg=0, sample_begin=0, precision=32, pixels=None, nthreads=0, nee=0):
        """Per-pixel sum and sum of squares of per-sample radiance (float64), and rays traced
        (nee=1: the next-event estimator; shadow rays count as rays)."""
        a = RenderArgs()
        a.width, a.height, a.max_depth = width, height, max_depth
        a.ray_bias = self.scene.ray_bias if ray_bias is None else ray_bias
        a.seed, a.job, a.isect, a.exact_hg = seed, job, isect, exact_hg
        a.spp, a.sample_begin, a.precision = spp, sample_begin, precision
        a.nthreads = nthreads
        a.nee = nee
        pix = None
        if pixels is not None:
            pix = np.ascontiguousarray(pixels, dtype=np.int32)
            a.num_pixels = pix.size
            a.pixels = pix.ctypes.data_as(POINTER(c_int32))
        n = pix.size if pix is not None else width * height
        s = np.zeros((n, 3), np.float64)
        s2 = np.zeros((n, 3), np.float64)
        rays = lib().oracle_render(self.handle, ctypes.byref(a), s.ctypes.data_as(POINTER(c_double)),
                                   s2.ctypes.data_as(POINTER(c_double)))
        return s, s2, int(rays)

    def light_info(self):
        """(env_w, env_h, env_integral, env_prob, number of emissive triangles)."""
        wh = (c_int32 * 2)()
        fp2 = np.zeros(2, np.float32)
        nt = c_int32()
        lib().oracle_light_info(self.handle, wh, _fp(fp2), ctypes.byref(nt))
        return int(wh[0]), int(wh[1]), float(fp2[0]), float(fp2[1]), int(nt.value)

    def texture_eval(self, tex, u, v):
        out = np.zeros(3, np.float32)
        lib().oracle_texture_eval(self.handle, tex, u, v, _fp(out))
        return out


def hits_to_numpy(hits):
    a = np.ctypeslib.as_array(hits)
    return {k: a[k].copy() for k in ("t", "u", "v", "inst", "prim", "sphere")}


def tonemap_image(sum_rgb: np.ndarray, samples: float, op: int) -> np.ndarray:
    s = np.ascontiguousarray(sum_rgb, dtype=np.float32).reshape(-1, 3)
    out = np.zeros(s.shape, np.uint8)
    lib().oracle_tonemap_image(_fp(s), s.shape[0], samples, op, out.ctypes.data_as(POINTER(ctypes.c_uint8)))
    return out


def philox(ctr, key):
    c = (c_uint32 * 4)(*ctr)
    k = (c_uint32 * 2)(*key)
    o = (c_uint32 * 4)()
    lib().oracle_philox(c, k, o)
    return list(o)


def bsdf_batch(material_type: int, distribution: int, inputs: np.ndarray, precision: int = 64) -> np.ndarray:
    x = np.ascontiguousarray(inputs, dtype=np.float32).reshape(-1, 16)
    y = np.zeros_like(x)
    lib().oracle_bsdf_batch(material_type, distribution, _fp(x), x.shape[0], _fp(y), precision)
    return y


def alias_table(weights):
    """The oracle's alias table of the weights: (probabilities, aliases)."""
    w = np.ascontiguousarray(weights, dtype=np.float64)
    n = w.size
    prob = np.zeros(n, np.float32)
    alias = np.zeros(n, np.int32)
    lib().oracle_alias_build(w.ctypes.data_as(POINTER(c_double)), n, _fp(prob), alias.ctypes.data_as(POINTER(c_int32)))
    return prob, alias
