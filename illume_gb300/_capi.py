"""ctypes mirror of include/illume.h and the loader of the native library.

The library is loaded lazily from illume_gb300/_lib/libillume_gb300.so (built in-tree by
illume_gb300.build). There is no fallback: if the library is missing, every call raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_size_t, c_uint8, c_uint32, c_uint64, c_void_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libillume_gb300.so")

# status codes (enum illume_status)
OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_OOM = -3
ERR_IO = -4
ERR_PARSE = -5
ERR_BUDGET = -6
ERR_TIMEOUT = -7
ERR_CANCELLED = -8
ERR_UNSUPPORTED = -9
ERR_NOT_READY = -10
ERR_TRAVERSAL = -11

MAT_EMISSIVE, MAT_LAMBERT, MAT_REFLECTIVE, MAT_REFRACTIVE, MAT_ROUGHREFLECTIVE, MAT_ROUGHREFRACTIVE, \
    MAT_CONDUCTOR, MAT_ROUGHCONDUCTOR, MAT_PLASTIC = range(9)
TEX_CONSTANT, TEX_CHECKERBOARD, TEX_BITMAP = range(3)
DIST_BECKMANN, DIST_GGX = range(2)
TONE_LINEAR, TONE_REINHARD, TONE_FILMIC, TONE_UNCHARTED = range(4)
ISECT_MT, ISECT_WATERTIGHT = range(2)
BVH_BINARY, BVH_WIDE8, BVH_WIDE8_PERSISTENT, BVH_WIDE4 = range(4)
BVH_BUILD_HOST, BVH_BUILD_DEVICE = range(2)
ACCUM_FP32, ACCUM_KAHAN, ACCUM_FP64 = range(3)
ESTIMATOR_REFERENCE, ESTIMATOR_NEE = range(2)
(SERVER_PATH_CAPACITY, SERVER_PASSES_PER_STEP, SERVER_AUTOTUNE, SERVER_TRACE_VARIANT, SERVER_LANES,
 SERVER_QUEUE_SLOTS, SERVER_REGEN_THRESHOLD) = range(7)

_pi32 = POINTER(c_int32)
_pf = POINTER(c_float)


class SceneDesc(ctypes.Structure):
    """illume_scene_desc"""
    _fields_ = [
        ("num_meshes", c_int32),
        ("mesh_vertex_offset", _pi32), ("mesh_num_vertices", _pi32), ("mesh_tri_offset", _pi32),
        ("mesh_num_tris", _pi32), ("mesh_has_normals", _pi32), ("mesh_has_texcoords", _pi32),
        ("mesh_bvh_leaf_size", _pi32),
        ("positions", _pf), ("normals", _pf), ("texcoords", _pf), ("tris", _pi32),
        ("num_instances", c_int32),
        ("inst_mesh", _pi32), ("inst_material", _pi32), ("inst_mat", _pf), ("inst_inv", _pf), ("inst_trans_inv", _pf),
        ("num_spheres", c_int32),
        ("sphere_center_radius", _pf), ("sphere_material", _pi32),
        ("num_materials", c_int32),
        ("mat_type", _pi32), ("mat_albedo_tex", _pi32), ("mat_roughness_tex", _pi32), ("mat_medium", _pi32),
        ("mat_distribution", _pi32), ("mat_ior", _pf), ("mat_diffuse_fresnel", _pf), ("mat_eta", _pf), ("mat_k", _pf),
        ("num_mediums", c_int32),
        ("med_absorption", _pf), ("med_scattering", _pf), ("med_g", _pf), ("med_active", _pi32),
        ("num_textures", c_int32),
        ("tex_type", _pi32), ("tex_color", _pf), ("tex_off", _pf), ("tex_scale", _pf), ("tex_width", _pi32),
        ("tex_height", _pi32), ("tex_hdr", _pi32), ("tex_texel_offset", POINTER(c_int64)), ("texels", _pf),
        ("env_tex", c_int32),
        ("camera_transform", c_float * 12),
        ("camera_fov", c_float), ("camera_dof", c_float), ("camera_aperture", c_float),
        ("width", c_int32), ("height", c_int32),
        ("ray_bias", c_float),
        ("tonemapper", c_int32),
    ]


class RenderParams(ctypes.Structure):
    """illume_render_params"""
    _fields_ = [
        ("width", c_int32), ("height", c_int32), ("spp", c_int32), ("max_depth", c_int32),
        ("sample_begin", c_int32), ("ray_bias", c_float), ("tonemapper", c_int32),
        ("seed", c_uint32), ("job", c_uint32), ("accum_mode", c_int32), ("intersector", c_int32),
        ("bvh_kind", c_int32), ("exact_hg", c_int32), ("samples_per_pass", c_int32),
        ("camera", _pf), ("trace_variant", c_int32), ("shade_variant", c_int32), ("estimator", c_int32),
        ("engines", c_int32), ("queue_slots", c_int32), ("regen_threshold", c_float), ("ray_group", c_int32),
    ]


class RenderStats(ctypes.Structure):
    """illume_render_stats"""
    _fields_ = [
        ("rays", c_int64), ("paths", c_int64), ("render_ms", c_double), ("total_ms", c_double),
        ("kernel_launches", c_int64), ("h2d_bytes", c_int64), ("d2h_bytes", c_int64),
    ]


class Profile(ctypes.Structure):
    """illume_profile"""
    _fields_ = [("raygen_ms", c_double), ("trace_ms", c_double), ("shade_ms", c_double), ("accumulate_ms", c_double),
                ("trace_launches", c_int64), ("shade_launches", c_int64), ("rays", c_int64),
                ("node_fetches", c_int64), ("tri_tests", c_int64), ("node_bytes", c_int64), ("tri_bytes", c_int64),
                ("lane_slots", c_int64)]


class ServerStats(ctypes.Structure):
    """illume_server_stats"""
    _fields_ = [("rays", c_int64), ("passes", c_int64), ("kernel_launches", c_int64), ("jobs_done", c_int64),
                ("device_ms", c_double), ("path_capacity", c_int64), ("trace_variant", c_int32), ("tuned", c_int32),
                ("device_bytes", c_int64), ("queue_slots", c_int32), ("regen_threshold", c_float)]


class Hit(ctypes.Structure):
    """illume_hit"""
    _fields_ = [("t", c_float), ("u", c_float), ("v", c_float), ("inst", c_int32), ("prim", c_int32),
                ("sphere", c_int32), ("pad", c_int32 * 2)]


class Pixel(ctypes.Structure):
    """illume_pixel (src/bitmap.h:6-12 layout: size_t channels)"""
    _fields_ = [("red", c_size_t), ("green", c_size_t), ("blue", c_size_t)]


class Bitmap(ctypes.Structure):
    """illume_bitmap (src/bitmap.h:14-20 layout)"""
    _fields_ = [("pixels", POINTER(Pixel)), ("width", c_size_t), ("height", c_size_t)]


# Every exported symbol of include/illume.h: name -> (restype, argtypes).
PROTOTYPES = {
    "illume_last_error": (c_char_p, []),
    "illume_abi_version": (c_int, []),
    "illume_context_create": (c_int, [c_int, c_size_t, POINTER(c_void_p)]),
    "illume_context_destroy": (c_int, [c_void_p]),
    "illume_context_stream": (c_void_p, [c_void_p]),
    "illume_context_set_bvh_builder": (c_int, [c_void_p, c_int]),
    "illume_scene_build_info": (c_int, [c_void_p, POINTER(c_int), POINTER(c_double)]),
    "illume_scene_load_json": (c_int, [c_void_p, c_char_p, c_char_p, POINTER(c_void_p)]),
    "illume_scene_load_json_string": (c_int, [c_void_p, c_char_p, c_char_p, POINTER(c_void_p)]),
    "illume_scene_create": (c_int, [c_void_p, POINTER(SceneDesc), POINTER(c_void_p)]),
    "illume_scene_describe": (c_int, [c_void_p, POINTER(SceneDesc)]),
    "illume_scene_device_bytes": (c_int, [c_void_p, POINTER(c_size_t)]),
    "illume_scene_check_bvh": (c_int, [c_void_p, c_char_p, c_size_t]),
    "illume_scene_bvh_digest": (c_int, [c_void_p, c_int, POINTER(c_uint64)]),
    "illume_bvh_cache_stats": (c_int, [POINTER(c_int64), POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]),
    "illume_bvh_cache_clear": (c_int, []),
    "illume_scene_upload": (c_int, [c_void_p, POINTER(c_size_t)]),
    "illume_renderer_profile": (c_int, [c_void_p, c_int, POINTER(Profile)]),
    "illume_scene_destroy": (c_int, [c_void_p]),
    "illume_render_params_default": (c_int, [c_void_p, c_int, c_int, POINTER(RenderParams)]),
    "illume_renderer_create": (c_int, [c_void_p, c_void_p, POINTER(RenderParams), POINTER(c_void_p)]),
    "illume_renderer_destroy": (c_int, [c_void_p]),
    "illume_renderer_get_width": (c_int, [c_void_p]),
    "illume_renderer_get_height": (c_int, [c_void_p]),
    "illume_render_to_bitmap": (c_int, [c_void_p, POINTER(Bitmap), POINTER(RenderStats)]),
    "illume_render": (c_int, [c_void_p, _pf, POINTER(c_double), POINTER(c_double), POINTER(c_uint8),
                              POINTER(RenderStats)]),
    "illume_render_device": (c_int, [c_void_p, c_int, POINTER(RenderStats)]),
    "illume_renderer_read": (c_int, [c_void_p, _pf, POINTER(c_double), POINTER(c_double), POINTER(c_uint8)]),
    "illume_render_noalloc": (c_int, [c_void_p, c_void_p, POINTER(RenderParams), c_void_p]),
    "illume_bitmap_new": (POINTER(Bitmap), [c_size_t, c_size_t]),
    "illume_bitmap_free": (None, [POINTER(Bitmap)]),
    "illume_bitmap_save_png": (c_int, [POINTER(Bitmap), c_char_p]),
    "illume_bitmap_save_ppm": (c_int, [POINTER(Bitmap), c_char_p]),
    "illume_save_pfm": (c_int, [_pf, c_int, c_int, c_char_p]),
    "illume_trace_closest": (c_int, [c_void_p, c_void_p, _pf, c_int, c_int, c_int, POINTER(Hit)]),
    "illume_trace_closest_device": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p]),
    "illume_bsdf_batch": (c_int, [c_void_p, c_int, c_int, _pf, c_int, _pf]),
    "illume_server_create": (c_int, [c_void_p, c_size_t, c_int, POINTER(c_void_p)]),
    "illume_server_destroy": (c_int, [c_void_p]),
    "illume_job_submit": (c_int, [c_void_p, c_void_p, POINTER(RenderParams), POINTER(c_int64)]),
    "illume_server_step": (c_int, [c_void_p, POINTER(c_int)]),
    "illume_job_poll": (c_int, [c_void_p, c_int64, _pf, POINTER(c_uint8), POINTER(RenderStats)]),
    "illume_job_cancel": (c_int, [c_void_p, c_int64]),
    "illume_server_set_option": (c_int, [c_void_p, c_int, c_int64]),
    "illume_server_get_stats": (c_int, [c_void_p, POINTER(ServerStats)]),
    "illume_plan_pass_shares": (c_int, [c_int, _pi32, _pi32, c_int64, _pi32]),
    "illume_alias_table": (c_int, [c_int, POINTER(c_double), _pf, _pi32]),
    "illume_measure_l2_read": (c_int, [c_void_p, c_size_t, c_int, POINTER(c_double)]),
    "illume_render_batch": (c_int, [c_void_p, c_int, POINTER(c_void_p), POINTER(RenderParams), POINTER(_pf),
                                    POINTER(POINTER(c_uint8)), POINTER(RenderStats), c_int, POINTER(ServerStats)]),
}

_LIB = None


class IllumeError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"illume status {status}: {message}")
        self.status = status


def lib() -> ctypes.CDLL:
    """Load the native library once; raise if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(status: int) -> int:
    if status != OK:
        msg = lib().illume_last_error()
        raise IllumeError(status, msg.decode() if msg else "")
    return status


def fptr(a):
    return a.ctypes.data_as(_pf) if a is not None else None


def dptr(a):
    return a.ctypes.data_as(POINTER(c_double)) if a is not None else None


def u8ptr(a):
    return a.ctypes.data_as(POINTER(c_uint8)) if a is not None else None
