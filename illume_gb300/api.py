"""Python mirror of the reference's render interface, over the C-ABI of include/illume.h.

    ctx = Context()                                  # one device, one CUDA stream
    scene = HostScene.from_json_file(ctx, path)      # HostScene(doc) + SceneRef (src/scene/scene.h:11-28)
    renderer = Renderer(ctx, scene, spp, max_depth)  # Renderer(json, scene, spp, max_depth) (src/renderer.h:12)
    bitmap = Bitmap(renderer.get_width(), renderer.get_height())
    renderer.render_to_bitmap(bitmap)                # src/renderer.cu:498-597
    bitmap.save_png(path)                            # bitmap_save_to_png (src/bitmap.h:30)

Every call goes to the native library; nothing here computes pixels.
"""
from __future__ import annotations

import ctypes
import os
import weakref
from typing import Optional

import numpy as np

from . import _capi as C
from .scenedata import SceneData


class Context:
    """One device and one CUDA stream. Closing a context first closes the servers,
    renderers and scenes made with it (newest first), which must not outlive it."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.handle = ctypes.c_void_p()
        self._children = []
        C.check(C.lib().illume_context_create(device, hbm_budget_bytes, ctypes.byref(self.handle)))

    def _adopt(self, obj):
        self._children.append(weakref.ref(obj))

    def close(self):
        if self.handle:
            for ref in reversed(self._children):
                obj = ref()
                if obj is not None:
                    obj.close()
            self._children = []
            C.lib().illume_context_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return C.lib().illume_context_stream(self.handle) or 0

    def set_bvh_builder(self, builder: int) -> None:
        """C.BVH_BUILD_HOST (binned SAH on the host cores, the default) or
        C.BVH_BUILD_DEVICE (locally-ordered clustering on this context's GPU) for the
        scenes made on this context from now on."""
        C.check(C.lib().illume_context_set_bvh_builder(self.handle, builder))


class HostScene:
    """A scene resident on the device (geometry, BVHs, materials, textures)."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self.ctx = ctx
        self.handle = handle
        ctx._adopt(self)

    @staticmethod
    def from_json_file(ctx: Context, path: str, base_dir: Optional[str] = None) -> "HostScene":
        h = ctypes.c_void_p()
        C.check(C.lib().illume_scene_load_json(ctx.handle, path.encode(), base_dir.encode() if base_dir else None,
                                               ctypes.byref(h)))
        return HostScene(ctx, h)

    @staticmethod
    def from_json_string(ctx: Context, text: str, base_dir: Optional[str] = None) -> "HostScene":
        h = ctypes.c_void_p()
        C.check(C.lib().illume_scene_load_json_string(ctx.handle, text.encode(), base_dir.encode() if base_dir else None,
                                                      ctypes.byref(h)))
        return HostScene(ctx, h)

    @staticmethod
    def from_data(ctx: Context, data: SceneData) -> "HostScene":
        desc, keep = data.to_desc()
        h = ctypes.c_void_p()
        C.check(C.lib().illume_scene_create(ctx.handle, ctypes.byref(desc), ctypes.byref(h)))
        del keep
        return HostScene(ctx, h)

    def describe(self) -> SceneData:
        d = C.SceneDesc()
        C.check(C.lib().illume_scene_describe(self.handle, ctypes.byref(d)))
        return SceneData.from_desc(d)

    def build_info(self) -> dict:
        """Meshes whose BVHs came from the device build, and the BVH build's wall time."""
        d, ms = ctypes.c_int(), ctypes.c_double()
        C.check(C.lib().illume_scene_build_info(self.handle, ctypes.byref(d), ctypes.byref(ms)))
        return {"device_meshes": d.value, "build_ms": ms.value}

    def check_bvh(self) -> str:
        """Checks every mesh's BVH invariants (raises on a violation); returns the report."""
        buf = ctypes.create_string_buffer(1 << 16)
        C.check(C.lib().illume_scene_check_bvh(self.handle, buf, len(buf)))
        return buf.value.decode()

    def device_bytes(self) -> int:
        n = ctypes.c_size_t()
        C.check(C.lib().illume_scene_device_bytes(self.handle, ctypes.byref(n)))
        return n.value

    def default_params(self, spp: int, max_depth: int) -> C.RenderParams:
        p = C.RenderParams()
        C.check(C.lib().illume_render_params_default(self.handle, spp, max_depth, ctypes.byref(p)))
        return p

    def trace_closest(self, rays8: np.ndarray, intersector=C.ISECT_WATERTIGHT, bvh_kind=C.BVH_WIDE8) -> dict:
        rays8 = np.ascontiguousarray(rays8, dtype=np.float32)
        n = rays8.shape[0]
        hits = (C.Hit * max(n, 1))()
        C.check(C.lib().illume_trace_closest(self.ctx.handle, self.handle, C.fptr(rays8), n, intersector, bvh_kind, hits))
        a = np.ctypeslib.as_array(hits)[:n]
        return {k: a[k].copy() for k in ("t", "u", "v", "inst", "prim", "sphere")}

    def close(self):
        if self.handle:
            C.lib().illume_scene_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Bitmap:
    """Caller-owned RGB bitmap with the reference's Pixel{size_t r, g, b} layout."""

    def __init__(self, width: int, height: int):
        self.ptr = C.lib().illume_bitmap_new(width, height)
        if not self.ptr:
            raise MemoryError("illume_bitmap_new failed")
        self.width, self.height = width, height

    def rgb8(self) -> np.ndarray:
        px = np.ctypeslib.as_array(self.ptr.contents.pixels, shape=(self.width * self.height,))
        return np.stack([px["red"], px["green"], px["blue"]], axis=1).astype(np.uint8).reshape(self.height, self.width, 3)

    def save_png(self, path: str):
        C.check(C.lib().illume_bitmap_save_png(self.ptr, path.encode()))

    def save_ppm(self, path: str):
        C.check(C.lib().illume_bitmap_save_ppm(self.ptr, path.encode()))

    def __del__(self):
        if getattr(self, "ptr", None):
            C.lib().illume_bitmap_free(self.ptr)
            self.ptr = None


class Renderer:
    def __init__(self, ctx: Context, scene: HostScene, spp: int = 1, max_depth: int = 8,
                 params: Optional[C.RenderParams] = None, **overrides):
        self.ctx, self.scene = ctx, scene
        p = params if params is not None else scene.default_params(spp, max_depth)
        for k, v in overrides.items():
            setattr(p, k, v)
        self.params = p
        self.handle = ctypes.c_void_p()
        C.check(C.lib().illume_renderer_create(ctx.handle, scene.handle, ctypes.byref(p), ctypes.byref(self.handle)))
        ctx._adopt(self)

    def get_width(self) -> int:
        return C.lib().illume_renderer_get_width(self.handle)

    def get_height(self) -> int:
        return C.lib().illume_renderer_get_height(self.handle)

    def render_to_bitmap(self, bitmap: Bitmap) -> C.RenderStats:
        st = C.RenderStats()
        C.check(C.lib().illume_render_to_bitmap(self.handle, bitmap.ptr, ctypes.byref(st)))
        return st

    def render(self, mean=True, sums=False, rgb8=False):
        """Full render; returns dict with the requested host arrays and the stats."""
        n = self.get_width() * self.get_height()
        out = {}
        m = np.zeros((n, 3), np.float32) if mean else None
        s = np.zeros((n, 3), np.float64) if sums else None
        s2 = np.zeros((n, 3), np.float64) if sums else None
        r8 = np.zeros((n, 3), np.uint8) if rgb8 else None
        st = C.RenderStats()
        C.check(C.lib().illume_render(self.handle, C.fptr(m), C.dptr(s), C.dptr(s2), C.u8ptr(r8), ctypes.byref(st)))
        out.update(mean=m, sum=s, sumsq=s2, rgb8=r8, stats=st)
        return out

    def render_device(self, accumulate: bool = False) -> C.RenderStats:
        st = C.RenderStats()
        C.check(C.lib().illume_render_device(self.handle, int(accumulate), ctypes.byref(st)))
        return st

    def read(self, mean=True, sums=False, rgb8=False):
        n = self.get_width() * self.get_height()
        m = np.zeros((n, 3), np.float32) if mean else None
        s = np.zeros((n, 3), np.float64) if sums else None
        s2 = np.zeros((n, 3), np.float64) if sums else None
        r8 = np.zeros((n, 3), np.uint8) if rgb8 else None
        C.check(C.lib().illume_renderer_read(self.handle, C.fptr(m), C.dptr(s), C.dptr(s2), C.u8ptr(r8)))
        return dict(mean=m, sum=s, sumsq=s2, rgb8=r8)

    def close(self):
        if self.handle:
            C.lib().illume_renderer_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bsdf_batch(ctx: Context, material_type: int, distribution: int, inputs: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(inputs, dtype=np.float32).reshape(-1, 16)
    y = np.zeros_like(x)
    C.check(C.lib().illume_bsdf_batch(ctx.handle, material_type, distribution, C.fptr(x), x.shape[0], C.fptr(y)))
    return y


class Server:
    """Continuous-batching render server (illume_server_* of include/illume.h)."""

    def __init__(self, ctx: Context, hbm_budget_bytes: int = 0, max_jobs_in_flight: int = 0, **options):
        self.ctx = ctx
        self.handle = ctypes.c_void_p()
        C.check(C.lib().illume_server_create(ctx.handle, hbm_budget_bytes, max_jobs_in_flight, ctypes.byref(self.handle)))
        ctx._adopt(self)
        self._npix = {}
        names = {"path_capacity": C.SERVER_PATH_CAPACITY, "passes_per_step": C.SERVER_PASSES_PER_STEP,
                 "autotune": C.SERVER_AUTOTUNE, "trace_variant": C.SERVER_TRACE_VARIANT, "lanes": C.SERVER_LANES,
                 "queue_slots": C.SERVER_QUEUE_SLOTS, "regen_threshold_permille": C.SERVER_REGEN_THRESHOLD}
        for k, v in options.items():
            C.check(C.lib().illume_server_set_option(self.handle, names[k], int(v)))

    def submit(self, scene: HostScene, params: C.RenderParams) -> int:
        jid = ctypes.c_int64()
        C.check(C.lib().illume_job_submit(self.handle, scene.handle, ctypes.byref(params), ctypes.byref(jid)))
        self._npix[jid.value] = params.width * params.height
        return jid.value

    def step(self) -> int:
        running = ctypes.c_int()
        C.check(C.lib().illume_server_step(self.handle, ctypes.byref(running)))
        return running.value

    def run(self, max_steps: int = 1_000_000) -> int:
        """Steps until no job is running or queued; returns the number of steps."""
        n = 0
        while self.step():
            n += 1
            if n >= max_steps:
                raise RuntimeError("server did not drain")
        return n + 1

    def poll(self, job: int, rgb8: bool = False):
        """None while the job runs, else {'mean', 'rgb8'?, 'stats'}; raises if cancelled or failed."""
        n = self._npix[job]
        mean = np.zeros((n, 3), np.float32)
        px = np.zeros((n, 3), np.uint8) if rgb8 else None
        st = C.RenderStats()
        s = C.lib().illume_job_poll(self.handle, job, C.fptr(mean), C.u8ptr(px), ctypes.byref(st))
        if s == C.ERR_NOT_READY:
            return None
        C.check(s)
        out = {"mean": mean, "stats": st}
        if rgb8:
            out["rgb8"] = px
        return out

    def cancel(self, job: int):
        C.check(C.lib().illume_job_cancel(self.handle, job))

    def stats(self) -> C.ServerStats:
        s = C.ServerStats()
        C.check(C.lib().illume_server_get_stats(self.handle, ctypes.byref(s)))
        return s

    def close(self):
        if self.handle:
            C.lib().illume_server_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_batch(ctx: Context, scenes, params, autotune: bool = False, rgb8: bool = False):
    """illume_render_batch: every job rendered together; returns ([mean per job], [rgb8 per job] or None,
    [RenderStats per job], ServerStats)."""
    n = len(scenes)
    means = [np.zeros((p.width * p.height, 3), np.float32) for p in params]
    pix = [np.zeros((p.width * p.height, 3), np.uint8) for p in params] if rgb8 else None
    sc = (ctypes.c_void_p * n)(*[s.handle.value for s in scenes])
    pa = (C.RenderParams * n)(*params)
    mp = (C._pf * n)(*[C.fptr(m) for m in means])
    rp = (ctypes.POINTER(ctypes.c_uint8) * n)(*[C.u8ptr(x) for x in pix]) if rgb8 else None
    js = (C.RenderStats * n)()
    bs = C.ServerStats()
    C.check(C.lib().illume_render_batch(ctx.handle, n, sc, pa, mp, rp, js, int(autotune), ctypes.byref(bs)))
    return means, pix, list(js), bs
