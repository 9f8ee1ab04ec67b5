"""illume_render_noalloc: rendering for callers that cannot allocate device memory at
render time (a host whose own memory pool owns the GPU, a frame loop that must not stall
on cudaMalloc/cudaFree). It renders through a fixed scratch array inside the library
instead of allocating, so its images must equal those of the allocating entry point.

Checked through the C-ABI against illume_render (same scene, parameters and Philox
streams, FP32 accumulation in sample order) on two calls in a row, the second on a
different scene and size so that leftovers of the first call would show; plus the size
limit. This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def reference_sums(ctx, scene, p):
    """The allocating path: illume_renderer_create + illume_render, FP32 sums."""
    L = C.lib()
    r = ctypes.c_void_p()
    C.check(L.illume_renderer_create(ctx.handle, scene.handle, ctypes.byref(p), ctypes.byref(r)))
    n = p.width * p.height
    s = np.zeros((n, 3), np.float64)
    st = C.RenderStats()
    C.check(L.illume_render(r, None, C.dptr(s), None, None, ctypes.byref(st)))
    L.illume_renderer_destroy(r)
    return s.astype(np.float32)


def noalloc_sums(ctx, scene, p):
    import torch
    n = p.width * p.height
    out = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda:0")   # caller-owned output
    torch.cuda.synchronize()
    C.check(C.lib().illume_render_noalloc(ctx.handle, scene.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr())))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_render_on_two_calls(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene
    cases = [(synth.cornell_scene(64, 64), 64, 64, 6, 8), (synth.traversal_scene(tris=6000, env_size=(64, 32)), 48, 40, 4, 12)]
    for sd, w, h, spp, depth in cases:
        scene = HostScene.from_data(ctx, sd)
        p = scene.default_params(spp, depth)
        p.width, p.height = w, h
        p.accum_mode = C.ACCUM_FP32
        want = reference_sums(ctx, scene, p)
        got = noalloc_sums(ctx, scene, p)
        assert np.isfinite(got).all()
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
        scene.close()


def test_noalloc_rejects_images_beyond_the_scratch_limit(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene
    import torch
    scene = HostScene.from_data(ctx, synth.cornell_scene(8, 8))
    p = scene.default_params(1, 4)
    p.width, p.height = 512, 512                      # 262,144 pixels > ILLUME_NOALLOC_MAX_PIXELS (65,536)
    out = torch.zeros(16, dtype=torch.float32, device="cuda:0")
    st = C.lib().illume_render_noalloc(ctx.handle, scene.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr()))
    assert st == C.ERR_INVALID
    assert b"scratch limit" in C.lib().illume_last_error()
    scene.close()
