"""illume_render_noalloc: rendering for callers that cannot allocate device memory at
render time (a host whose own memory pool owns the GPU, a frame loop that must not stall
on cudaMalloc/cudaFree). It renders through a fixed scratch array inside the library
instead of allocating, so its images must equal those of the allocating entry point.

Checked through the C-ABI against illume_render (same scene, parameters and Philox
streams, FP32 accumulation in sample order) on two calls in a row, the second on a
different scene and size so that leftovers of the first call would show; on every BVH
layout with both triangle tests; on the golden scene with a participating medium (the
medium index travels packed beside the job row in the queued rays); plus the size limit
and the parameters this entry point does not take. This file is collected last.
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


@pytest.mark.parametrize("bvh", [C.BVH_BINARY, C.BVH_WIDE8, C.BVH_WIDE8_PERSISTENT, C.BVH_WIDE4])
@pytest.mark.parametrize("isect", [C.ISECT_MT, C.ISECT_WATERTIGHT])
def test_noalloc_matches_render_per_layout(ctx, bvh, isect):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene
    scene = HostScene.from_data(ctx, synth.traversal_scene(tris=3000, env_size=(64, 32)))
    p = scene.default_params(2, 8)
    p.width, p.height = 32, 32
    p.accum_mode = C.ACCUM_FP32
    p.bvh_kind, p.intersector = bvh, isect
    want = reference_sums(ctx, scene, p)
    got = noalloc_sums(ctx, scene, p)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
    scene.close()


def test_noalloc_matches_render_with_a_medium(ctx):
    from conftest import golden_scene
    from illume_gb300.api import HostScene
    sd = golden_scene("materials")
    assert len(sd.mediums) > 0
    scene = HostScene.from_data(ctx, sd)
    p = scene.default_params(4, 12)
    p.width, p.height = 40, 30
    p.accum_mode = C.ACCUM_FP32
    want = reference_sums(ctx, scene, p)
    got = noalloc_sums(ctx, scene, p)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)
    scene.close()


def test_noalloc_rejects_what_it_does_not_take(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene
    import torch
    scene = HostScene.from_data(ctx, synth.cornell_scene(8, 8))
    out = torch.zeros(3 * 64, dtype=torch.float32, device="cuda:0")
    L = C.lib()
    for field, value, status in [("samples_per_pass", 4, C.ERR_UNSUPPORTED), ("engines", 2, C.ERR_UNSUPPORTED),
                                 ("queue_slots", 1024, C.ERR_UNSUPPORTED),
                                 ("trace_variant", 9, C.ERR_INVALID), ("shade_variant", 9, C.ERR_INVALID),
                                 ("accum_mode", C.ACCUM_FP64, C.ERR_INVALID)]:
        p = scene.default_params(1, 4)
        p.width, p.height = 8, 8
        p.accum_mode = C.ACCUM_FP32
        setattr(p, field, value)
        st = L.illume_render_noalloc(ctx.handle, scene.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr()))
        assert st == status, (field, st)
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
