"""Contexts used from several host threads at once, on the GPU.

A context may be used from one host thread at a time and different contexts may be used
concurrently (include/illume.h). Here each thread has its own context on device 0 and
renders its own scene while the others render theirs; every image must equal the one the
same render gives alone (a path's random numbers depend only on pixel, sample and bounce,
and each pixel's samples are summed in sample order). ctypes releases the interpreter
lock for every library call, so the renders overlap on the host and on the device. The
reference renders on one thread (src/main.cu:14-43)."""
import threading

import numpy as np
import pytest

from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def _scenes():
    from illume_gb300 import synth
    return [synth.cornell_scene(40, 40),
            synth.traversal_scene(tris=8000, env_size=(64, 32), width=48, height=40),
            synth.sss_scene(tris=6000, width=40, height=32),
            synth.instanced_scene(4, 2000, seed=2, env=synth.environment_map(3, 32, 16))]


def _render(ctx, sd, spp, depth, bvh):
    from illume_gb300.api import HostScene, Renderer
    sc = HostScene.from_data(ctx, sd)
    p = sc.default_params(spp, depth)
    p.width, p.height, p.accum_mode, p.bvh_kind = sd.width, sd.height, C.ACCUM_FP64, bvh
    r = Renderer(ctx, sc, params=p)
    out = r.render(mean=False, sums=True)
    r.close()
    sc.close()
    return out["sum"], out["stats"].rays


@pytest.mark.parametrize("bvh", [C.BVH_WIDE4, C.BVH_WIDE8])
def test_contexts_render_concurrently_as_they_render_alone(native_lib, bvh):
    import torch
    from illume_gb300.api import Context
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    scenes = _scenes()
    for sd in scenes:
        sd.width, sd.height = min(sd.width, 48), min(sd.height, 40)
    contexts = [Context(0) for _ in scenes]
    try:
        alone = [_render(c, sd, 16, 10, bvh) for c, sd in zip(contexts, scenes)]
        together, errors = {}, []
        barrier = threading.Barrier(len(scenes))

        def work(i):
            try:
                barrier.wait(timeout=120)
                together[i] = [_render(contexts[i], scenes[i], 16, 10, bvh) for _ in range(2)]
            except Exception as e:      # reported by the main thread
                errors.append((i, repr(e)))

        threads = [threading.Thread(target=work, args=(i,)) for i in range(len(scenes))]
        for t in threads:
            t.start()
        for t in threads:
            t.join(timeout=600)
        assert not errors, errors
        for i, (s, rays) in enumerate(alone):
            assert rays > 0
            for s2, rays2 in together[i]:
                assert rays2 == rays, i
                assert np.array_equal(s2, s, equal_nan=True), i
    finally:
        for c in contexts:
            c.close()
