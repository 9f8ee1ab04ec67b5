"""Traversal scheduling that must not change any image, on the GPU.

Path regeneration: a pass whose paths outnumber the queue slots runs as a loop on the
device (a while node of the pass's CUDA graph) in which new paths enter the queues as
earlier ones end. A path's arithmetic and random numbers depend only on its (pixel,
sample, bounce) and its job, and each pixel's samples are still summed in sample order,
so the image must be bit-identical to the render without regeneration, for every queue
size and threshold, accumulation mode, estimator, engine count and progressive call.

Camera-ray order: a pass's samples of a pixel are queued next to each other in groups
(`ray_group`); the order of the queue changes which rays share a warp, never a path's
result.

Sorted instance walk (the default 4-wide trace kernel; variant 4 walks in index order):
the instances a ray enters are visited nearest box entry first; ties between instances
still go to the lower index, so images must equal the index-order walk's, including
scenes whose instances coincide."""
import numpy as np
import pytest

from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def render(ctx, sd, w, h, spp, depth, calls=1, **kw):
    from illume_gb300.api import HostScene, Renderer
    scene = HostScene.from_data(ctx, sd)
    p = scene.default_params(spp, depth)
    p.width, p.height = w, h
    for k, v in kw.items():
        setattr(p, k, v)
    r = Renderer(ctx, scene, params=p)
    stats = []
    for c in range(calls):
        stats.append(r.render_device(accumulate=c > 0))
    out = r.read(mean=False, sums=True)
    out["stats"] = stats
    r.close()
    scene.close()
    return out


def scenes():
    from illume_gb300 import synth
    from conftest import golden_scene
    return {"traversal": synth.traversal_scene(tris=20000, env_size=(64, 32), width=48, height=40),
            "materials": golden_scene("materials"),     # a medium: paths of very different lengths
            "cornell": synth.cornell_scene(40, 40)}


@pytest.mark.parametrize("name", ["traversal", "materials", "cornell"])
@pytest.mark.parametrize("mode", [C.ACCUM_FP32, C.ACCUM_FP64])
def test_regeneration_gives_the_same_image(ctx, name, mode):
    sd = scenes()[name]
    w, h, spp, depth = 48, 40, 24, 12
    ref = render(ctx, sd, w, h, spp, depth, accum_mode=mode, samples_per_pass=8)
    paths_per_pass = 8 * w * h
    for slots, thr in [(paths_per_pass // 4, 1.0), (paths_per_pass // 3, 0.5), (1000, 0.0), (3 * w * h, 0.25)]:
        got = render(ctx, sd, w, h, spp, depth, accum_mode=mode, samples_per_pass=8, queue_slots=slots,
                     regen_threshold=thr)
        assert np.array_equal(got["sum"], ref["sum"], equal_nan=True), (name, slots, thr)
        assert np.array_equal(got["sumsq"], ref["sumsq"], equal_nan=True), (name, slots, thr)
        assert sum(s.rays for s in got["stats"]) == sum(s.rays for s in ref["stats"])
        # every loop iteration's launches are counted
        assert got["stats"][0].kernel_launches > 5


def test_regeneration_with_next_event_estimation_and_engines(ctx):
    from illume_gb300 import synth
    sd = synth.cornell_scene(32, 32)
    w, h, spp, depth = 32, 32, 32, 10
    kw = dict(accum_mode=C.ACCUM_FP64, estimator=C.ESTIMATOR_NEE, samples_per_pass=8)
    ref = render(ctx, sd, w, h, spp, depth, calls=2, **kw)
    for engines in (1, 3):
        got = render(ctx, sd, w, h, spp, depth, calls=2, engines=engines, queue_slots=3000, regen_threshold=0.6, **kw)
        assert np.array_equal(got["sum"], ref["sum"], equal_nan=True), engines


def test_regeneration_profiled_pass(ctx):
    """The profiling hook drives the loop from the host: same rays as a graph pass."""
    import ctypes
    from illume_gb300 import synth
    from illume_gb300.api import HostScene, Renderer
    scene = HostScene.from_data(ctx, synth.cornell_scene(32, 32))
    p = scene.default_params(8, 8)
    p.width = p.height = 32
    p.samples_per_pass, p.queue_slots, p.regen_threshold = 8, 2000, 0.5
    r = Renderer(ctx, scene, params=p)
    prof = C.Profile()
    C.check(C.lib().illume_renderer_profile(r.handle, 0, ctypes.byref(prof)))
    assert prof.rays > 0 and prof.trace_launches > 8 and prof.trace_ms > 0
    r.close()
    scene.close()


def test_regeneration_parameters_are_checked(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene, Renderer
    scene = HostScene.from_data(ctx, synth.cornell_scene(8, 8))
    for slots, thr in [(-1, 0.5), (100, 1.5), (100, -0.1)]:
        p = scene.default_params(4, 4)
        p.queue_slots, p.regen_threshold = slots, thr
        with pytest.raises(C.IllumeError):
            Renderer(ctx, scene, params=p)
    scene.close()


def _coincident_instances():
    """Three instances of one mesh under the same transform (every hit ties between them)
    with different materials, plus a smaller one in front: whichever instance the walk
    keeps decides the image."""
    from illume_gb300 import synth
    from illume_gb300.scenedata import Material, Mesh, SceneData
    s = SceneData()
    P, T = synth.displaced_icosphere(12, 3)
    m = s.add_mesh(Mesh(P, T))
    mats = [s.add_material(Material(C.MAT_LAMBERT, s.constant(c), s.constant((1e-4,) * 3)))
            for c in ((0.9, 0.1, 0.1), (0.1, 0.9, 0.1), (0.1, 0.1, 0.9), (0.8, 0.8, 0.2))]
    M = np.zeros((3, 4), np.float32)
    M[:, :3] = np.eye(3)
    for k in (2, 0, 1):
        s.add_instance(m, mats[k], M)
    M2 = M.copy()
    M2[:, :3] *= 0.3
    M2[:, 3] = (0.2, 0.1, -1.3)
    s.add_instance(m, mats[3], M2)
    s.env_tex = s.constant((0.8, 0.9, 1.0))
    s.camera_transform = synth.lookat((0.0, 0.5, -4.0), (0.0, 0.0, 0.0))
    s.width = s.height = 40
    s.ray_bias = 1e-4
    return s


@pytest.mark.parametrize("name", ["mesh", "instanced", "coincident"])
def test_sorted_instance_walk_gives_the_same_image(ctx, name):
    from illume_gb300 import synth
    from conftest import golden_scene
    if name == "mesh":
        sd = golden_scene("mesh")
    elif name == "instanced":
        sd = synth.instanced_scene(16, 3000, seed=5, env=synth.environment_map(1, 64, 32))
    else:
        sd = _coincident_instances()
    w, h = 40, 32
    kw = dict(accum_mode=C.ACCUM_FP64, bvh_kind=C.BVH_WIDE4)
    ref = render(ctx, sd, w, h, 8, 10, trace_variant=4, **kw)
    got = render(ctx, sd, w, h, 8, 10, trace_variant=0, **kw)
    assert np.array_equal(got["sum"], ref["sum"], equal_nan=True)
    assert got["stats"][0].rays == ref["stats"][0].rays


@pytest.mark.parametrize("name", ["traversal", "materials"])
def test_camera_ray_grouping_gives_the_same_image(ctx, name):
    sd = scenes()[name]
    w, h, spp, depth = 48, 40, 30, 12
    # 30 samples in passes of 7: groups of 4 and 16 leave smaller last groups
    ref = render(ctx, sd, w, h, spp, depth, accum_mode=C.ACCUM_FP64, samples_per_pass=7, ray_group=1)
    for g in (4, 16, 32, 0):
        got = render(ctx, sd, w, h, spp, depth, accum_mode=C.ACCUM_FP64, samples_per_pass=7, ray_group=g)
        assert np.array_equal(got["sum"], ref["sum"], equal_nan=True), (name, g)
        assert got["stats"][0].rays == ref["stats"][0].rays
    got = render(ctx, sd, w, h, spp, depth, accum_mode=C.ACCUM_FP64, samples_per_pass=7, ray_group=16,
                 queue_slots=900, regen_threshold=0.5)
    assert np.array_equal(got["sum"], ref["sum"], equal_nan=True)
