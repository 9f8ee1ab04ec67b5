"""Batched and served rendering on the GPU: jobs share one wavefront job table (continuous
batching), and every job's image is bit-identical to its render alone, whatever the mix,
the admission order, the split of path slots, the autotuner's choices or cancellations
around it."""
import numpy as np
import pytest

from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def params(scene, w, h, spp, depth, seed=0, job=0, accum=C.ACCUM_FP32, bvh=None):
    p = scene.default_params(spp, depth)
    p.width, p.height, p.seed, p.job, p.accum_mode = w, h, seed, job, accum
    if bvh is not None:
        p.bvh_kind = bvh
    return p


@pytest.fixture(scope="module")
def scenes(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene
    a = HostScene.from_data(ctx, synth.cornell_scene(48, 48))
    b = HostScene.from_data(ctx, synth.traversal_scene(tris=5000, env_size=(64, 32), width=64, height=48))
    return a, b


def job_list(scenes, bvh=None):
    a, b = scenes
    return [(a, params(a, 48, 48, 40, 8, seed=1, job=1, bvh=bvh)), (b, params(b, 64, 48, 24, 12, seed=2, job=2, bvh=bvh)),
            (a, params(a, 32, 24, 64, 6, seed=3, job=3, bvh=bvh)),
            (b, params(b, 40, 40, 9, 20, seed=4, job=4, accum=C.ACCUM_KAHAN, bvh=bvh)),
            (a, params(a, 24, 16, 100, 8, seed=5, job=5, accum=C.ACCUM_FP64, bvh=bvh))]


def alone(ctx, sc, p):
    from illume_gb300.api import Server
    srv = Server(ctx)
    j = srv.submit(sc, p)
    srv.run()
    out = srv.poll(j, rgb8=True)
    srv.close()
    return out


@pytest.mark.parametrize("bvh", [C.BVH_WIDE4, C.BVH_BINARY])
def test_same_alone_and_in_the_mix(ctx, scenes, bvh):
    """Every server setting (slots, passes per step, each trace kernel variant of the
    layout, path regeneration) gives each job the image it gets alone with the default
    settings."""
    from illume_gb300.api import Server
    jobs = job_list(scenes, bvh)
    ref = [alone(ctx, sc, p) for sc, p in jobs]
    variants = [{"trace_variant": v} for v in ((1, 2, 3, 4) if bvh == C.BVH_BINARY else (1, 2, 3))]
    regen = [{"queue_slots": 5000}, {"queue_slots": 20000, "regen_threshold_permille": 300},
             {"path_capacity": 40000, "queue_slots": 9000, "regen_threshold_permille": 0, "lanes": 2}]
    for opts in [{}, {"path_capacity": 40000}, {"passes_per_step": 4}, {"lanes": 1}, {"lanes": 3}] + variants + regen:
        srv = Server(ctx, **opts)
        ids = [srv.submit(sc, p) for sc, p in jobs]
        srv.run()
        for k, j in enumerate(ids):
            out = srv.poll(j, rgb8=True)
            assert np.array_equal(out["mean"], ref[k]["mean"]), (opts, k)
            assert np.array_equal(out["rgb8"], ref[k]["rgb8"]), (opts, k)
            assert out["stats"].rays == ref[k]["stats"].rays, (opts, k)
        assert srv.stats().jobs_done == len(jobs)
        srv.close()


def test_server_equals_renderer(ctx, scenes):
    """A served job's image equals the plain renderer's image of the same parameters."""
    from illume_gb300.api import Renderer
    for sc, p in job_list(scenes):
        r = Renderer(ctx, sc, params=p)
        want = r.render(mean=True, rgb8=True)
        got = alone(ctx, sc, p)
        assert np.array_equal(got["mean"], want["mean"])
        assert np.array_equal(got["rgb8"], want["rgb8"])
        assert got["stats"].rays == want["stats"].rays


def test_arrivals_while_running_and_cancel(ctx, scenes):
    """Jobs submitted while others are on the device join the next pass; cancelling a
    running job leaves the others' images unchanged."""
    from illume_gb300.api import Server
    jobs = job_list(scenes)
    ref = [alone(ctx, sc, p) for sc, p in jobs]
    a, b = scenes
    srv = Server(ctx, path_capacity=20000)
    ids = [srv.submit(*jobs[0]), srv.submit(*jobs[1])]
    srv.step()
    victim = srv.submit(b, params(b, 40, 40, 4000, 20, seed=9, job=9))   # far from done when cancelled
    srv.step()
    ids.append(srv.submit(*jobs[2]))
    srv.step()
    srv.cancel(victim)
    ids.append(srv.submit(*jobs[4]))
    srv.run()
    for k, j in zip([0, 1, 2, 4], ids):
        out = srv.poll(j, rgb8=True)
        assert np.array_equal(out["mean"], ref[k]["mean"]), k
    with pytest.raises(C.IllumeError):
        srv.poll(victim)
    srv.close()


def test_batch_and_autotune(ctx, scenes):
    from illume_gb300.api import render_batch
    jobs = job_list(scenes) * 3
    ref = [alone(ctx, sc, p) for sc, p in jobs[:5]]
    for tune in (False, True):
        means, pix, stats, bs = render_batch(ctx, [s for s, _ in jobs], [p for _, p in jobs], autotune=tune, rgb8=True)
        for k in range(len(jobs)):
            assert np.array_equal(means[k], ref[k % 5]["mean"]), (tune, k)
            assert np.array_equal(pix[k], ref[k % 5]["rgb8"]), (tune, k)
            assert stats[k].rays == ref[k % 5]["stats"].rays
        assert bs.jobs_done == len(jobs) and bs.rays == sum(s.rays for s in stats)
        assert bs.passes > 0 and bs.device_ms > 0


def test_budget_admission(ctx, scenes):
    from illume_gb300.api import Server
    a, _ = scenes
    p = params(a, 64, 64, 16, 6)
    srv = Server(ctx, hbm_budget_bytes=1 << 16)   # below one job's footprint
    with pytest.raises(C.IllumeError) as e:
        srv.submit(a, p)
    assert e.value.status == C.ERR_BUDGET
    srv.close()
    # room for one job's buffers and a small table at a time: jobs run one after another
    srv = Server(ctx, hbm_budget_bytes=16 << 20, max_jobs_in_flight=1, path_capacity=64 * 64 * 4)
    ids = [srv.submit(a, p) for _ in range(3)]
    srv.cancel(ids[1])
    srv.run()
    m0 = srv.poll(ids[0])["mean"]
    with pytest.raises(C.IllumeError) as e:
        srv.poll(ids[1])
    assert e.value.status == C.ERR_CANCELLED
    assert np.array_equal(srv.poll(ids[2])["mean"], m0)
    assert srv.stats().device_bytes <= 16 << 20
    srv.close()


@pytest.mark.parametrize("accum", [C.ACCUM_FP32, C.ACCUM_KAHAN, C.ACCUM_FP64])
def test_split_render_same_image(ctx, scenes, accum):
    """A render large enough to split its passes over two engines taking turns (4M paths
    per pass and more) gives the image of the same job rendered in small passes on one
    engine, and of the same job served: accumulations stay in sample order."""
    from illume_gb300.api import Renderer
    _, b = scenes
    p = params(b, 512, 512, 24, 12, seed=7, job=7, accum=accum)   # 16 samples per pass -> 2 x 8, 3 passes
    big = Renderer(ctx, b, params=p)
    got = big.render(mean=True, sums=True)
    p1 = params(b, 512, 512, 24, 12, seed=7, job=7, accum=accum)
    p1.samples_per_pass = 3                                         # 0.8M paths per pass: one engine
    small = Renderer(ctx, b, params=p1)
    want = small.render(mean=True, sums=True)
    assert np.array_equal(got["mean"], want["mean"])
    assert np.array_equal(got["sum"], want["sum"])
    assert got["stats"].rays == want["stats"].rays
    served = alone(ctx, b, params(b, 512, 512, 24, 12, seed=7, job=7, accum=accum))
    assert np.array_equal(got["mean"], served["mean"])
    # progressive: a second call continues the sample sequence in both engines
    for r in (big, small):
        r.render_device(accumulate=False)
        r.render_device(accumulate=True)
    assert np.array_equal(big.read(mean=False, sums=True)["sum"], small.read(mean=False, sums=True)["sum"])
    big.close()
    small.close()


def test_shade_variants_same_image(ctx, scenes):
    """Every register bound of the shade kernel gives the same image, for both estimators."""
    from illume_gb300.api import Renderer
    for est in (C.ESTIMATOR_REFERENCE, C.ESTIMATOR_NEE):
        for sc, p in job_list(scenes)[:3]:
            p.estimator = est
            want = Renderer(ctx, sc, params=p).render(mean=True)
            for v in (1, 2, 3, 4):
                q = C.RenderParams.from_buffer_copy(p)
                q.shade_variant = v
                got = Renderer(ctx, sc, params=q).render(mean=True)
                assert np.array_equal(got["mean"], want["mean"], equal_nan=True), (est, v)
                assert got["stats"].rays == want["stats"].rays


def test_a_table_that_does_not_fit_falls_back():
    """A context whose memory budget holds one job table but not two: the second table's
    allocation is refused and the setting's first table takes every job, each image
    still the one it gets alone."""
    from illume_gb300 import synth
    from illume_gb300.api import Context, HostScene, Server
    slots = 1 << 22                                       # ~0.74 GB of path state per table
    ctx = Context(0, hbm_budget_bytes=(1 << 30) + (1 << 28))
    try:
        a = HostScene.from_data(ctx, synth.cornell_scene(48, 48))
        jobs = [params(a, 48, 48, 16, 6, seed=s, job=s) for s in (1, 2, 3)]
        ref = []
        for p in jobs:
            srv = Server(ctx, path_capacity=slots)
            j = srv.submit(a, p)
            srv.run()
            ref.append(srv.poll(j)["mean"])
            srv.close()
        srv = Server(ctx, path_capacity=slots, lanes=4)
        ids = [srv.submit(a, p) for p in jobs]
        srv.run()
        for k, j in enumerate(ids):
            assert np.array_equal(srv.poll(j)["mean"], ref[k]), k
        assert srv.stats().jobs_done == len(jobs)
        srv.close()
    finally:
        ctx.close()
