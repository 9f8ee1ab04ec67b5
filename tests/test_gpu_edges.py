"""Edge cases of a render on the GPU: nothing to hit, no bounces, no samples, images of one
pixel and of sizes that leave partial camera-ray tiles, sizes at the limit, and the
parameter checks that turn bad input into an error instead of a launch."""
import numpy as np
import pytest

from conftest import golden_scene
from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def renderer(ctx, sd, w, h, spp, depth, **kw):
    from illume_gb300.api import HostScene, Renderer
    scene = HostScene.from_data(ctx, sd)
    p = scene.default_params(spp, depth)
    p.width, p.height = w, h
    for k, v in kw.items():
        setattr(p, k, v)
    return scene, Renderer(ctx, scene, params=p)


def empty_scene(color):
    from illume_gb300.scenedata import SceneData
    s = SceneData()
    s.env_tex = s.constant(color)
    s.width = s.height = 8
    return s


def test_nothing_to_hit_is_the_environment(ctx):
    """A scene without geometry: every camera ray escapes at once."""
    _, r = renderer(ctx, empty_scene((0.25, 0.5, 1.0)), 40, 12, 16, 8)
    out = r.render(mean=True, sums=True)
    assert np.array_equal(out["mean"], np.tile(np.float32([0.25, 0.5, 1.0]), (40 * 12, 1)))
    assert out["stats"].rays == 40 * 12 * 16


def test_no_bounces_and_no_samples(ctx):
    sd = golden_scene("box")
    _, r = renderer(ctx, sd, 16, 16, 8, 0)   # max depth 0: no closest-hit query at all
    out = r.render(mean=True, sums=True, rgb8=True)
    assert out["stats"].rays == 0
    assert not out["sum"].any() and not out["mean"].any() and not out["rgb8"].any()
    _, r = renderer(ctx, sd, 16, 16, 0, 8)   # no samples: black, no NaN
    out = r.render(mean=True, sums=True)
    assert out["stats"].rays == 0 and np.isfinite(out["mean"]).all() and not out["mean"].any()


@pytest.mark.parametrize("size", [(1, 1), (37, 5), (1, 33), (9, 4), (8, 3), (130, 7)])
def test_odd_sizes_match_the_oracle(ctx, size):
    """Sizes that leave partial 8x4 camera-ray tiles: every pixel's camera rays are the
    oracle's. One closest-hit query per path (depth 1), so nothing after the camera ray
    and its hit or escape can part the two: sums agree to FP32 rounding of the
    accumulation and the ray counts exactly."""
    from illume_gb300 import synth
    from oracle import pyoracle
    w, h = size
    sd = synth.traversal_scene(tris=2000, env_size=(64, 32), width=w, height=h)
    _, r = renderer(ctx, sd, w, h, 4, 1, accum_mode=C.ACCUM_FP64, seed=5)
    out = r.render(mean=True, sums=True)
    s, _, rays = pyoracle.OracleScene(sd).render(w, h, 4, 1, seed=5, isect=C.ISECT_WATERTIGHT, precision=32)
    assert out["stats"].rays == rays == w * h * 4
    assert np.allclose(out["sum"], s, rtol=1e-5, atol=1e-6)


def test_bad_parameters_are_errors(ctx):
    from illume_gb300.api import HostScene, Renderer
    scene = HostScene.from_data(ctx, golden_scene("box"))
    cases = [dict(width=0), dict(height=-1), dict(spp=-1), dict(max_depth=-2), dict(bvh_kind=7),
             dict(intersector=9), dict(accum_mode=5), dict(trace_variant=9), dict(shade_variant=9),
             dict(estimator=4), dict(samples_per_pass=-3), dict(width=1 << 15, height=1 << 14)]
    for kw in cases:
        p = scene.default_params(1, 4)
        p.width, p.height = 8, 8
        for k, v in kw.items():
            setattr(p, k, v)
        with pytest.raises(C.IllumeError) as e:
            Renderer(ctx, scene, params=p)
        assert e.value.status == C.ERR_INVALID, kw
