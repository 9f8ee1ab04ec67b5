"""The opt-in next-event estimator on the GPU: path by path equal to the oracle's
restatement of the estimator on the same Philox streams, same expectation as the
reference estimator (per-pixel 3-sigma test between independent renders of the two),
lower variance where light sampling pays, and the same image alone and in a server mix."""
import numpy as np
import pytest

from illume_gb300 import _capi as C
from nee_scenes import SCENES

pytestmark = pytest.mark.gpu


def render(ctx, sd, w, h, spp, depth, **kw):
    from illume_gb300.api import HostScene, Renderer
    scene = HostScene.from_data(ctx, sd)
    p = scene.default_params(spp, depth)
    p.width, p.height = w, h
    p.accum_mode = C.ACCUM_FP64
    for k, v in kw.items():
        setattr(p, k, v)
    r = Renderer(ctx, scene, params=p)
    out = r.render(mean=False, sums=True)
    r.close()
    scene.close()
    return out


def three_sigma(a, b, n_a, n_b):
    ma, mb = a["sum"] / n_a, b["sum"] / n_b
    va = np.maximum(a["sumsq"] / n_a - ma * ma, 0) / n_a
    vb = np.maximum(b["sumsq"] / n_b - mb * mb, 0) / n_b
    return np.abs(ma - mb) <= 3 * np.sqrt(va + vb) + 1e-7




@pytest.mark.parametrize("name", list(SCENES))
def test_nee_matches_the_oracle_path_by_path(ctx, name):
    """Same (pixel, sample, bounce) streams and the light slot 0x40000000 | bounce: the
    GPU's light choice (alias tables), densities, MIS weights and shadow tests against
    the oracle's FP32 restatement, per pixel within 1e-4 relative on >= 99% of pixels
    (the GPU's sinf/cosf/atan2f may differ from the host's by an ulp, which can move a
    rare path)."""
    from oracle import pyoracle
    sd = SCENES[name]()
    w, h, spp, depth = sd.width, sd.height, 16, 8
    out = render(ctx, sd, w, h, spp, depth, seed=6, intersector=C.ISECT_WATERTIGHT, estimator=C.ESTIMATOR_NEE)
    s, _, rays = pyoracle.OracleScene(sd).render(w, h, spp, depth, seed=6, isect=C.ISECT_WATERTIGHT, precision=32,
                                                 nee=1)
    rel = np.abs(out["sum"] - s) / np.maximum(np.abs(s), 1e-3)
    assert (rel.max(1) < 1e-4).mean() >= 0.99, (name, (rel.max(1) < 1e-4).mean())
    assert abs(out["stats"].rays - rays) <= 0.01 * rays, (out["stats"].rays, rays)


@pytest.mark.parametrize("name", list(SCENES))
def test_same_expectation_as_reference(ctx, name):
    sd = SCENES[name]()
    w, h = sd.width, sd.height
    spp = 2048
    ref = render(ctx, sd, w, h, spp, 8, seed=1)
    nee = render(ctx, sd, w, h, spp, 8, seed=2, estimator=C.ESTIMATOR_NEE)
    ok = three_sigma(ref, nee, spp, spp)
    assert ok.mean() >= 0.985, (name, ok.mean())
    # no NaN or infinite radiance
    assert np.isfinite(nee["sum"]).all()


def test_variance_reduction_on_small_light(ctx):
    from illume_gb300 import synth
    sd = synth.cornell_scene(24, 24)
    spp = 512
    ref = render(ctx, sd, 24, 24, spp, 8, seed=3)
    nee = render(ctx, sd, 24, 24, spp, 8, seed=4, estimator=C.ESTIMATOR_NEE)

    def var(o):
        m = o["sum"] / spp
        return np.maximum(o["sumsq"] / spp - m * m, 0).mean()

    assert var(nee) < 0.5 * var(ref), (var(nee), var(ref))


def test_nee_jobs_same_alone_and_in_the_mix(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene, Server
    a = HostScene.from_data(ctx, synth.cornell_scene(32, 32))
    b = HostScene.from_data(ctx, synth.traversal_scene(tris=5000, env_size=(64, 32), width=32, height=24))

    def params(sc, w, h, spp, depth, est, seed):
        p = sc.default_params(spp, depth)
        p.width, p.height, p.seed, p.job, p.estimator = w, h, seed, seed, est
        return p

    jobs = [(a, params(a, 32, 32, 24, 8, C.ESTIMATOR_NEE, 1)), (b, params(b, 32, 24, 16, 12, C.ESTIMATOR_REFERENCE, 2)),
            (b, params(b, 32, 24, 20, 10, C.ESTIMATOR_NEE, 3)), (a, params(a, 16, 16, 40, 6, C.ESTIMATOR_REFERENCE, 4))]
    alone = []
    for sc, p in jobs:
        srv = Server(ctx)
        j = srv.submit(sc, p)
        srv.run()
        alone.append(srv.poll(j)["mean"])
        srv.close()
    srv = Server(ctx, path_capacity=30000)
    ids = [srv.submit(sc, p) for sc, p in jobs]
    srv.run()
    for k, j in enumerate(ids):
        assert np.array_equal(srv.poll(j)["mean"], alone[k], equal_nan=True), k
    srv.close()
