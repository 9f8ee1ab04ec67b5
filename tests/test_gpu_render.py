"""Image parity on the GPU.

* Same Philox streams as the reference and the oracle: with the reference's
  Moller-Trumbore test the GPU render equals the reference integrator's render of the
  golden scenes path by path (FP32 transcendentals on the GPU differ from glibc's by an
  ulp, so a few paths may diverge; per-pixel tolerance 1e-4 relative on >= 99%).
* Converged images: a per-pixel 3-sigma test against the FP64 oracle rendered with
  independent samples (different seed): failing fraction <= 0.5% on the full 256x256
  Cornell frame, <= 1% on the small golden crops.
* Accumulation modes, progressive and sharded renders, tonemap output.
"""
import numpy as np
import pytest

from conftest import golden, golden_scene
from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def render(ctx, sd, w, h, spp, depth, **kw):
    from illume_gb300.api import HostScene, Renderer
    scene = HostScene.from_data(ctx, sd)
    p = scene.default_params(spp, depth)
    p.width, p.height = w, h
    fields = {f[0] for f in type(p)._fields_}
    for k, v in kw.items():
        assert k in fields, k     # a ctypes structure would take a misspelt name silently
        setattr(p, k, v)
    r = Renderer(ctx, scene, params=p)
    out = r.render(mean=True, sums=True, rgb8=True)
    out["renderer"], out["scene"] = r, scene
    return out


@pytest.mark.parametrize("name", ["box", "materials", "mesh", "textured"])
@pytest.mark.parametrize("bvh", [C.BVH_BINARY, C.BVH_WIDE8, C.BVH_WIDE8_PERSISTENT, C.BVH_WIDE4])
def test_matches_reference_render(ctx, name, bvh):
    z = golden(f"ref_scene_{name}.npz")
    sd = golden_scene(name)
    w, h, spp, depth = (int(v) for v in z["render_size"])
    out = render(ctx, sd, w, h, spp, depth, intersector=C.ISECT_MT, bvh_kind=bvh, accum_mode=C.ACCUM_FP64)
    ref = z["render_sum"].astype(np.float64)
    rel = np.abs(out["sum"] - ref) / np.maximum(np.abs(ref), 1e-3)
    frac = (rel.max(1) < 1e-4).mean()
    assert frac >= 0.99, frac
    rays = out["stats"].rays
    assert abs(rays - int(z["render_rays"])) <= 0.01 * int(z["render_rays"])
    assert (out["rgb8"] == z["render_rgb8"]).all(1).mean() >= 0.98


@pytest.mark.parametrize("name", ["box", "materials", "mesh", "textured"])
def test_matches_oracle_watertight(ctx, name):
    from oracle import pyoracle
    sd = golden_scene(name)
    w, h, spp, depth = 32, 24, 4, 10
    out = render(ctx, sd, w, h, spp, depth, accum_mode=C.ACCUM_FP64, seed=7)
    s, s2, rays = pyoracle.OracleScene(sd).render(w, h, spp, depth, seed=7, isect=C.ISECT_WATERTIGHT, precision=32)
    rel = np.abs(out["sum"] - s) / np.maximum(np.abs(s), 1e-3)
    assert (rel.max(1) < 1e-4).mean() >= 0.99
    assert abs(out["stats"].rays - rays) <= 0.01 * rays


def test_traversal_scene_matches_oracle(ctx):
    from illume_gb300 import synth
    from oracle import pyoracle
    sd = synth.traversal_scene(tris=20000, env_size=(256, 128), width=64, height=64)
    out = render(ctx, sd, 64, 64, 4, 25, accum_mode=C.ACCUM_FP64)
    s, s2, rays = pyoracle.OracleScene(sd).render(64, 64, 4, 25, isect=C.ISECT_WATERTIGHT, precision=32)
    rel = np.abs(out["sum"] - s) / np.maximum(np.abs(s), 1e-2)
    assert (rel.max(1) < 1e-4).mean() >= 0.98
    assert abs(out["stats"].rays - rays) <= 0.01 * rays


def three_sigma(gpu_sum, gpu_sq, n_gpu, ref_sum, ref_sq, n_ref):
    mg, mr = gpu_sum / n_gpu, ref_sum / n_ref
    vg = np.maximum(gpu_sq / n_gpu - mg * mg, 0) / n_gpu
    vr = np.maximum(ref_sq / n_ref - mr * mr, 0) / n_ref
    sig = np.sqrt(vg + vr)
    ok = np.abs(mg - mr) <= 3 * sig + 1e-9
    return ok


@pytest.mark.parametrize("name", ["box", "materials"])
def test_three_sigma_against_fp64_oracle(ctx, name):
    from oracle import pyoracle
    sd = golden_scene(name)
    w, h = (24, 24) if name == "box" else (32, 24)
    depth = 8
    out = render(ctx, sd, w, h, 512, depth, accum_mode=C.ACCUM_FP64, seed=11)
    s, s2, _ = pyoracle.OracleScene(sd).render(w, h, 256, depth, seed=12345, isect=C.ISECT_WATERTIGHT, precision=64)
    ok = three_sigma(out["sum"], out["sumsq"], 512, s, s2, 256)
    assert ok.mean() >= 0.99, ok.mean()


def test_three_sigma_full_cornell_frame(ctx):
    """The plain small configuration (the Cornell box of five quads with a mirror and a
    dielectric sphere, 256x256, depth 8): every pixel's GPU mean against the FP64
    oracle's, 1024 independent samples each, |mu_gpu - mu_ref| <= 3 sqrt(s2_gpu/n_gpu +
    s2_ref/n_ref) on all three channels. Under a Gaussian model a channel fails with
    probability 0.27%; the caustics of the small light through the spheres make the
    per-pixel distributions heavy tailed, so the bar is set from two independent oracle
    renders of this frame at 1024 samples each, which fail on 0.34% of pixels (0.20% of
    channels): at most 0.5% of pixels may fail, 3.2 binomial standard deviations above
    that rate over 65,536 pixels. (Unequal sample counts are avoided: the side with
    fewer samples misses rare caustic paths and understates its variance, and 1024
    against 256 samples fails 3.8% of pixels even between two oracle renders.)"""
    from illume_gb300 import synth
    from oracle import pyoracle
    w = h = 256
    n = 1024
    sd = synth.cornell_scene(w, h)
    out = render(ctx, sd, w, h, n, 8, accum_mode=C.ACCUM_FP64, seed=31)
    s, s2, _ = pyoracle.OracleScene(sd).render(w, h, n, 8, seed=4242, isect=C.ISECT_WATERTIGHT, precision=64)
    ok = three_sigma(out["sum"], out["sumsq"], n, s, s2, n).all(1)
    npx = ok.size
    fails = int(npx - ok.sum())
    p0 = 0.0034
    z = (fails - npx * p0) / np.sqrt(npx * p0 * (1 - p0))
    assert fails / npx <= 0.005, (fails, npx, z)


@pytest.mark.parametrize("isect", [C.ISECT_MT, C.ISECT_WATERTIGHT])
def test_matches_the_reference_shipped_render(ctx, isect):
    """The reference's one shipped render (renders/cornell-1024x1024-100000spp-100md.png of
    res/scenes/cornell_box.json, depth 100, from an older revision with cuRAND streams:
    a statistical pin). The reference's present code, built for the host, lies more than
    4 standard errors outside the render's linear radiance bounds in 5 of its 16 x 16
    regions in a 128x128 render at 2048 spp (tests/golden/make_render_pin.py); the GPU's
    render of the same size, samples and streams, of the scene as the reference's
    loader parsed it, may lie outside in those regions and in at most 1% more, and its
    image mean within 4 standard errors of the bounds, with either triangle test."""
    from conftest import render_pin_check, render_pin_scene
    sd, pin = render_pin_scene()
    w, spp = int(pin["ref_code_res"]), int(pin["ref_code_spp"])
    out = render(ctx, sd, w, w, spp, int(pin["render_depth"]), accum_mode=C.ACCUM_FP64, intersector=isect)
    far, usable, image_z = render_pin_check(out["sum"], out["sumsq"], spp, w, pin, return_mask=True)
    out["renderer"].close()
    out["scene"].close()
    known = pin["ref_code_far"]
    assert usable >= 240 and known.sum() <= 0.05 * usable
    assert (far & ~known).sum() <= 0.01 * usable, np.argwhere(far & ~known)
    assert (image_z <= 4.0).all(), image_z


def test_exact_hg_matches_the_oracle(ctx):
    """The opt-in exact Henyey-Greenstein sampler (sin theta = sqrt(1 - cos^2 theta); the
    reference's sampler, src/math/sample.cu:36-52, takes sqrt(1 - cos theta)): path by
    path against the oracle's exact sampler on the golden scene with a medium, and
    different from the reference sampler's image."""
    from oracle import pyoracle
    sd = golden_scene("materials")
    assert len(sd.mediums) > 0
    w, h, spp, depth = 32, 24, 8, 16
    out = render(ctx, sd, w, h, spp, depth, accum_mode=C.ACCUM_FP64, seed=5, exact_hg=1)
    ora = pyoracle.OracleScene(sd)
    s, _, rays = ora.render(w, h, spp, depth, seed=5, isect=C.ISECT_WATERTIGHT, precision=32, exact_hg=1)
    rel = np.abs(out["sum"] - s) / np.maximum(np.abs(s), 1e-3)
    assert (rel.max(1) < 1e-4).mean() >= 0.99
    assert abs(out["stats"].rays - rays) <= 0.01 * rays
    s_ref, _, _ = ora.render(w, h, spp, depth, seed=5, isect=C.ISECT_WATERTIGHT, precision=32, exact_hg=0)
    assert not np.allclose(s_ref, s, rtol=1e-4)


def test_accumulation_modes_agree(ctx):
    from illume_gb300 import synth
    sd = synth.cornell_scene(32, 32)
    res = {m: render(ctx, sd, 32, 32, 64, 8, accum_mode=m, seed=3)["sum"] for m in (C.ACCUM_FP32, C.ACCUM_KAHAN, C.ACCUM_FP64)}
    ref = res[C.ACCUM_FP64]
    for m in (C.ACCUM_FP32, C.ACCUM_KAHAN):
        rel = np.abs(res[m] - ref) / np.maximum(np.abs(ref), 1e-3)
        assert rel.max() < 1e-4
    # the compensated sum is closer to the FP64 sum than the plain FP32 sum
    e32 = np.abs(res[C.ACCUM_FP32] - ref).sum()
    ek = np.abs(res[C.ACCUM_KAHAN] - ref).sum()
    assert ek <= e32


def test_progressive_and_sharded_sums_are_exact(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene, Renderer
    sd = synth.cornell_scene(24, 24)
    full = render(ctx, sd, 24, 24, 16, 8, accum_mode=C.ACCUM_FP64, samples_per_pass=3)["sum"]
    scene = HostScene.from_data(ctx, sd)
    p = scene.default_params(8, 8)
    p.width = p.height = 24
    p.accum_mode = C.ACCUM_FP64
    r = Renderer(ctx, scene, params=p)
    r.render_device(accumulate=False)
    r.render_device(accumulate=True)
    prog = r.read(mean=False, sums=True)["sum"]
    assert np.array_equal(prog, full)
    # shard: samples [8, 16) rendered separately
    a = render(ctx, sd, 24, 24, 8, 8, accum_mode=C.ACCUM_FP64)["sum"]
    b = render(ctx, sd, 24, 24, 8, 8, accum_mode=C.ACCUM_FP64, sample_begin=8)["sum"]
    np.testing.assert_allclose(a + b, full, rtol=1e-12, atol=1e-12)


def test_render_to_bitmap_and_tonemap(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import Bitmap, HostScene, Renderer
    from oracle import pyoracle
    sd = synth.cornell_scene(40, 30)
    scene = HostScene.from_data(ctx, sd)
    for op in range(4):
        r = Renderer(ctx, scene, spp=8, max_depth=6, tonemapper=op, width=40, height=30)
        bm = Bitmap(40, 30)
        st = r.render_to_bitmap(bm)
        assert st.rays > 0 and st.kernel_launches > 0
        rgb = bm.rgb8().reshape(-1, 3)
        m = r.read(mean=False, sums=True)["sum"]
        want = pyoracle.tonemap_image(m.astype(np.float32), 8.0, op)
        assert np.abs(rgb.astype(int) - want.astype(int)).max() <= 1
        assert (rgb == want).all(1).mean() >= 0.99


def test_accumulator_precision_at_high_spp(ctx):
    """20,000 samples per pixel: against the FP64 sum of the same samples, the compensated
    FP32 sum stays within a few FP32 ulps while the plain FP32 sum drifts further."""
    from illume_gb300 import synth
    sd = synth.cornell_scene(8, 8)
    res = {m: render(ctx, sd, 8, 8, 20000, 8, accum_mode=m, seed=21)["sum"] for m in (C.ACCUM_FP32, C.ACCUM_KAHAN, C.ACCUM_FP64)}
    ref = res[C.ACCUM_FP64]
    scale = np.maximum(np.abs(ref), 1e-6)
    ek = np.abs(res[C.ACCUM_KAHAN] - ref) / scale
    e32 = np.abs(res[C.ACCUM_FP32] - ref) / scale
    assert ek.max() < 4e-7, ek.max()
    assert e32.mean() > 4 * ek.mean()
    assert e32.max() < 1e-2
