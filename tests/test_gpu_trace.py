"""Closest-hit parity on the GPU: the sm_103a traversal kernels against the oracle.

Instance, triangle and sphere indices must be bit-exact and t within 2 ulp (the kernels
evaluate the triangle tests operation by operation like the oracle, so t is expected to
be exact); barycentrics must match as well. Both BVH layouts and both triangle tests.
"""
import numpy as np
import pytest

from conftest import f32_normalize, golden_scene, rays6_to_8
from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu

KINDS = [(C.BVH_BINARY, C.ISECT_MT), (C.BVH_BINARY, C.ISECT_WATERTIGHT), (C.BVH_WIDE8, C.ISECT_MT),
         (C.BVH_WIDE8, C.ISECT_WATERTIGHT), (C.BVH_WIDE8_PERSISTENT, C.ISECT_MT),
         (C.BVH_WIDE8_PERSISTENT, C.ISECT_WATERTIGHT), (C.BVH_WIDE4, C.ISECT_MT), (C.BVH_WIDE4, C.ISECT_WATERTIGHT)]


def ulp(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


def scene_bounds(sd):
    pts = []
    for (m, mat, M, inv, ti) in sd.instances:
        P = sd.meshes[m].positions.astype(np.float64)
        pts.append(P @ M[:, :3].T + M[:, 3])
    for (c, r, mat) in sd.spheres:
        pts += [np.array([c]) - r, np.array([c]) + r]
    P = np.concatenate(pts)
    return P.min(0), P.max(0)


def ray_set(sd, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = scene_bounds(sd)
    ext = hi - lo
    lo, hi = lo - 0.1 * ext, hi + 0.1 * ext
    o = lo + rng.random((n, 3)) * (hi - lo)
    d = rng.normal(size=(n, 3))
    # a share of axis-parallel and coordinate-plane directions
    k = n // 16
    d[:k, 1:] = 0.0
    d[k:2 * k, 0] = 0.0
    d[2 * k:3 * k, :2] = 0.0
    d[:, :][np.abs(d).sum(1) == 0] = [0.0, 1.0, 0.0]
    r = np.concatenate([o, f32_normalize(d)], 1).astype(np.float32)
    # origins on mesh vertices (rays leaving a surface)
    m0 = sd.instances[0]
    P = sd.meshes[m0[0]].positions
    idx = rng.integers(0, len(P), size=k)
    M = m0[2]
    r[3 * k:4 * k, :3] = (P[idx].astype(np.float64) @ M[:, :3].T + M[:, 3]).astype(np.float32)
    return rays6_to_8(r)


def compare(sd, rays8, ctx, bvh, isect):
    from illume_gb300.api import HostScene
    from oracle import pyoracle
    scene = HostScene.from_data(ctx, sd)
    got = scene.trace_closest(rays8, intersector=isect, bvh_kind=bvh)
    want = pyoracle.OracleScene(sd).closest_hit(rays8, isect=isect)
    for k in ("inst", "prim", "sphere"):
        bad = np.nonzero(got[k] != want[k])[0]
        assert len(bad) == 0, (k, bvh, isect, bad[:5], got[k][bad[:5]], want[k][bad[:5]], got["t"][bad[:5]],
                               want["t"][bad[:5]])
    hit = want["inst"] >= 0
    assert ulp(got["t"], want["t"]).max() <= 2
    assert (got["t"] == want["t"]).all()
    assert np.array_equal(got["u"][hit], want["u"][hit]) and np.array_equal(got["v"][hit], want["v"][hit])
    return int((want["inst"] >= 0).sum() + (want["sphere"] >= 0).sum())


@pytest.mark.parametrize("name", ["box", "materials", "mesh", "textured"])
@pytest.mark.parametrize("bvh,isect", KINDS)
def test_golden_scenes(ctx, name, bvh, isect):
    sd = golden_scene(name)
    hits = compare(sd, ray_set(sd, 20000, seed=1), ctx, bvh, isect)
    assert hits > 1000


@pytest.mark.parametrize("bvh,isect", KINDS)
def test_displaced_icosphere(ctx, bvh, isect):
    from illume_gb300 import synth
    sd = synth.traversal_scene(tris=20000, env_size=(16, 8), width=64, height=64)
    compare(sd, ray_set(sd, 30000, seed=2), ctx, bvh, isect)


@pytest.mark.parametrize("bvh", [C.BVH_BINARY, C.BVH_WIDE8, C.BVH_WIDE8_PERSISTENT, C.BVH_WIDE4])
def test_camera_rays_full_size_mesh(ctx, bvh):
    """Primary rays of the 100k-triangle traversal scene (the benchmark's mesh)."""
    from illume_gb300 import synth
    from oracle import pyoracle
    sd = synth.traversal_scene(tris=100_000, env_size=(16, 8), width=128, height=128)
    cam = pyoracle.OracleScene(sd).camera_rays(128, 128, sample=0)
    compare(sd, rays6_to_8(cam), ctx, bvh, C.ISECT_WATERTIGHT)


def test_empty_and_miss(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene
    sd = synth.cornell_scene(16, 16)
    scene = HostScene.from_data(ctx, sd)
    assert len(scene.trace_closest(np.zeros((0, 8), np.float32))["t"]) == 0
    r = np.zeros((2, 8), np.float32)
    r[:, :3] = [278, 273, -800]
    r[0, 4:7] = [0, 0, -1]          # away from the box: miss
    r[1, 4:7] = [0, 0, 1]
    h = scene.trace_closest(r)
    assert h["inst"][0] == -1 and h["sphere"][0] == -1 and h["t"][0] == np.finfo(np.float32).max
    assert h["inst"][1] == 2        # back wall


@pytest.mark.parametrize("bvh", [C.BVH_WIDE4, C.BVH_BINARY])
def test_full_ray_sets_on_the_benchmark_mesh(ctx, bvh):
    """2^20 seeded rays (origins in the scene box inflated 10%, directions on the sphere,
    with axis-parallel shares and origins on mesh vertices) plus the 2^20 primary rays of
    the 1024x1024 camera, on the 100k-triangle traversal scene: bit-exact against the
    oracle, watertight test."""
    from illume_gb300 import synth
    from oracle import pyoracle
    sd = synth.traversal_scene(tris=100_000, env_size=(16, 8), width=1024, height=1024)
    compare(sd, ray_set(sd, 1 << 20, seed=3), ctx, bvh, C.ISECT_WATERTIGHT)
    cam = pyoracle.OracleScene(sd).camera_rays(1024, 1024, sample=0)
    assert len(cam) == 1 << 20
    hits = compare(sd, rays6_to_8(cam), ctx, bvh, C.ISECT_WATERTIGHT)
    assert hits > (1 << 18)
