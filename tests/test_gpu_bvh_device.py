"""Scene ingest on the device (illume_context_set_bvh_builder), on the GPU.

The device builder sorts a mesh's triangles by the Morton code of their box centroids and
merges mutual nearest clusters within 16 positions (locally-ordered clustering); the host
makes leaves and node layouts from that tree. Its trees differ from the host's binned SAH
trees; the closest hits may not: a hit is decided by the triangle tests, ties going to
the lower primitive index, so every hit record and every image must equal the host-built
scene's. The reference builds its tree on one host thread (src/accel/bvh.cpp:65-439)."""
import ctypes

import numpy as np
import pytest

from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def build_both(ctx, sd):
    from illume_gb300.api import HostScene
    ctx.set_bvh_builder(C.BVH_BUILD_HOST)
    host = HostScene.from_data(ctx, sd)
    ctx.set_bvh_builder(C.BVH_BUILD_DEVICE)
    try:
        dev = HostScene.from_data(ctx, sd)
    finally:
        ctx.set_bvh_builder(C.BVH_BUILD_HOST)
    return host, dev


def meshes_with_triangles(sd):
    return sum(1 for m in sd.meshes if len(m.tris) > 0)


def scenes():
    from illume_gb300 import synth
    from conftest import golden_scene
    return {"traversal": lambda: synth.traversal_scene(tris=20000, env_size=(64, 32), width=64, height=48),
            "instanced": lambda: synth.instanced_scene(16, 3000, seed=5, env=synth.environment_map(1, 64, 32)),
            "mesh": lambda: golden_scene("mesh"),
            "cornell": lambda: synth.cornell_scene(48, 48),
            "subsurface": lambda: synth.sss_scene(tris=20000, width=48, height=36)}


def random_rays(sd, n, seed):
    from illume_gb300 import synth
    lo, hi = synth.scene_bounds(sd)
    c, ext = 0.5 * (lo + hi), (hi - lo).max()
    rng = np.random.default_rng(seed)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = c + rng.uniform(-0.75, 0.75, (n, 3)) * ext
    d = rng.normal(size=(n, 3))
    r[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    # a quarter of the rays aimed at triangle centroids, so most of those hit
    m = sd.meshes[0]
    if len(m.tris):
        M = sd.instances[0][2].astype(np.float64)
        k = n // 4
        tri = m.tris[rng.integers(0, len(m.tris), k)]
        cen = m.positions[tri].astype(np.float64).mean(1) @ M[:, :3].T + M[:, 3]
        v = cen - r[:k, 0:3]
        r[:k, 4:7] = v / np.linalg.norm(v, axis=1, keepdims=True)
    return r


@pytest.mark.parametrize("name", ["traversal", "instanced", "mesh", "cornell", "subsurface"])
def test_device_trees_keep_the_invariants(ctx, name):
    sd = scenes()[name]()
    host, dev = build_both(ctx, sd)
    report = dev.check_bvh()
    info = dev.build_info()
    assert info["device_meshes"] == meshes_with_triangles(sd), report
    assert "replaced" not in report, report
    assert host.build_info()["device_meshes"] == 0
    host.close()
    dev.close()


@pytest.mark.parametrize("name", ["traversal", "instanced", "mesh", "subsurface"])
@pytest.mark.parametrize("bvh", [C.BVH_WIDE4, C.BVH_BINARY, C.BVH_WIDE8])
def test_device_trees_give_the_same_closest_hits(ctx, name, bvh):
    sd = scenes()[name]()
    host, dev = build_both(ctx, sd)
    rays = random_rays(sd, 1 << 16, seed=3)
    for isect in (C.ISECT_MT, C.ISECT_WATERTIGHT):
        a = host.trace_closest(rays, intersector=isect, bvh_kind=bvh)
        b = dev.trace_closest(rays, intersector=isect, bvh_kind=bvh)
        assert (a["inst"] >= 0).mean() > 0.1
        for k in ("t", "u", "v", "inst", "prim", "sphere"):
            assert np.array_equal(a[k], b[k], equal_nan=True), (k, isect)
    host.close()
    dev.close()


@pytest.mark.parametrize("name", ["traversal", "instanced", "cornell", "subsurface"])
@pytest.mark.parametrize("bvh", [C.BVH_WIDE4, C.BVH_BINARY, C.BVH_WIDE8])
def test_device_trees_give_the_same_image(ctx, name, bvh):
    from illume_gb300.api import Renderer
    sd = scenes()[name]()
    host, dev = build_both(ctx, sd)
    out = []
    for sc in (host, dev):
        p = sc.default_params(8, 12)
        p.width, p.height, p.accum_mode, p.bvh_kind = 48, 40, C.ACCUM_FP64, bvh
        r = Renderer(ctx, sc, params=p)
        out.append(r.render(mean=False, sums=True))
        r.close()
    assert np.array_equal(out[0]["sum"], out[1]["sum"], equal_nan=True)
    assert out[0]["stats"].rays == out[1]["stats"].rays
    host.close()
    dev.close()


def _mesh_scene(P, T):
    from illume_gb300.scenedata import Material, Mesh, SceneData
    s = SceneData()
    m = s.add_material(Material(C.MAT_LAMBERT, s.constant((0.5, 0.5, 0.5)), s.constant((0, 0, 0))))
    s.add_instance(s.add_mesh(Mesh(np.asarray(P, np.float32), np.asarray(T, np.int32))), m)
    s.width = s.height = 16
    return s


@pytest.mark.parametrize("case", ["1", "2", "3", "5", "17", "coincident", "collinear_centroids"])
def test_device_build_of_small_and_degenerate_meshes(ctx, case):
    from illume_gb300 import synth
    rng = np.random.default_rng(7)
    if case.isdigit():
        n = int(case)
        P = rng.uniform(-1, 1, (3 * n, 3))
        T = np.arange(3 * n).reshape(n, 3)
    elif case == "coincident":                      # 40 copies of one triangle: every key equal
        P = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64)
        T = np.zeros((40, 3), np.int64) + np.array([0, 1, 2])
    else:                                           # centroids on one line, far apart
        n = 64
        x = np.arange(n, dtype=np.float64) * 10.0
        P = np.stack([np.stack([x, np.zeros(n), np.zeros(n)], 1), np.stack([x + 1, np.zeros(n), np.zeros(n)], 1),
                      np.stack([x, np.ones(n), np.zeros(n)], 1)], 1).reshape(-1, 3)
        T = np.arange(3 * n).reshape(n, 3)
    sd = _mesh_scene(P, T)
    host, dev = build_both(ctx, sd)
    dev.check_bvh()
    assert dev.build_info()["device_meshes"] == 1
    rays = random_rays(sd, 4096, seed=11)
    for bvh in (C.BVH_WIDE4, C.BVH_BINARY, C.BVH_WIDE8):
        a = host.trace_closest(rays, intersector=C.ISECT_WATERTIGHT, bvh_kind=bvh)
        b = dev.trace_closest(rays, intersector=C.ISECT_WATERTIGHT, bvh_kind=bvh)
        for k in ("t", "inst", "prim"):
            assert np.array_equal(a[k], b[k], equal_nan=True), (k, bvh)
    host.close()
    dev.close()


def _digest(scene):
    out = (ctypes.c_uint64 * 4)()
    C.check(C.lib().illume_scene_bvh_digest(scene.handle, 0, out))
    return tuple(out)


def test_device_build_is_deterministic_and_cached_apart_from_the_host_build(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene
    L = C.lib()
    P, T = synth.displaced_icosphere(synth.freq_for_tris(30000), seed=4)
    sd = _mesh_scene(P, T)
    assert L.illume_bvh_cache_clear() == C.OK
    host, dev = build_both(ctx, sd)
    v = [ctypes.c_int64() for _ in range(4)]
    L.illume_bvh_cache_stats(*[ctypes.byref(x) for x in v])
    assert v[0].value == 2                          # one entry per builder
    assert _digest(host) != _digest(dev)
    assert L.illume_bvh_cache_clear() == C.OK        # built again on the device: the same tree
    ctx.set_bvh_builder(C.BVH_BUILD_DEVICE)
    again = HostScene.from_data(ctx, sd)
    ctx.set_bvh_builder(C.BVH_BUILD_HOST)
    assert _digest(again) == _digest(dev)
    for s in (host, dev, again):
        s.close()
    assert L.illume_bvh_cache_clear() == C.OK


def test_device_build_of_a_large_mesh(ctx):
    """700k triangles: the device build is faster than the host build (printed), and its
    trees keep every invariant."""
    from illume_gb300 import synth
    P, T = synth.displaced_icosphere(synth.freq_for_tris(700_000), seed=3)
    sd = _mesh_scene(P, T)
    assert C.lib().illume_bvh_cache_clear() == C.OK
    host, dev = build_both(ctx, sd)
    hi, di = host.build_info(), dev.build_info()
    report = dev.check_bvh()
    print(f"BVH_BUILD host {hi['build_ms']:.1f} ms, device {di['build_ms']:.1f} ms: {report.strip()}")
    assert di["device_meshes"] == 1
    assert di["build_ms"] < hi["build_ms"]
    rays = random_rays(sd, 1 << 15, seed=5)
    a = host.trace_closest(rays, intersector=C.ISECT_MT, bvh_kind=C.BVH_WIDE4)
    b = dev.trace_closest(rays, intersector=C.ISECT_MT, bvh_kind=C.BVH_WIDE4)
    assert np.array_equal(a["t"], b["t"]) and np.array_equal(a["prim"], b["prim"])
    host.close()
    dev.close()
    assert C.lib().illume_bvh_cache_clear() == C.OK


def test_bvh_builder_is_checked(ctx):
    assert C.lib().illume_context_set_bvh_builder(ctx.handle, 2) == C.ERR_INVALID
    assert C.lib().illume_context_set_bvh_builder(None, 0) == C.ERR_INVALID
