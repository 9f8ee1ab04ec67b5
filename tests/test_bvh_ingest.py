"""Scene ingest (BVH build) on the host: the build is identical on any number of host
threads, and the in-process BVH cache keyed by mesh content returns the build it
stored (the reference keeps a BVH cache file per OBJ, src/accel/bvh.cpp:399-439; this
library keeps the cache in memory and writes nothing next to the inputs)."""
import ctypes
import os
import subprocess
import sys

import numpy as np

from conftest import ROOT
from illume_gb300 import _capi as C

_DIGEST_SCRIPT = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
from illume_gb300 import _capi as C, synth
from illume_gb300.scenedata import Mesh, SceneData, Material
P, T = synth.displaced_icosphere(int(sys.argv[2]), seed=11)
s = SceneData()
m = s.add_material(Material(C.MAT_LAMBERT, s.constant((0.5, 0.5, 0.5)), s.constant((0, 0, 0))))
s.add_instance(s.add_mesh(Mesh(P, T)), m)
desc, keep = s.to_desc()
h = ctypes.c_void_p()
L = C.lib()
assert L.illume_scene_create(None, ctypes.byref(desc), ctypes.byref(h)) == C.OK
out = (ctypes.c_uint64 * 4)()
assert L.illume_scene_bvh_digest(h, 0, out) == C.OK
print(" ".join("%016x" % v for v in out))
L.illume_scene_destroy(h)
"""


def _digest_with_threads(freq, threads):
    env = dict(os.environ, ILLUME_BUILD_THREADS=str(threads))
    r = subprocess.run([sys.executable, "-c", _DIGEST_SCRIPT, ROOT, str(freq)], env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout.strip()


def test_bvh_identical_on_any_thread_count(native_lib):
    # 20 * 40^2 = 32,000 triangles: above the size at which subtrees are built in parallel
    digests = {t: _digest_with_threads(40, t) for t in (1, 3, 8)}
    assert len(set(digests.values())) == 1, digests


def _host_scene(P, T):
    from illume_gb300.scenedata import Mesh, SceneData, Material
    s = SceneData()
    m = s.add_material(Material(C.MAT_LAMBERT, s.constant((0.5, 0.5, 0.5)), s.constant((0, 0, 0))))
    s.add_instance(s.add_mesh(Mesh(P, T)), m)
    desc, keep = s.to_desc()
    h = ctypes.c_void_p()
    assert C.lib().illume_scene_create(None, ctypes.byref(desc), ctypes.byref(h)) == C.OK
    return h


def _stats():
    v = [ctypes.c_int64() for _ in range(4)]
    assert C.lib().illume_bvh_cache_stats(*[ctypes.byref(x) for x in v]) == C.OK
    return tuple(x.value for x in v)


def _digest(h):
    out = (ctypes.c_uint64 * 4)()
    assert C.lib().illume_scene_bvh_digest(h, 0, out) == C.OK
    return tuple(out)


def test_bvh_cache_hits_on_equal_content_and_returns_the_same_build(native_lib):
    from illume_gb300 import synth
    L = C.lib()
    assert L.illume_bvh_cache_clear() == C.OK
    e0, b0, h0, m0 = _stats()
    assert (e0, b0) == (0, 0)
    P, T = synth.displaced_icosphere(12, seed=3)
    a = _host_scene(P, T)
    da = _digest(a)
    e1, b1, h1, m1 = _stats()
    assert (e1, m1 - m0, h1 - h0) == (1, 1, 0) and b1 > 0
    b = _host_scene(P.copy(), T.copy())            # equal content in other buffers: a hit
    e2, b2, h2, m2 = _stats()
    assert (e2, m2 - m1, h2 - h1, b2) == (1, 0, 1, b1)
    assert _digest(b) == da
    P2 = P.copy()
    P2[0, 0] = np.nextafter(P2[0, 0], np.float32(np.inf))   # one ulp of one vertex: a new entry
    c = _host_scene(P2, T)
    e3, b3, h3, m3 = _stats()
    assert (e3, m3 - m2, h3 - h2) == (2, 1, 0) and b3 > b2
    assert _digest(c) != da
    for h in (a, b, c):
        L.illume_scene_destroy(h)
    assert L.illume_bvh_cache_clear() == C.OK
    e4, b4, h4, m4 = _stats()
    assert (e4, b4) == (0, 0)
    d = _host_scene(P, T)                          # built again after a clear: the same tree
    assert _stats()[3] == m4 + 1
    assert _digest(d) == da
    L.illume_scene_destroy(d)


def test_bvh_digest_rejects_a_bad_mesh_index(native_lib):
    from illume_gb300 import synth
    P, T = synth.displaced_icosphere(4, seed=1)
    h = _host_scene(P, T)
    out = (ctypes.c_uint64 * 4)()
    assert C.lib().illume_scene_bvh_digest(h, 1, out) == C.ERR_INVALID
    C.lib().illume_scene_destroy(h)


def test_concurrent_scene_builds_match_serial_builds(native_lib):
    """Host threads building, checking and digesting scenes at the same time (one scene per
    thread; the BVH cache and the build's own worker threads shared) give the trees a
    serial build gives: ctypes releases the interpreter lock for every library call, so
    the calls overlap."""
    import threading
    from illume_gb300 import synth
    L = C.lib()
    meshes = [synth.displaced_icosphere(f, seed=s) for f, s in ((14, 1), (20, 2), (14, 1), (42, 3), (20, 2), (8, 4))]
    assert L.illume_bvh_cache_clear() == C.OK
    serial = []
    for P, T in meshes:
        h = _host_scene(P, T)
        serial.append(_digest(h))
        L.illume_scene_destroy(h)
    assert L.illume_bvh_cache_clear() == C.OK
    results, errors = {}, []
    barrier = threading.Barrier(len(meshes))

    def work(i):
        try:
            P, T = meshes[i]
            barrier.wait(timeout=60)
            got = []
            for _ in range(3):
                h = _host_scene(P.copy(), T.copy())
                buf = ctypes.create_string_buffer(1 << 14)
                assert L.illume_scene_check_bvh(h, buf, len(buf)) == C.OK, buf.value
                got.append(_digest(h))
                L.illume_scene_destroy(h)
            results[i] = got
        except Exception as e:          # reported by the main thread
            errors.append((i, repr(e)))

    threads = [threading.Thread(target=work, args=(i,)) for i in range(len(meshes))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for i in range(len(meshes)):
        assert results[i] == [serial[i]] * 3, i
    entries = _stats()[0]
    assert entries == 4                    # four distinct meshes, each cached once
    assert L.illume_bvh_cache_clear() == C.OK
