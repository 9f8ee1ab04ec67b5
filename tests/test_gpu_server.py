"""Served rendering: jobs admitted by device-memory footprint, progressive samples
interleaved across running jobs; every job's image is the same alone and in the mix."""
import ctypes

import numpy as np
import pytest

from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def make_server(ctx, budget=0, slots=8):
    s = ctypes.c_void_p()
    C.check(C.lib().illume_server_create(ctx.handle, budget, slots, ctypes.byref(s)))
    return s


def run_all(server, ids, npix):
    L = C.lib()
    running = ctypes.c_int(1)
    steps = 0
    while running.value:
        C.check(L.illume_server_step(server, ctypes.byref(running)))
        steps += 1
        assert steps < 10000
    out = {}
    for j, n in zip(ids, npix):
        m = np.zeros((n, 3), np.float32)
        st = C.RenderStats()
        C.check(L.illume_job_poll(server, j, C.fptr(m), None, ctypes.byref(st)))
        out[j] = (m, st)
    return out


def params(scene, w, h, spp, depth, seed=0, job=0):
    p = scene.default_params(spp, depth)
    p.width, p.height, p.seed, p.job = w, h, seed, job
    return p


def test_same_alone_and_in_the_mix(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene
    L = C.lib()
    a = HostScene.from_data(ctx, synth.cornell_scene(48, 48))
    b = HostScene.from_data(ctx, synth.traversal_scene(tris=5000, env_size=(64, 32), width=64, height=48))
    jobs = [(a, params(a, 48, 48, 40, 8, seed=1, job=1)), (b, params(b, 64, 48, 24, 12, seed=2, job=2)),
            (a, params(a, 32, 24, 64, 6, seed=3, job=3))]
    alone = []
    for sc, p in jobs:
        srv = make_server(ctx)
        jid = ctypes.c_int64()
        C.check(L.illume_job_submit(srv, sc.handle, ctypes.byref(p), ctypes.byref(jid)))
        alone.append(run_all(srv, [jid.value], [p.width * p.height])[jid.value][0])
        L.illume_server_destroy(srv)
    srv = make_server(ctx)
    ids = []
    for sc, p in jobs:
        jid = ctypes.c_int64()
        C.check(L.illume_job_submit(srv, sc.handle, ctypes.byref(p), ctypes.byref(jid)))
        ids.append(jid.value)
    mixed = run_all(srv, ids, [p.width * p.height for _, p in jobs])
    for k, j in enumerate(ids):
        assert np.array_equal(mixed[j][0], alone[k]), k
        assert mixed[j][1].rays > 0
    L.illume_server_destroy(srv)


def test_budget_admission_and_cancel(ctx):
    from illume_gb300 import synth
    from illume_gb300.api import HostScene
    L = C.lib()
    sc = HostScene.from_data(ctx, synth.cornell_scene(64, 64))
    p = params(sc, 64, 64, 16, 6)
    srv = make_server(ctx, budget=1 << 20)   # far below one job's footprint
    jid = ctypes.c_int64()
    assert L.illume_job_submit(srv, sc.handle, ctypes.byref(p), ctypes.byref(jid)) == C.ERR_BUDGET
    L.illume_server_destroy(srv)
    srv = make_server(ctx, budget=64 << 20, slots=1)
    ids = []
    for k in range(3):
        C.check(L.illume_job_submit(srv, sc.handle, ctypes.byref(p), ctypes.byref(jid)))
        ids.append(jid.value)
    C.check(L.illume_job_cancel(srv, ids[1]))
    running = ctypes.c_int(1)
    while running.value:
        C.check(L.illume_server_step(srv, ctypes.byref(running)))
    m = np.zeros((64 * 64, 3), np.float32)
    assert L.illume_job_poll(srv, ids[0], C.fptr(m), None, None) == C.OK
    assert L.illume_job_poll(srv, ids[1], C.fptr(m), None, None) == C.ERR_CANCELLED
    assert L.illume_job_poll(srv, ids[2], C.fptr(m), None, None) == C.OK
    L.illume_server_destroy(srv)
