"""The command line front end, the reference's `illume <save> <scene.json> <spp> <maxdepth>`:
its usage reply, the output name, and (GPU) that the image it writes is the library's
render of the same scene and settings."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import SCENES


def cli():
    from illume_gb300 import build
    if not os.path.exists(build.CLI):
        build.build()
    return build.CLI


def test_usage_with_too_few_arguments(native_lib):
    out = subprocess.run([cli(), "a", "b"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0
    assert "usage" in out.stdout


def read_pfm(path):
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        w, h = (int(v) for v in f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(), dtype="<f4" if scale < 0 else ">f4").reshape(h, w, 3)
    return np.flipud(data)   # PFM rows run bottom to top


@pytest.mark.gpu
def test_render_writes_the_libraries_image(ctx, tmp_path):
    from illume_gb300.api import HostScene, Renderer
    work = tmp_path / "scene"
    shutil.copytree(SCENES, work)
    out = subprocess.run([cli(), str(tmp_path / "shot"), "box.json", "6", "5", "--pfm"], cwd=work,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert "Rays per sec" in out.stdout
    names = sorted(p.name for p in tmp_path.iterdir() if p.name.startswith("shot-"))
    png = [n for n in names if n.endswith(".png")]
    assert len(png) == 1 and png[0].endswith("spp-5md.png") and "-6spp-" in png[0]
    assert (tmp_path / png[0]).read_bytes()[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = (int(v) for v in png[0].split("-")[1].split("x"))
    img = read_pfm(str(tmp_path / png[0].replace(".png", ".pfm")))
    assert img.shape == (h, w, 3)
    # the same render through the library
    cwd = os.getcwd()
    os.chdir(work)
    try:
        from illume_gb300 import _capi as C
        import ctypes
        hnd = ctypes.c_void_p()
        C.check(C.lib().illume_scene_load_json(ctx.handle, b"box.json", None, ctypes.byref(hnd)))
        scene = HostScene(ctx, hnd)
        r = Renderer(ctx, scene, spp=6, max_depth=5)
        want = r.render(mean=True)["mean"].reshape(h, w, 3)
    finally:
        os.chdir(cwd)
    assert np.array_equal(img, want)
