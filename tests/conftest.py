import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
SCENES = os.path.join(GOLDEN, "scenes")
for p in (ROOT, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def pytest_collection_modifyitems(config, items):
    # files collect in name order; keep that order (tests/test_zz_* run last)
    pass


@pytest.fixture(scope="session")
def native_lib():
    """The in-tree native library; built here if missing, never replaced by a fallback."""
    from illume_gb300 import _capi, build
    if not os.path.exists(_capi.LIB_PATH):
        build.build()
    return _capi.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle.lib()


@pytest.fixture(scope="session")
def ctx(native_lib):
    import torch  # noqa: F401  (only to fail fast with a clear message when CUDA is absent)
    from illume_gb300.api import Context
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    c = Context(0)
    yield c
    c.close()


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def golden_scene(name):
    import golden_io
    return golden_io.scene_from_arrays(golden(f"ref_scene_{name}.npz"))


def f32_normalize(d):
    """Normalise float32 directions the way the reference does (reciprocal length)."""
    d = np.asarray(d, np.float32)
    l2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    inv = np.float32(1.0) / np.sqrt(l2)
    return (d * inv[:, None]).astype(np.float32)


def rays6_to_8(r6):
    r8 = np.zeros((len(r6), 8), np.float32)
    r8[:, :3] = r6[:, :3]
    r8[:, 4:7] = r6[:, 3:6]
    return r8


def render_pin_scene():
    """The reference's cornell_box.json as its own loader parses it, with the linear
    radiance bounds of its shipped 100,000-spp render (tests/golden/make_render_pin.py)."""
    import golden_io
    z = golden("ref_render_pin_cornell.npz")
    return golden_io.scene_from_arrays(z), z


def render_pin_check(s, s2, spp, width, pin, z_limit=4.0, return_mask=False):
    """Region means of a render (per-pixel radiance sums s and sums of squares s2 over
    spp samples, width x width pixels) against the pinned render's bounds: returns the
    regions (of the usable ones) lying more than z_limit standard errors outside their
    bounds (their count, or with return_mask their mask), the number of usable regions,
    and per channel the same distance for the mean over all usable regions."""
    g = pin["region_lo"].shape[0]
    k = width // g
    m = (np.asarray(s, np.float64) / spp).reshape(width, width, 3)
    var = np.maximum((np.asarray(s2, np.float64) / spp).reshape(width, width, 3) - m * m, 0.0)
    reg = m.reshape(g, k, g, k, 3).mean(axis=(1, 3))
    se = np.sqrt(var.reshape(g, k, g, k, 3).sum(axis=(1, 3)) / spp) / (k * k)
    lo, hi, ok = pin["region_lo"], pin["region_hi"], pin["region_usable"]
    outside = np.maximum(lo - reg, 0.0) + np.maximum(reg - hi, 0.0)
    far = (outside > z_limit * np.maximum(se, 1e-300)).any(axis=-1) & ok
    t, tlo, thi = reg[ok].mean(axis=0), lo[ok].mean(axis=0), hi[ok].mean(axis=0)
    tse = np.sqrt((se[ok] ** 2).sum(axis=0)) / ok.sum()
    image_z = (np.maximum(tlo - t, 0.0) + np.maximum(t - thi, 0.0)) / tse
    return (far if return_mask else int(far.sum())), int(ok.sum()), image_z
