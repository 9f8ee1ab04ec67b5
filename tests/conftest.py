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
