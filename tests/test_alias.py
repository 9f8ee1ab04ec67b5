"""Alias tables of the next-event estimator's light choice (host code, CPU): every table
must give each slot exactly its weight's share of probability, including zero weights,
a single slot and weights spanning many orders of magnitude."""
import ctypes

import numpy as np
import pytest

from illume_gb300 import _capi as C


def table(w):
    w = np.ascontiguousarray(w, np.float64)
    n = len(w)
    keep = np.zeros(n, np.float32)
    alias = np.zeros(n, np.int32)
    st = C.lib().illume_alias_table(n, w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), C.fptr(keep),
                                    alias.ctypes.data_as(C._pi32))
    return st, keep, alias


def implied(keep, alias):
    n = len(keep)
    p = keep.astype(np.float64).copy()
    np.add.at(p, alias, 1.0 - keep.astype(np.float64))
    return p / n


@pytest.mark.parametrize("seed", range(12))
def test_probabilities_match_weights(native_lib, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 3000))
    w = rng.random(n) ** int(rng.integers(1, 8))
    w[rng.random(n) < 0.1] = 0.0
    if w.sum() == 0:
        w[0] = 1.0
    st, keep, alias = table(w)
    assert st == C.OK
    assert ((keep >= 0) & (keep <= 1)).all() and ((alias >= 0) & (alias < n)).all()
    assert np.allclose(implied(keep, alias), w / w.sum(), rtol=1e-5, atol=1e-9)
    assert (implied(keep, alias)[w == 0] < 1e-7).all()


def test_edge_cases(native_lib):
    st, keep, alias = table([5.0])
    assert st == C.OK and keep[0] == 1.0 and alias[0] == 0
    st, keep, alias = table([1e-30, 1.0, 1e30])
    assert st == C.OK
    assert np.allclose(implied(keep, alias), np.array([1e-30, 1.0, 1e30]) / (1e30 + 1.0 + 1e-30), atol=1e-7)
    st, _, _ = table([0.0, 0.0])
    assert st == C.ERR_INVALID
