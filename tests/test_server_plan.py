"""Host logic of the render server: how running jobs split a job table's path slots.

Every pass gives job i per_pass[i] samples of each of its npix[i] pixels. The split must
fit the slots, give every job at least one sample, never exceed a job's remaining
samples, and leave no slots idle that some unfinished job could still use.
"""
import numpy as np
import pytest

from illume_gb300 import _capi as C


def plan(npix, left, cap):
    n = len(npix)
    a = np.ascontiguousarray(npix, np.int32)
    b = np.ascontiguousarray(left, np.int32)
    out = np.zeros(n, np.int32)
    st = C.lib().illume_plan_pass_shares(n, a.ctypes.data_as(C._pi32), b.ctypes.data_as(C._pi32), cap,
                                         out.ctypes.data_as(C._pi32))
    return st, out


@pytest.mark.parametrize("seed", range(20))
def test_split_properties(native_lib, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 64))
    npix = rng.choice([128 * 128, 256 * 256, 512 * 512, 1024 * 1024, 64 * 64, 1920 * 1080], size=n)
    left = rng.integers(1, 4096, size=n)
    cap = int(max(npix.sum(), rng.integers(1 << 20, 1 << 24)))
    st, pp = plan(npix, left, cap)
    assert st == C.OK
    assert (pp >= 1).all() and (pp <= left).all()
    used = int((pp.astype(np.int64) * npix).sum())
    assert used <= cap
    spare = cap - used
    # no unfinished job could take one more sample of all its pixels
    assert not ((pp < left) & (npix <= spare)).any()


def test_equal_jobs_get_equal_shares(native_lib):
    st, pp = plan([65536] * 4, [1000] * 4, 1 << 22)
    assert st == C.OK
    assert (pp == 16).all()


def test_small_jobs_are_capped_by_their_samples(native_lib):
    st, pp = plan([16384, 1 << 20], [8, 1000], 1 << 22)
    assert st == C.OK
    assert pp[0] == 8
    assert pp[1] == ((1 << 22) - 8 * 16384) // (1 << 20)


def test_errors(native_lib):
    st, _ = plan([1 << 20, 1 << 20], [4, 4], (1 << 21) - 1)
    assert st == C.ERR_BUDGET
    st, _ = plan([0], [4], 100)
    assert st == C.ERR_INVALID
    assert C.lib().illume_plan_pass_shares(0, None, None, 10, None) == C.OK
    assert C.lib().illume_plan_pass_shares(1, None, None, 10, None) == C.ERR_INVALID
