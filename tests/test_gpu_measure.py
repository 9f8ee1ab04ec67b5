"""Measurement hooks on the GPU: the L2 read-bandwidth probe the bench reports beside the
trace kernel's roofline."""
import ctypes

import pytest

from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def test_l2_read_probe(ctx):
    gbs = ctypes.c_double(0.0)
    assert C.lib().illume_measure_l2_read(ctx.handle, 32 << 20, 20, ctypes.byref(gbs)) == C.OK
    # an L2-resident sweep outruns the HBM copy rate of the part (several TB/s)
    assert gbs.value > 3000.0
    assert C.lib().illume_measure_l2_read(ctx.handle, 8, 1, ctypes.byref(gbs)) == C.ERR_INVALID
