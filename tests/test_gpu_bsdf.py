"""BSDF sample / eval / pdf on the GPU (the device code the shade kernel runs) against
the oracle: FP32 GPU vs FP32 oracle (same arithmetic), and FP32 GPU vs the FP64 oracle
within 1e-5 relative on well-conditioned inputs.

Decisions: |wi.n| >= 0.05, every Fresnel/probability decision more than 1e-4 from its
threshold, and the kill test (wi.n)(wo.n) more than 1e-4 from zero: statuses must equal
FP64's and directions be within 1e-5. Values (weight, D, pdf, G, F, eval): within 1e-5
relative (to max(|ref|, 1e-3)) on >= 99.5% of the tuples whose FP64 values move by less
than 4e-6 under a 4-ulp perturbation of the inputs, and within 5e-5 on all of them.
"""
import json

import numpy as np
import pytest

from illume_gb300 import _capi as C

pytestmark = pytest.mark.gpu

CASES = [(C.MAT_LAMBERT, C.DIST_BECKMANN), (C.MAT_REFLECTIVE, C.DIST_BECKMANN), (C.MAT_REFRACTIVE, C.DIST_BECKMANN),
         (C.MAT_ROUGHREFLECTIVE, C.DIST_BECKMANN), (C.MAT_ROUGHREFLECTIVE, C.DIST_GGX),
         (C.MAT_ROUGHREFRACTIVE, C.DIST_BECKMANN), (C.MAT_ROUGHREFRACTIVE, C.DIST_GGX),
         (C.MAT_CONDUCTOR, C.DIST_BECKMANN), (C.MAT_ROUGHCONDUCTOR, C.DIST_BECKMANN),
         (C.MAT_ROUGHCONDUCTOR, C.DIST_GGX), (C.MAT_PLASTIC, C.DIST_BECKMANN)]


def tuples(n, seed, mat):
    rng = np.random.default_rng(seed)
    N = rng.normal(size=(n, 3))
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    w = rng.normal(size=(n, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    # most wi on the normal's side; refractive materials also from inside
    flip_share = 0.3 if mat in (C.MAT_REFRACTIVE, C.MAT_ROUGHREFRACTIVE) else 0.05
    side = np.where(rng.random(n) < flip_share, -1.0, 1.0)
    w = np.where(((w * N).sum(1) * side < 0)[:, None], -w, w)
    x = np.zeros((n, 16), np.float32)
    x[:, 0:3] = w
    x[:, 3:6] = N
    x[:, 6:9] = (np.floor(rng.random((n, 3)) * 16777216) + 1) / 16777216
    x[:, 9] = rng.uniform(0.05, 0.6, n)
    x[:, 10] = rng.uniform(1.2, 2.0, n) if mat != C.MAT_PLASTIC else 1.5
    x[:, 11:14] = (0.143, 0.374, 1.442)
    x[:, 14] = 3.983
    return x


def conditioned(x, ref):
    wi, N = x[:, 0:3].astype(np.float64), x[:, 3:6].astype(np.float64)
    wdn = (wi * N).sum(1)
    wo = ref[:, 0:3].astype(np.float64)
    ok = np.abs(wdn) >= 0.05
    ok &= np.abs(wdn * (wo * N).sum(1)) > 1e-4
    F = ref[:, 9].astype(np.float64)
    for k in (6, 8):
        ok &= np.abs(x[:, k] - F) > 1e-4
    ok &= (F < 1.0 - 1e-6)
    return ok


@pytest.mark.parametrize("mat,dist", CASES)
def test_bsdf_against_oracle(ctx, mat, dist):
    from illume_gb300.api import bsdf_batch
    from oracle import pyoracle
    x = tuples(8192, seed=mat * 10 + dist, mat=mat)
    got = bsdf_batch(ctx, mat, dist, x)
    f32 = pyoracle.bsdf_batch(mat, dist, x, precision=32)
    f64 = pyoracle.bsdf_batch(mat, dist, x, precision=64)
    # same FP32 formulation as the reference: sampling decisions identical
    assert (got[:, 12] == f32[:, 12]).mean() >= 0.999
    # FP64 oracle, well-conditioned tuples: identical decisions, directions within 1e-5
    ok = conditioned(x, f64)
    assert ok.mean() > 0.5
    assert np.array_equal(got[ok, 12], f64[ok, 12])
    live = ok & (f64[:, 12] > 0)
    d = np.abs(got[live, 0:3] - f64[live, 0:3])
    assert d.max() < 1e-5, d.max()
    # values (weight, D, pdf_m, G, F, eval, pdf) within 1e-5 relative of FP64 wherever the
    # values are stable under a 4-ulp perturbation of the inputs (an FP32 evaluation
    # cannot be more accurate than its inputs allow: near m = n the reference's
    # (cos^2 - 1) / cos^2 amplifies an ulp of m by orders of magnitude)
    vals = [3, 4, 5, 6, 7, 8, 9, 10, 11]
    xp = x.copy()
    xp[:, 0:6] *= np.float32(1.0 - 4.0 * 2.0 ** -24)
    xp[:, 6:9] *= np.float32(1.0 - 4.0 * 2.0 ** -24)
    f64p = pyoracle.bsdf_batch(mat, dist, xp, precision=64)
    ref = np.maximum(np.abs(f64[:, vals]), 1e-3)
    sens = (np.abs(f64p[:, vals] - f64[:, vals]) / ref).max(1)
    stable = live & (sens < 4e-6) & (f64p[:, 12] == f64[:, 12])
    assert stable.sum() >= 0.3 * live.sum(), (stable.sum(), live.sum())
    rel_gpu = (np.abs(got[stable][:, vals] - f64[stable][:, vals]) / ref[stable]).max(1)
    # the FP32 formulation itself (FP32 oracle) leaves a small tail above 1e-5 on these
    assert (rel_gpu < 1e-5).mean() >= 0.995, (rel_gpu < 1e-5).mean()
    assert rel_gpu.max() < 5e-5, rel_gpu.max()
    # reported over every live tuple, conditioned or not (printed; pytest -s shows it):
    # the share within 1e-5 of FP64, the worst case, and the same for the FP32 oracle,
    # whose arithmetic the kernels follow
    alive = (f64[:, 12] > 0) & (got[:, 12] == f64[:, 12])
    rel_all = (np.abs(got[alive][:, vals] - f64[alive][:, vals]) / ref[alive]).max(1)
    rel_f32 = (np.abs(f32[alive][:, vals] - f64[alive][:, vals]) / ref[alive]).max(1)
    print("BSDF_STATS", json.dumps({"material": int(mat), "distribution": int(dist), "live": int(alive.sum()),
                                    "stable": int(stable.sum()),
                                    "gpu_within_1e-5_all_live": round(float((rel_all < 1e-5).mean()), 4),
                                    "gpu_max_rel_all_live": float(rel_all.max()) if alive.any() else 0.0,
                                    "fp32_oracle_within_1e-5_all_live": round(float((rel_f32 < 1e-5).mean()), 4),
                                    "fp32_oracle_max_rel_all_live": float(rel_f32.max()) if alive.any() else 0.0}))
