"""Fused warp + integration (integrate_matrix_warped_{mean,sigma_clip}).

The reference defines the fused path as the integration of the warped stack
without writing it (glass_cuda.py:5142-5287; integration_kernels.cu:3840-4123;
it has no CPU fallback).  So the bar is:
  - bit-exact equality with this library's own two-step path (warp the frames
    in place with NaN fill, then integrate), maps, counts and DQ included;
  - the geometric coverage equals the warp coverage accumulator;
  - against the oracle (oracle.warp + oracle.integration on the warped stack):
    masks and counts exact, maps within 1e-6 relative for bilinear.
The resident frames are left untouched.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import integration as ointeg
from oracle import warp as owarp

pytestmark = pytest.mark.gpu


def _stack(rng, n, h, w, nan_frac=0.0):
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    base = np.full((h, w), 800.0)
    for _ in range(12):
        x0, y0 = rng.uniform(3, w - 4), rng.uniform(3, h - 4)
        base += rng.uniform(300, 5000) * np.exp(-((xx - x0) ** 2 + (yy - y0) ** 2) / (2 * 1.5 ** 2))
    frames = np.stack([base + 15.0 * rng.standard_normal((h, w)) for _ in range(n)]).astype(np.float32)
    hits = rng.random(frames.shape) < 0.01
    frames[hits] += np.float32(20000.0)
    if nan_frac:
        frames[rng.random(frames.shape) < nan_frac] = np.nan
    return frames


def _matrices(rng, n):
    mats = []
    for k in range(n):
        t = np.deg2rad(rng.uniform(-0.8, 0.8)) if k else 0.0
        dx, dy = (rng.uniform(-3, 3), rng.uniform(-3, 3)) if k else (0.0, 0.0)
        mats.append([[np.cos(t), -np.sin(t), dx], [np.sin(t), np.cos(t), dy], [0.0, 0.0, 1.0]])
    return np.asarray(mats, dtype=np.float32).astype(np.float64)


CASES = [("bilinear", False, -1.0), ("bilinear", True, -1.0), ("lanczos3", False, -1.0), ("lanczos3", True, 0.0)]


@pytest.mark.parametrize("interp,winsorize,clamp", CASES)
@pytest.mark.parametrize("n", [5, 13, 32, 40, 70])
def test_fused_equals_two_step(native, interp, winsorize, clamp, n):
    """n > 32 runs the warp-per-pixel integrator on a sampled tile."""
    rng = np.random.default_rng(100 + n)
    h, w = 37, 45
    frames = _stack(rng, n, h, w, nan_frac=0.01 if winsorize else 0.0)
    mats = _matrices(rng, n)
    weights = rng.uniform(0.5, 2.0, n).astype(np.float32)
    s = native.ResidentCalibratedStack(n, h, w)
    try:
        for k in range(n):
            s.upload_calibrated_frame(k, frames[k])
        fused = s.integrate_matrix_warped_sigma_clip(mats, weights, interp, clamp, 3.0, 3.0, winsorize)
        mean = s.integrate_matrix_warped_mean(mats, weights, interp, clamp)
        # the resident frames are unchanged
        for k in range(n):
            np.testing.assert_array_equal(s.download_frame(k), frames[k])
        # two-step: warp in place (NaN fill, coverage), then integrate
        s.reset_warp_coverage()
        idx = np.arange(n)
        s.warp_frames_async(idx, mats, 1 if interp == "bilinear" else 3, np.nan, clamp, True)
        geo = s.warp_coverage_map()
        two = s.integrate_sigma_clip(weights, 3.0, 3.0, winsorize)
        two_mean = s.integrate_mean(weights)
    finally:
        s.close()
    for a, b, name in zip(fused[:5], two, ("master", "weight", "coverage", "low", "high")):
        np.testing.assert_array_equal(a, b, err_msg=f"{interp} {name}")
    np.testing.assert_array_equal(fused[5], geo)
    np.testing.assert_array_equal(mean[0], two_mean[0])
    np.testing.assert_array_equal(mean[1], two_mean[1])
    np.testing.assert_array_equal(mean[3], geo)


def test_fused_bilinear_matches_oracle(native):
    rng = np.random.default_rng(7)
    n, h, w = 9, 33, 41
    frames = _stack(rng, n, h, w, nan_frac=0.005)
    mats = _matrices(rng, n)
    s = native.ResidentCalibratedStack(n, h, w)
    try:
        for k in range(n):
            s.upload_calibrated_frame(k, frames[k])
        got = s.integrate_matrix_warped_sigma_clip(mats, None, "bilinear", -1.0, 3.0, 3.0, True)
    finally:
        s.close()
    warped, covs = zip(*(owarp.warp_matrix(frames[k], mats[k], "bilinear", np.nan) for k in range(n)))
    exp = ointeg.weighted_integrate_stack(np.stack(warped), None, "winsorized_sigma")
    for k, name in ((2, "coverage"), (3, "low"), (4, "high")):
        np.testing.assert_array_equal(got[k], exp[k], err_msg=name)
    np.testing.assert_allclose(got[0], exp[0], rtol=1e-6, atol=1e-3)
    np.testing.assert_allclose(got[1], exp[1], rtol=1e-6)
    np.testing.assert_array_equal(got[5], np.sum(covs, axis=0))


def test_fused_argument_errors(native):
    s = native.ResidentCalibratedStack(2, 8, 8)
    try:
        for k in range(2):
            s.upload_calibrated_frame(k, np.ones((8, 8), np.float32))
        with pytest.raises(ValueError):
            s.integrate_matrix_warped_mean(np.eye(3)[None].repeat(3, 0))
        with pytest.raises(ValueError):
            s.integrate_matrix_warped_mean(np.eye(3)[None].repeat(2, 0), interpolation="nearest")
        sing = np.zeros((2, 3, 3))
        with pytest.raises(ValueError):
            s.integrate_matrix_warped_mean(sing)
    finally:
        s.close()
