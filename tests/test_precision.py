"""Precision of each output of the device step against the float64 oracle.

The device path keeps the bulk in float32 (samples, weights, thresholds) with
compensated (float-float) accumulation of means, variances and weight sums,
and uses float64 on the GPU only in the registration solves.  This file
states each output's error against oracle/fp64.py (the same definitions with
every operation in float64) on a synthetic stack: 12 frames 256 x 256,
Gaussian stars, sky 1000 ADU, read noise 5 ADU, hot pixels and cosmic rays,
shifts up to 6 px and rotations up to 0.3 deg, calibrated from uint16 with
bias / dark / flat masters, Lanczos3-warped through the known matrices,
simple-SNR weights, winsorized 3 / 3 sigma integration.

Bounds (asserted; the measured values are printed as one PRECISION line):
  calibrated frames   |err| <= 4 ulp of the value (3 float32 operations)
  warped frames       RMS <= 2e-7, max <= 2e-6 of the frame's robust range
  weights             relative <= 1e-6
  master              over pixels with the same kept set: RMS <= 1e-3 and
                      max <= 2e-2 noise units (winsorized scale / sqrt(kept));
                      relative max <= 2e-6
  weight map          relative <= 1e-6 where the kept sets agree
  coverage / low / high counts, DQ
                      identical on >= 99.99 % of the pixels (a sample within
                      float32 rounding of a threshold may flip)
"""

from __future__ import annotations

import json

import numpy as np
import pytest

from oracle import fp64
from oracle import integration as ointeg


def _stack():
    from glass_gb300.synthetic import StackConfig, generate

    cfg = StackConfig(frames=12, height=256, width=256, stars=160, fwhm=(2.5, 3.5), hot_pixel_fraction=1e-4,
                      cosmic_ray_density=1e-4, max_shift=6.0, max_rotation_deg=0.3, calibration_frames=4, seed=7)
    return generate(cfg)


def _masters(data):
    b = data.bias_frames.astype(np.float64).mean(0)
    d = data.dark_frames.astype(np.float64).mean(0) - b
    f = data.flat_frames.astype(np.float64).mean(0) - b
    f = np.maximum(f / np.median(f), 1e-6)
    return b.astype(np.float32), d.astype(np.float32), f.astype(np.float32)


def test_fp64_oracle_agrees_with_reference_semantics():
    """The float64 restatement and the float32-rounding oracle describe the
    same integration: masters within float32 rounding, counts equal except
    at thresholds."""
    rng = np.random.default_rng(3)
    stack = rng.normal(1000.0, 10.0, (9, 40, 48)).astype(np.float32)
    stack[2, 5, 5] = 5000.0
    stack[4, :3, :4] = np.nan
    w = rng.uniform(0.5, 2.0, 9).astype(np.float32)
    m32, w32, c32, l32, h32 = ointeg.weighted_integrate_stack(stack, w, "winsorized_sigma", 3.0, 3.0)
    m64, w64, c64, l64, h64, _ = fp64.winsorized_integrate_f64(stack, w, 3.0, 3.0)
    same = (c32 == c64) & (l32 == l64) & (h32 == h64)
    assert same.mean() >= 0.999
    np.testing.assert_allclose(m32[same], m64[same], rtol=2e-6)
    np.testing.assert_allclose(w32[same], w64[same], rtol=1e-6)
    assert h64[5, 5] >= 1


def _ulp(v):
    return np.spacing(np.abs(v).astype(np.float32)).astype(np.float64)


@pytest.mark.gpu
def test_gpu_step_error_against_fp64(native):
    from glass_gb300.pipeline import Masters, ResidentPipeline, StepConfig

    data = _stack()
    n, h, w = data.lights.shape
    bias, dark, flat = _masters(data)
    pipe = ResidentPipeline(n, h, w, Masters(bias, dark, flat), StepConfig())
    try:
        pipe.calibrate_host(np.ascontiguousarray(data.lights))
        pipe.stack.synchronize()
        cal = np.stack([pipe.stack.download_frame(k) for k in range(n)])
        pipe.warp(data.truth_matrices)
        pipe.stack.synchronize()
        warped = np.stack([pipe.stack.download_frame(k) for k in range(n)])
        weights = pipe.stack.compute_frame_weights("simple_snr", None, 1.0e-6, download=True)
        pipe.integrate()
        master, wmap, cov, low, high, dq = pipe.stack.download_maps("full", include_dq=True)
    finally:
        pipe.close()

    cal64 = np.stack([fp64.calibrate_f64(data.lights[k], bias, dark, flat, 1.0) for k in range(n)])
    warp64 = cal64.copy()
    warp64[1:] = fp64.warp_frames_f64(cal64[1:], data.truth_matrices[1:])
    w64 = fp64.simple_snr_weights_f64(warp64)
    m64, wm64, c64, l64, h64, s64 = fp64.winsorized_integrate_f64(warp64, w64, 3.0, 3.0, 3, 0.5)

    report = {}
    cal_err = np.abs(cal.astype(np.float64) - cal64) / _ulp(cal64)
    report["calibrated_max_ulp"] = float(cal_err.max())
    fin = np.isfinite(warp64) & np.isfinite(warped)
    assert np.array_equal(np.isfinite(warp64), np.isfinite(warped))
    rng_ = np.percentile(warp64[fin], 99.9) - np.percentile(warp64[fin], 0.1)
    werr = np.abs(warped.astype(np.float64)[fin] - warp64[fin]) / rng_
    report["warped_rms_of_range"] = float(np.sqrt(np.mean(werr ** 2)))
    report["warped_max_of_range"] = float(werr.max())
    report["weights_max_rel"] = float(np.max(np.abs(weights - w64) / w64))
    same = (cov == c64) & (low == l64) & (high == h64)
    report["counts_identical_fraction"] = float(same.mean())
    noise = s64 / np.sqrt(np.maximum(c64, 1))
    ok = same & (c64 > 0) & (noise > 0)
    merr = np.abs(master.astype(np.float64) - m64)[ok]
    report["master_rms_noise_units"] = float(np.sqrt(np.mean((merr / noise[ok]) ** 2)))
    report["master_max_noise_units"] = float(np.max(merr / noise[ok]))
    report["master_max_rel"] = float(np.max(merr / np.maximum(np.abs(m64[ok]), 1e-30)))
    report["weight_map_max_rel"] = float(np.max(np.abs(wmap.astype(np.float64) - wm64)[ok] / wm64[ok]))
    dq64 = ointeg.dq_map(m64.astype(np.float32), wm64.astype(np.float32), c64.astype(np.float32),
                         l64.astype(np.float32), h64.astype(np.float32), None, n)
    report["dq_identical_fraction"] = float(np.mean(dq64 == dq))
    print("PRECISION " + json.dumps(report, sort_keys=True))

    assert report["calibrated_max_ulp"] <= 4.0
    assert report["warped_rms_of_range"] <= 2e-7 and report["warped_max_of_range"] <= 2e-6
    assert report["weights_max_rel"] <= 1e-6
    assert report["counts_identical_fraction"] >= 0.9999
    assert report["master_rms_noise_units"] <= 1e-3 and report["master_max_noise_units"] <= 2e-2
    assert report["master_max_rel"] <= 2e-6
    assert report["weight_map_max_rel"] <= 1e-6
    assert report["dq_identical_fraction"] >= 0.9999
