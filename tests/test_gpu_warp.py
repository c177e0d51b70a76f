"""GPU parity of the TMA-staged warps against the oracle / reference warp oracles.

Tolerances: coverage bit-exact; bilinear and nearest within one float32 ulp
(the kernel replays the float32 arithmetic of the reference; the float64
source coordinate is evaluated in float-float); Lanczos3 within
3e-6 x max|image| + 1e-5 x |value| (float32 weights vs the reference's float64
weights; the reference's own CUDA test allows 3e-5 on O(10) data,
tests/test_gpu_warp_vs_cpu.py:176-234).
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import warp as owarp

from .conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden_warp():
    return np.load(GOLDEN / "warp.npz", allow_pickle=False)


def lanczos_tol(image):
    fin = np.abs(image[np.isfinite(image)])
    return 3e-6 * (float(fin.max()) if fin.size else 1.0) + 1e-6


def check_warp(out, cov, exp_out, exp_cov, image, interp, tag):
    np.testing.assert_array_equal(cov, exp_cov, err_msg=tag + " coverage")
    ok = exp_cov > 0
    if interp == "lanczos3":
        # rtol covers pixels where dropping non-finite taps leaves nearly
        # cancelling weights, which amplifies the float32 weight rounding.
        np.testing.assert_allclose(out[ok], exp_out[ok], rtol=1e-5, atol=lanczos_tol(image), err_msg=tag)
    else:
        a, b = out[ok].astype(np.float64), exp_out[ok].astype(np.float64)
        tol = np.spacing(np.maximum(np.abs(a), np.abs(b)).astype(np.float32)).astype(np.float64)
        assert np.all((np.abs(a - b) <= tol) | (np.isnan(a) & np.isnan(b))), tag
    # uncovered pixels hold the fill value
    np.testing.assert_array_equal(np.isnan(out[~ok]), np.isnan(exp_out[~ok]), err_msg=tag + " fill")


def test_module_warps_match_reference_golden(native, golden_warp):
    g = golden_warp
    for name in [str(n) for n in g["_names"]]:
        code, fill, clamp = g[f"{name}/params"]
        image, matrix = g[f"{name}/image"], g[f"{name}/matrix"]
        if code == 1.0:
            out, cov = native.warp_matrix_bilinear_f32(image, matrix, fill)
            check_warp(out, cov, g[f"{name}/out"], g[f"{name}/coverage"], image, "bilinear", name)
        else:
            out, cov = native.warp_matrix_lanczos3_f32(image, matrix, fill, clamp)
            check_warp(out, cov, g[f"{name}/out"], g[f"{name}/coverage"], image, "lanczos3", name)


def test_translations_match_reference_golden(native, golden_warp):
    g = golden_warp
    img = g["translation_image"]
    for k in range(4):
        dx, dy = g[f"translation{k}/shift"]
        out, cov = native.warp_translation_f32(img, dx, dy, -1.0)
        np.testing.assert_array_equal(out, g[f"translation{k}/out"])
        np.testing.assert_array_equal(cov, g[f"translation{k}/coverage"])
        bout, bcov = native.warp_translation_bilinear_f32(img, dx, dy, -1.0)
        np.testing.assert_array_equal(bcov, g[f"translation{k}/bilinear_coverage"])
        np.testing.assert_array_equal(bout, g[f"translation{k}/bilinear_out"])


def _random_similarity(rng, max_deg, max_shift):
    t = np.deg2rad(rng.uniform(-max_deg, max_deg))
    s = rng.uniform(0.995, 1.005)
    return np.array([[s * np.cos(t), -s * np.sin(t), rng.uniform(-max_shift, max_shift)],
                     [s * np.sin(t), s * np.cos(t), rng.uniform(-max_shift, max_shift)], [0, 0, 1]], np.float32)


@pytest.mark.parametrize("shape", [(96, 128), (77, 131), (130, 64)])
def test_resident_batch_warp_and_slot_rotation(native, shape):
    """Several frames per launch, TMA path (W % 4 == 0) and the global-load
    path (W % 4 != 0); two successive warps exercise the slot swap."""
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    n = 6
    h, w = shape
    frames = (1000 + 30 * rng.standard_normal((n, h, w))).astype(np.float32)
    frames[:, 10:12, 20:23] += 15000.0
    s = native.ResidentCalibratedStack(n, h, w)
    for i in range(n):
        s.upload_calibrated_frame(i, frames[i])
    assert s.tma_enabled == (w % 4 == 0)
    m1 = np.stack([_random_similarity(rng, 1.0, 6.0) for _ in range(n - 1)])
    idx = np.arange(1, n)
    s.apply_matrix_lanczos3_frames(idx, m1, np.nan, -1.0, "chunked", 0, False)
    expected = frames.copy()
    for k, f in enumerate(idx):
        expected[f], _ = owarp.warp_matrix(frames[f], m1[k], "lanczos3", np.nan, -1.0)
    got = s.download_frames_tile(np.arange(n), 0, 0, w, h)
    for f in range(n):
        fin = np.isfinite(expected[f])
        np.testing.assert_array_equal(np.isfinite(got[f]), fin, err_msg=f"frame {f}")
        np.testing.assert_allclose(got[f][fin], expected[f][fin], rtol=0, atol=lanczos_tol(frames[f]))
    # second pass on the warped frames (slots rotated once already)
    m2 = np.stack([_random_similarity(rng, 0.5, 3.0) for _ in range(3)])
    idx2 = np.array([4, 1, 2])
    s.apply_matrix_bilinear_frames(idx2, m2, np.nan, False)
    got2 = s.download_frames_tile(np.arange(n), 0, 0, w, h)
    for k, f in enumerate(idx2):
        exp, _ = owarp.warp_matrix(got[f], m2[k], "bilinear", np.nan)
        fin = np.isfinite(exp)
        np.testing.assert_array_equal(np.isfinite(got2[f]), fin)
        np.testing.assert_array_equal(got2[f][fin], exp[fin])
    for f in (0, 3, 5):
        np.testing.assert_array_equal(got2[f], got[f])


def test_resident_warp_then_integrate_mean_reference_cases(native):
    """tests/test_gpu_warp_vs_cpu.py:196-234 of the reference, restated."""
    data = np.arange(36, dtype=np.float32).reshape(6, 6)
    matrix = np.array([[1.0, 0.0, 1.25], [0.0, 1.0, -0.5], [0.0, 0.0, 1.0]], dtype=np.float32)
    s = native.ResidentCalibratedStack(1, 6, 6)
    s.upload_calibrated_frame(0, data)
    s.apply_matrix_bilinear_frame(0, matrix, np.nan)
    warped, weight = s.integrate_mean()
    exp, exp_cov = owarp.warp_matrix(data, matrix, "bilinear", np.nan)
    valid = exp_cov > 0
    assert np.allclose(warped[valid], exp[valid], atol=1e-5)
    assert np.all(warped[~valid] == 0.0)
    assert np.array_equal(weight, exp_cov)

    yy, xx = np.indices((12, 13), dtype=np.float32)
    data = (np.sin(xx * 0.3) + np.cos(yy * 0.2)).astype(np.float32)
    matrix = np.array([[1.0, 0.0, 0.4], [0.0, 1.0, -0.35], [0.0, 0.0, 1.0]], dtype=np.float32)
    s = native.ResidentCalibratedStack(1, 12, 13)
    s.upload_calibrated_frame(0, data)
    s.apply_matrix_lanczos3_frame(0, matrix, np.nan, 0.30)
    warped, weight = s.integrate_mean()
    exp, exp_cov = owarp.warp_matrix(data, matrix, "lanczos3", np.nan, 0.30)
    valid = exp_cov > 0
    assert np.allclose(warped[valid], exp[valid], atol=3e-5)
    assert np.all(warped[~valid] == 0.0)
    assert np.array_equal(weight, exp_cov)


def test_warp_coverage_accumulator(native):
    rng = np.random.default_rng(4)
    n, h, w = 4, 40, 48
    s = native.ResidentCalibratedStack(n, h, w)
    for i in range(n):
        s.upload_calibrated_frame(i, rng.standard_normal((h, w)).astype(np.float32))
    s.reset_warp_coverage()
    s.accumulate_full_warp_coverage_frame()
    mats = np.stack([_random_similarity(rng, 2.0, 5.0) for _ in range(n - 1)])
    s.apply_matrix_lanczos3_frames(np.arange(1, n), mats, np.nan, -1.0, True)
    cov = s.warp_coverage_map()
    expected = np.ones((h, w), np.float32)
    for k in range(n - 1):
        expected += owarp.warp_matrix(np.zeros((h, w), np.float32), mats[k], "lanczos3")[1]
    np.testing.assert_array_equal(cov, expected)
    assert s.warp_coverage_frame_count == n


def test_warp_errors(native):
    s = native.ResidentCalibratedStack(2, 8, 8)
    s.upload_calibrated_frame(0, np.zeros((8, 8), np.float32))
    with pytest.raises(RuntimeError, match="loaded"):
        s.apply_matrix_bilinear_frame(1, np.eye(3), np.nan)
    with pytest.raises(ValueError, match="singular"):
        s.apply_matrix_bilinear_frame(0, np.zeros((3, 3)), np.nan)
    with pytest.raises(IndexError):
        s.apply_matrix_bilinear_frame(5, np.eye(3), np.nan)
    with pytest.raises(ValueError):
        s.apply_matrix_lanczos3_frames([0, 0], np.stack([np.eye(3)] * 2), np.nan, -1.0, False)
