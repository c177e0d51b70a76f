"""Alignment metrics and sub-pixel translation refinement: the oracle is
pinned to the reference's matrix_alignment_metrics_f32,
refine_matrix_translation_with_metrics_f32 and
estimate_translation_subpixel_ncc_f32 (golden vectors from src/glass_cuda.py),
and the GPU must agree.

GPU bar: valid/sampled counts, the chosen translation offsets and the
candidate counts exact; rms / mean |d| / ncc within 1e-6 relative (float64
statistics in the reference, float32 chunk sums folded into float-float and
float64 here; the bilinear samples themselves are bit-exact).
"""

from __future__ import annotations

import ast

import numpy as np
import pytest

from oracle import alignment as oal

from .conftest import GOLDEN

RTOL = 1e-6


@pytest.fixture(scope="module")
def golden_al():
    return np.load(GOLDEN / "alignment.npz", allow_pickle=False)


def _names(g, key):
    return [str(n) for n in g[key]]


def _close(a, b, rtol=RTOL, atol=1e-9):
    a, b = float(a), float(b)
    if np.isnan(b):
        return np.isnan(a)
    if np.isinf(b):
        return a == b
    return abs(a - b) <= atol + rtol * abs(b)


# ---- oracle pinning (CPU) -----------------------------------------------------------
def test_oracle_metrics_match_reference(golden_al):
    g = golden_al
    names = _names(g, "_metric_names")
    assert len(names) >= 20
    for name in names:
        got = oal.alignment_metrics(g[f"{name}/ref"], g[f"{name}/mov"], g[f"{name}/matrix"], int(g[f"{name}/stride"]))
        assert got["valid_pixels"] == int(g[f"{name}/valid_pixels"]), name
        assert got["sampled_pixels"] == int(g[f"{name}/sampled_pixels"]), name
        for k in ("rms", "mean_abs_diff", "ncc"):
            assert _close(got[k], g[f"{name}/{k}"], rtol=1e-12), (name, k, got[k], float(g[f"{name}/{k}"]))


def test_oracle_refine_matches_reference(golden_al):
    g = golden_al
    for name in _names(g, "_refine_names"):
        params = ast.literal_eval(str(g[f"{name}/params"]))
        got = oal.refine_translation(g[f"{name}/ref"], g[f"{name}/mov"], g[f"{name}/seed"], **params)
        assert got["dx_correction"] == float(g[f"{name}/dx_correction"]), name
        assert got["dy_correction"] == float(g[f"{name}/dy_correction"]), name
        assert got["coarse_candidates"] == int(g[f"{name}/coarse_candidates"]), name
        assert got["fine_candidates"] == int(g[f"{name}/fine_candidates"]), name
        np.testing.assert_array_equal(got["matrix"], g[f"{name}/matrix"])
        for k in ("rms", "mean_abs_diff", "ncc"):
            assert _close(got["metrics"][k], g[f"{name}/metrics_{k}"], rtol=1e-12), (name, k)


def test_oracle_translation_ncc_matches_reference(golden_al):
    g = golden_al
    for name in _names(g, "_ncc_names"):
        cdx, cdy, rad, step, stride = g[f"{name}/args"]
        got = oal.translation_ncc(g[f"{name}/ref"], g[f"{name}/mov"], cdx, cdy, int(rad), step, int(stride))
        assert got["dx"] == float(g[f"{name}/dx"]) and got["dy"] == float(g[f"{name}/dy"]), name
        assert got["candidate_count"] == int(g[f"{name}/candidate_count"])
        assert _close(got["score"], g[f"{name}/score"], rtol=1e-12), name


# ---- GPU parity -----------------------------------------------------------------------
@pytest.mark.gpu
def test_gpu_metrics_match_reference(native, golden_al):
    g = golden_al
    for name in _names(g, "_metric_names"):
        got = native.matrix_alignment_metrics_f32(g[f"{name}/ref"], g[f"{name}/mov"], g[f"{name}/matrix"],
                                                  int(g[f"{name}/stride"]))
        assert got["valid_pixels"] == int(g[f"{name}/valid_pixels"]), name
        assert got["sampled_pixels"] == int(g[f"{name}/sampled_pixels"]), name
        for k in ("rms", "mean_abs_diff", "ncc"):
            assert _close(got[k], g[f"{name}/{k}"]), (name, k, got[k], float(g[f"{name}/{k}"]))


@pytest.mark.gpu
def test_gpu_refine_matches_reference(native, golden_al):
    g = golden_al
    for name in _names(g, "_refine_names"):
        params = ast.literal_eval(str(g[f"{name}/params"]))
        got = native.refine_matrix_translation_with_metrics_f32(g[f"{name}/ref"], g[f"{name}/mov"],
                                                                g[f"{name}/seed"], **params)
        assert got["dx_correction"] == float(g[f"{name}/dx_correction"]), name
        assert got["dy_correction"] == float(g[f"{name}/dy_correction"]), name
        assert got["coarse_candidates"] == int(g[f"{name}/coarse_candidates"]), name
        assert got["fine_candidates"] == int(g[f"{name}/fine_candidates"]), name
        np.testing.assert_array_equal(np.asarray(got["matrix"], np.float32), g[f"{name}/matrix"])
        assert got["metrics"]["valid_pixels"] == int(g[f"{name}/metrics_valid_pixels"]), name
        assert got["metrics"]["sample_stride"] == int(g[f"{name}/metrics_sample_stride"]), name
        for k in ("rms", "mean_abs_diff", "ncc"):
            assert _close(got["metrics"][k], g[f"{name}/metrics_{k}"]), (name, k)


@pytest.mark.gpu
def test_gpu_translation_ncc_matches_reference(native, golden_al):
    g = golden_al
    for name in _names(g, "_ncc_names"):
        cdx, cdy, rad, step, stride = g[f"{name}/args"]
        got = native.estimate_translation_subpixel_ncc_f32(g[f"{name}/ref"], g[f"{name}/mov"], cdx, cdy, int(rad),
                                                           step, int(stride))
        assert got["dx"] == float(g[f"{name}/dx"]) and got["dy"] == float(g[f"{name}/dy"]), name
        assert got["candidate_count"] == int(g[f"{name}/candidate_count"])
        assert _close(got["score"], g[f"{name}/score"]), name


@pytest.mark.gpu
def test_gpu_resident_batch_refine_large_frames(native):
    """Batch refinement of several resident frames at bench-like strides,
    against the oracle on the same frames."""
    rng = np.random.default_rng(4)
    h, w = 160, 200
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    pts = np.column_stack([rng.uniform(4, w - 5, 60), rng.uniform(4, h - 5, 60)])
    flux = rng.uniform(300, 4000, 60)

    def render(shift):
        img = np.full((h, w), 500.0)
        for (x0, y0), f in zip(pts - np.asarray(shift), flux):
            img += f * np.exp(-((xx - x0) ** 2 + (yy - y0) ** 2) / (2 * 1.4 ** 2))
        return (img + 4.0 * rng.standard_normal((h, w))).astype(np.float32)

    shifts = [(0.0, 0.0), (0.31, -0.44), (-0.72, 0.18)]
    frames = [render(sh) for sh in shifts]
    s = native.ResidentCalibratedStack(3, h, w)
    try:
        for k, f in enumerate(frames):
            s.upload_calibrated_frame(k, f)
        seeds = [np.array([[1.0, 0, sx + 0.1], [0, 1.0, sy - 0.1], [0, 0, 1.0]]) for sx, sy in shifts[1:]]
        got = s.refine_matrix_translation_candidates_batch_to_reference(0, [1, 2], seeds, 1.0, 0.25, 0.25, 0.0625, 4,
                                                                        2)
    finally:
        s.close()
    for k in (1, 2):
        exp = oal.refine_translation(frames[0], frames[k], seeds[k - 1], 1.0, 0.25, 0.25, 0.0625, 4, 2)
        assert got[k - 1]["dx_correction"] == exp["dx_correction"]
        assert got[k - 1]["dy_correction"] == exp["dy_correction"]
        for key in ("rms", "ncc"):
            assert _close(got[k - 1]["metrics"][key], exp["metrics"][key]), key
