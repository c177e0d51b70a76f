"""Source DQ: isolated cosmetic defects.

CPU: the oracle reproduces the reference's detect_isolated_cosmetic_defects
and detect_star_protected_cosmetic_defects HOT / COLD bits (golden vectors
from src/glass/cpu/cosmetic.py, bit-exact).
GPU: the device detector flags the same pixels (exact), sets exactly those
to NaN, counts them in the frame's non-finite counter (so integration keeps
the right formulas), and the invalid-mask entry point NaNs a given mask.
Threshold-only mask: the oracle's known answers on CPU (strict > / <,
non-finite first, infinite thresholds allowed); on the GPU the same counts
and the same NaN pixels (finite values untouched, bit-exact), single-frame,
batch and count-only forms, then an integration that sees the new NaNs.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import cosmetic as ocos

from .conftest import GOLDEN


@pytest.fixture(scope="module")
def golden_cos():
    return np.load(GOLDEN / "cosmetic.npz", allow_pickle=False)


def test_oracle_matches_reference(golden_cos):
    g = golden_cos
    for name in [str(n) for n in g["_names"]]:
        img = g[f"{name}/image"]
        for kind, res in (("isolated", ocos.isolated_defects(img)), ("protected", ocos.star_protected_defects(img))):
            np.testing.assert_array_equal(res["hot"], g[f"{name}/{kind}/hot"], err_msg=f"{name} {kind} hot")
            np.testing.assert_array_equal(res["cold"], g[f"{name}/{kind}/cold"], err_msg=f"{name} {kind} cold")


@pytest.mark.gpu
@pytest.mark.parametrize("protect", [False, True])
def test_gpu_cosmetic_matches_oracle(native, golden_cos, protect):
    g = golden_cos
    for name in [str(n) for n in g["_names"]]:
        img = g[f"{name}/image"]
        h, w = img.shape
        s = native.ResidentCalibratedStack(1, h, w)
        try:
            s.upload_calibrated_frame(0, img)
            res = s.cosmetic_mask_frames([0], star_protection=protect)[0]
            got = s.download_frame(0)
            stats = s.frame_global_stats(0)
        finally:
            s.close()
        exp = ocos.star_protected_defects(img) if protect else ocos.isolated_defects(img)
        flagged = exp["hot"] | exp["cold"]
        assert res["hot_pixels"] == int(exp["hot"].sum()) and res["cold_pixels"] == int(exp["cold"].sum()), name
        assert res["candidate_hot_pixels"] == int(exp["candidate_hot"].sum())
        assert res["candidate_cold_pixels"] == int(exp["candidate_cold"].sum())
        if protect:
            assert res["star_protected_hot_pixels"] == int(exp["star_protected_hot"].sum())
        # exactly the flagged pixels became NaN
        np.testing.assert_array_equal(np.isnan(got), np.isnan(img) | flagged, err_msg=name)
        keep = ~np.isnan(got)
        np.testing.assert_array_equal(got[keep], img[keep])
        assert stats["nonfinite_pixels"] == int((np.isnan(img) | flagged).sum())


@pytest.mark.gpu
def test_gpu_cosmetic_count_only_and_invalid_mask(native, golden_cos):
    img = golden_cos["small/image"]
    h, w = img.shape
    s = native.ResidentCalibratedStack(1, h, w)
    try:
        s.upload_calibrated_frame(0, img)
        res = s.cosmetic_mask_frames([0], apply=False)[0]
        np.testing.assert_array_equal(s.download_frame(0), img)
        assert res["hot_pixels"] > 0
        mask = np.zeros((h, w), np.uint8)
        mask[10:12, 20:25] = 1
        out = s.apply_invalid_mask_frame(0, mask)
        got = s.download_frame(0)
        assert out["invalid_samples"] == 10
        assert np.all(np.isnan(got[10:12, 20:25]))
        with pytest.raises(ValueError):
            s.apply_invalid_mask_frame(0, np.zeros((h, w + 1), np.uint8))
    finally:
        s.close()


@pytest.mark.gpu
def test_gpu_cosmetic_then_integration_uses_masked_formulas(native):
    """After the defects become NaN the integrator must switch to the
    per-pixel-count formulas (the frame counters tell it), matching the
    oracle integration of the masked frames."""
    from oracle import integration as ointeg

    rng = np.random.default_rng(12)
    n, h, w = 6, 48, 64
    frames = rng.normal(900.0, 9.0, (n, h, w)).astype(np.float32)
    for k in range(n):
        frames[k, rng.integers(1, h - 1, 6), rng.integers(1, w - 1, 6)] += np.float32(2500.0)
    s = native.ResidentCalibratedStack(n, h, w)
    try:
        for k in range(n):
            s.upload_calibrated_frame(k, frames[k])
        s.cosmetic_mask_frames(list(range(n)))
        masked = np.stack([s.download_frame(k) for k in range(n)])
        assert np.isnan(masked).any()
        got = s.integrate_hardened_winsorized_sigma(None, 3.0, 3.0, 3, 0.5, "float32")[:5]
    finally:
        s.close()
    exp = ointeg.weighted_integrate_stack(masked, None, "winsorized_sigma", 3.0, 3.0)
    for k in (2, 3, 4):  # coverage, low, high: exact
        np.testing.assert_array_equal(got[k], exp[k], err_msg=f"map {k}")
    for k in (0, 1):  # master, weight: within one float32 ulp (the integration bar)
        np.testing.assert_allclose(got[k], exp[k], rtol=1.2e-7, atol=0, err_msg=f"map {k}")


def test_oracle_threshold_mask_known_answer():
    frame = np.array([[np.nan, np.inf, -np.inf, 5.0], [100.0, -3.0, 60.0, 0.0]], dtype=np.float32)
    out, hot, cold, nonfinite = ocos.threshold_mask(frame, 0.0, 60.0)
    assert (hot, cold, nonfinite) == (1, 1, 3)  # 60 is not above 60, 0 is not below 0
    np.testing.assert_array_equal(np.isnan(out), [[True, True, True, False], [True, True, False, False]])
    np.testing.assert_array_equal(out[~np.isnan(out)], [5.0, 60.0, 0.0])
    same, *counts = ocos.threshold_mask(frame, 0.0, 60.0, apply=False)
    assert counts == [1, 1, 3]
    np.testing.assert_array_equal(same, frame)
    _, hot, cold, nonfinite = ocos.threshold_mask(frame, -np.inf, np.inf)
    assert (hot, cold, nonfinite) == (0, 0, 3)
    for lo, hi in ((np.nan, 1.0), (0.0, np.nan), (2.0, 1.0)):
        with pytest.raises(ValueError):
            ocos.threshold_mask(frame, lo, hi)


def _threshold_frames(rng, n, h, w):
    frames = rng.normal(1000.0, 30.0, (n, h, w)).astype(np.float32)
    for k in range(n):
        frames[k, rng.integers(0, h, 9), rng.integers(0, w, 9)] = np.float32(5000.0)
        frames[k, rng.integers(0, h, 7), rng.integers(0, w, 7)] = np.float32(-20.0)
        frames[k, rng.integers(0, h, 3), rng.integers(0, w, 3)] = np.nan
        frames[k, rng.integers(0, h, 2), rng.integers(0, w, 2)] = np.inf
        frames[k, 0, 0] = np.float32(1100.0)  # exactly the high threshold below: not hot
        frames[k, h - 1, w - 1] = np.float32(900.0)  # exactly the low threshold: not cold
    return frames


def _same_pixels(got, exp, tag):
    np.testing.assert_array_equal(np.isnan(got), np.isnan(exp), err_msg=tag + " NaN pixels")
    fin = ~np.isnan(exp)
    np.testing.assert_array_equal(got[fin], exp[fin], err_msg=tag + " finite values")


@pytest.mark.gpu
def test_gpu_threshold_mask_matches_oracle(native):
    from oracle import integration as ointeg

    rng = np.random.default_rng(31)
    n, h, w = 5, 37, 53  # 1,961 pixels: the float4 loop plus a one-sample tail
    frames = _threshold_frames(rng, n, h, w)
    s = native.ResidentCalibratedStack(n, h, w)
    try:
        for k in range(n):
            s.upload_calibrated_frame(k, frames[k])
        expected = frames.copy()
        one = s.apply_cosmetic_threshold_mask_frame(0, 900.0, 1100.0)
        expected[0], hot, cold, nonf = ocos.threshold_mask(frames[0], 900.0, 1100.0)
        assert (one["hot_samples"], one["cold_samples"], one["nonfinite_samples"]) == (hot, cold, nonf)
        assert one["invalid_samples"] == hot + cold + nonf and one["applied"]
        batch = s.apply_cosmetic_threshold_mask_frames([1, 3], [900.0, -np.inf], [1100.0, 2000.0])
        for pos, (k, lo, hi) in enumerate(((1, 900.0, 1100.0), (3, -np.inf, 2000.0))):
            expected[k], hot, cold, nonf = ocos.threshold_mask(frames[k], lo, hi)
            r = batch["frames"][pos]
            assert r["frame_index"] == k and r["batch_position"] == pos
            assert (r["hot_samples"], r["cold_samples"], r["nonfinite_samples"]) == (hot, cold, nonf)
        counted = s.count_cosmetic_threshold_mask_frame(2, 900.0, 1100.0)
        _, hot, cold, nonf = ocos.threshold_mask(frames[2], 900.0, 1100.0, apply=False)
        assert (counted["hot_samples"], counted["cold_samples"], counted["nonfinite_samples"]) == (hot, cold, nonf)
        assert not counted["applied"]
        many = s.count_cosmetic_threshold_mask_frames([4, 2], [900.0, 900.0], [1100.0, 1100.0])
        assert many["frame_count"] == 2 and many["frames"][1]["hot_samples"] == hot
        for k in range(n):
            _same_pixels(s.download_frame(k), expected[k], f"frame {k}")
        for lo, hi in ((np.nan, 1.0), (2.0, 1.0)):
            with pytest.raises(ValueError):
                s.apply_cosmetic_threshold_mask_frame(0, lo, hi)
        with pytest.raises(ValueError):
            s.apply_cosmetic_threshold_mask_frames([0, 1], [0.0], [1.0, 2.0])
        # the new NaNs are in the frames' non-finite counters: the integrator
        # takes the per-pixel-count formulas, as the oracle does
        got = s.integrate_hardened_winsorized_sigma(None, 3.0, 3.0, 3, 0.5, "float32")[:5]
    finally:
        s.close()
    exp = ointeg.weighted_integrate_stack(expected, None, "winsorized_sigma", 3.0, 3.0)
    for k in (2, 3, 4):
        np.testing.assert_array_equal(got[k], exp[k], err_msg=f"map {k}")
    for k in (0, 1):
        np.testing.assert_allclose(got[k], exp[k], rtol=1.2e-7, atol=0, err_msg=f"map {k}")
