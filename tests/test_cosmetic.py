"""Source DQ: isolated cosmetic defects.

CPU: the oracle reproduces the reference's detect_isolated_cosmetic_defects
and detect_star_protected_cosmetic_defects HOT / COLD bits (golden vectors
from src/glass/cpu/cosmetic.py, bit-exact).
GPU: the device detector flags the same pixels (exact), sets exactly those
to NaN, counts them in the frame's non-finite counter (so integration keeps
the right formulas), and the invalid-mask entry point NaNs a given mask.
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
