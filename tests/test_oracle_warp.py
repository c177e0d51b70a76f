"""Pins the warp oracle against the reference's warp functions (golden vectors
from tests/test_gpu_warp_vs_cpu.py's CPU oracles, the glass_cuda NumPy
fallbacks and engine/warp.py's tile warp)."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import warp as owarp

from .conftest import GOLDEN


@pytest.fixture(scope="module")
def golden_warp():
    return np.load(GOLDEN / "warp.npz", allow_pickle=False)


def _interp(code: float) -> str:
    return "bilinear" if code == 1.0 else "lanczos3"


def test_oracle_matches_reference_warp_oracles(golden_warp):
    g = golden_warp
    names = [str(n) for n in g["_names"]]
    assert len(names) >= 30
    for name in names:
        code, fill, clamp = g[f"{name}/params"]
        out, cov = owarp.warp_matrix(g[f"{name}/image"], g[f"{name}/matrix"], _interp(code), fill, clamp)
        np.testing.assert_array_equal(cov, g[f"{name}/coverage"], err_msg=name)
        ok = cov > 0
        # float64 evaluation order differs only in the last bits of the weights
        np.testing.assert_allclose(out[ok], g[f"{name}/out"][ok], rtol=1e-6, atol=1e-6, err_msg=name)
        np.testing.assert_array_equal(np.isnan(out[~ok]), np.isnan(g[f"{name}/out"][~ok]))
        if f"{name}/engine_out" in g.files and clamp < 0.0:  # engine/warp.py has no overshoot clamp
            np.testing.assert_array_equal(cov, g[f"{name}/engine_coverage"], err_msg=name)
            np.testing.assert_allclose(out[ok], g[f"{name}/engine_out"][ok], rtol=1e-6, atol=1e-6, err_msg=name)
        if f"{name}/fallback_out" in g.files:
            np.testing.assert_array_equal(cov, g[f"{name}/fallback_coverage"], err_msg=name)
            np.testing.assert_allclose(out[ok], g[f"{name}/fallback_out"][ok], rtol=1e-6, atol=1e-6, err_msg=name)


def test_oracle_bilinear_is_bit_exact_for_reference_cases(golden_warp):
    g = golden_warp
    for name in [str(n) for n in g["_names"]]:
        code, fill, clamp = g[f"{name}/params"]
        if code != 1.0:
            continue
        out, cov = owarp.warp_matrix(g[f"{name}/image"], g[f"{name}/matrix"], "bilinear", fill, clamp)
        ok = cov > 0
        np.testing.assert_array_equal(out[ok], g[f"{name}/out"][ok], err_msg=name)


def test_oracle_translations(golden_warp):
    g = golden_warp
    img = g["translation_image"]
    for k in range(4):
        dx, dy = g[f"translation{k}/shift"]
        out, cov = owarp.warp_translation(img, dx, dy, -1.0)
        np.testing.assert_array_equal(out, g[f"translation{k}/out"])
        np.testing.assert_array_equal(cov, g[f"translation{k}/coverage"])
        m = np.array([[1, 0, dx], [0, 1, dy], [0, 0, 1]], np.float64)
        bout, bcov = owarp.warp_matrix(img, m, "bilinear", -1.0)
        np.testing.assert_array_equal(bcov, g[f"translation{k}/bilinear_coverage"])
        np.testing.assert_array_equal(bout, g[f"translation{k}/bilinear_out"])
