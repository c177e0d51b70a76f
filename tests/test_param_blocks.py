"""Per-call parameter blocks of every size reach the device intact.

Stages upload their per-frame descriptors in the launch parameters of a
small kernel (16 KB per launch, blocks up to 64 KB) and fall back to one
copy-engine copy above that.  One warp call over 200 frames sends 199
descriptors of 104 bytes (two launch-parameter blocks); one over 700 frames
sends about 73 KB (the copy).  Either way every frame must come out exactly
as calls of five frames warp it (the same kernel on the same inputs:
bit-identical), and the staging buffer may be reused at once: the calls are
issued back to back without a synchronisation in between.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _similarities(rng, n, h, w):
    mats = np.tile(np.eye(3), (n, 1, 1))
    for k in range(1, n):
        a = rng.uniform(-0.01, 0.01)
        c, s = np.cos(a), np.sin(a)
        cx, cy = (w - 1) / 2.0, (h - 1) / 2.0
        tx, ty = rng.uniform(-1.5, 1.5, 2)
        mats[k] = [[c, -s, cx - c * cx + s * cy + tx], [s, c, cy - s * cx - c * cy + ty], [0.0, 0.0, 1.0]]
    return mats


@pytest.mark.parametrize("n", [200, 700])
def test_one_warp_call_over_many_frames_equals_small_calls(native, n):
    from glass_gb300 import _lib

    rng = np.random.default_rng(n)
    h, w = 24, 40
    frames = rng.normal(100.0, 5.0, (n, h, w)).astype(np.float32)
    mats = _similarities(rng, n, h, w)
    whole = native.ResidentCalibratedStack(n, h, w)
    parts = native.ResidentCalibratedStack(n, h, w)
    try:
        for k in range(n):
            whole.upload_calibrated_frame(k, frames[k])
            parts.upload_calibrated_frame(k, frames[k])
        moving = np.arange(1, n)
        whole.warp_frames_async(moving, mats[1:], _lib.GG_INTERP_LANCZOS3, np.nan, -1.0, False)
        for lo in range(1, n, 5):
            idx = np.arange(lo, min(lo + 5, n))
            parts.warp_frames_async(idx, mats[idx], _lib.GG_INTERP_LANCZOS3, np.nan, -1.0, False)
        for k in range(n):
            a, b = whole.download_frame(k), parts.download_frame(k)
            np.testing.assert_array_equal(a, b, err_msg=f"frame {k}")
        # the frames moved (sub-pixel shifts change every interior sample)
        for k in (1, n // 2, n - 1):
            inner = (slice(4, h - 4), slice(4, w - 4))
            assert np.all(np.isfinite(whole.download_frame(k)[inner]))
            assert not np.allclose(whole.download_frame(k)[inner], frames[k][inner], rtol=0.0, atol=1e-3)
    finally:
        whole.close()
        parts.close()
