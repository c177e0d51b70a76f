"""The allocation-free frame-statistics entry point.

gg_frames_stats_f32_noalloc serves callers that cannot call cudaMalloc (code
running under stream capture, plugins whose host owns all allocations,
real-time loops): it reduces into a fixed __device__ scratch array instead of
allocating.  Here it is called through the C ABI on frames that live in a
resident stack's device memory and must agree with the existing entry point
(gg_stack_frame_stats) on two calls in a row - the second call reuses the
scratch the first one left behind.  This file is collected last so that a
failure here cannot hide the other tests' results.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from glass_gb300 import _lib

pytestmark = pytest.mark.gpu


def _noalloc_stats(dev_frames: int, count: int, pixels: int, stride: int):
    out = (_lib.FrameStats * count)()
    _lib.call("gg_frames_stats_f32_noalloc", ctypes.c_void_p(dev_frames), ctypes.c_int64(count),
              ctypes.c_int64(pixels), ctypes.c_int64(stride), None, out)
    return [(s.mean, s.std, s.valid_pixels, s.total_pixels) for s in out]


def test_noalloc_stats_match_stack_stats_twice(native):
    rng = np.random.default_rng(2024)
    n, h, w = 5, 67, 93
    frames = (900.0 + 35.0 * rng.standard_normal((n, h, w))).astype(np.float32)
    frames[1, :4, :7] = np.nan
    frames[3, 10, 10] = np.inf
    stack = native.ResidentCalibratedStack(n, h, w)
    for i in range(n):
        stack.upload_calibrated_frame(i, frames[i])
    ptrs = stack.device_pointers()
    stride = stack.frame_stride  # frames sit in slots 0..n-1 before any warp
    expected = stack.frames_global_stats(np.arange(n))
    for _ in range(2):
        got = _noalloc_stats(ptrs["slots"], n, h * w, stride)
        for k in range(n):
            mean, std, valid, total = got[k]
            assert valid == expected[k]["valid_pixels"]
            assert total == h * w
            np.testing.assert_allclose(mean, expected[k]["mean"], rtol=1e-12)
            np.testing.assert_allclose(std, expected[k]["std"], rtol=1e-7)
    # a different, smaller batch after the first two calls sees no stale scratch
    got = _noalloc_stats(ptrs["slots"] + 2 * stride * 4, 2, h * w, stride)
    for k in range(2):
        np.testing.assert_allclose(got[k][0], expected[k + 2]["mean"], rtol=1e-12)
    stack.close()


def test_noalloc_rejects_more_frames_than_the_scratch_holds(native):
    with pytest.raises(ValueError, match="at most 64 frames"):
        _noalloc_stats(1, 65, 16, 16)
