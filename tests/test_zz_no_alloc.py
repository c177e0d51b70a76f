"""The allocation-free frame-statistics entry point.

gg_frames_stats_f32_noalloc serves callers that cannot call cudaMalloc
(plugins whose host application owns every device allocation, real-time loops
that forbid allocation after start-up): it reduces into a fixed __device__
scratch array instead of allocating.  Here it is called through the C ABI on frames that live in a
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


def _noalloc_stats(dev_frames: int, count: int, pixels: int, stride: int, stream: int | None = None):
    out = (_lib.FrameStats * count)()
    _lib.call("gg_frames_stats_f32_noalloc", ctypes.c_void_p(dev_frames), ctypes.c_int64(count),
              ctypes.c_int64(pixels), ctypes.c_int64(stride), ctypes.c_void_p(stream), out)
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


def test_noalloc_on_a_caller_stream_at_the_frame_limit(native):
    """64 frames (the scratch's limit) on a non-default stream the caller owns,
    twice in a row, against the stack's own statistics."""
    import torch

    rng = np.random.default_rng(77)
    n, h, w = 64, 40, 52
    frames = (1200.0 + 50.0 * rng.standard_normal((n, h, w))).astype(np.float32)
    frames[7, 3:9, 2:5] = np.nan
    frames[63, -1, -1] = -np.inf
    stack = native.ResidentCalibratedStack(n, h, w)
    for i in range(n):
        stack.upload_calibrated_frame(i, frames[i])
    expected = stack.frames_global_stats(np.arange(n))
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    ptrs = stack.device_pointers()
    for _ in range(2):
        got = _noalloc_stats(ptrs["slots"], n, h * w, stack.frame_stride, stream.cuda_stream)
        for k in range(n):
            assert got[k][2] == expected[k]["valid_pixels"]
            np.testing.assert_allclose(got[k][0], expected[k]["mean"], rtol=1e-12)
            np.testing.assert_allclose(got[k][1], expected[k]["std"], rtol=1e-7)
    stack.close()


def test_noalloc_refuses_a_capturing_stream_and_keeps_the_capture(native):
    """A call on a stream under capture is refused before anything is
    enqueued; the capture still completes and replays."""
    import torch

    n, h, w = 2, 16, 24
    frames = np.arange(n * h * w, dtype=np.float32).reshape(n, h, w)
    dev = torch.from_numpy(frames).cuda()
    _noalloc_stats(dev.data_ptr(), n, h * w, h * w)  # resolves the scratch address before capture
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    out = torch.zeros(n * h * w, device="cuda")
    with torch.cuda.graph(graph, stream=stream):
        with pytest.raises(ValueError, match="being captured"):
            _noalloc_stats(dev.data_ptr(), n, h * w, h * w, torch.cuda.current_stream().cuda_stream)
        out.copy_(dev.reshape(-1) * 2.0)
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(out.cpu(), torch.from_numpy(frames.reshape(-1) * 2.0))
