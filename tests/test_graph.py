"""CUDA-graph capture of the resident step with fixed matrices.

The captured sequence (calibrate from device uint16 -> simple-SNR weights ->
fused Lanczos3 warp + winsorized rejection + integration) must reproduce the
eager launch sequence bit for bit, read the raw frames afresh at every
replay, and report the kernels it replays in the library's launch counter.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(seed, frames=8):
    from glass_gb300.synthetic import StackConfig, generate

    cfg = StackConfig(frames=frames, height=160, width=192, stars=60, hot_pixel_fraction=1e-4,
                      cosmic_ray_density=1e-4, max_shift=5.0, max_rotation_deg=0.2, calibration_frames=3, seed=seed)
    return generate(cfg)


@pytest.mark.parametrize("frames", [8, 40])
def test_graph_replay_matches_eager(native, frames):
    """8 frames: the column kernel; 40: the warp-per-pixel fused kernel."""
    import torch

    from glass_gb300 import _lib
    from glass_gb300.pipeline import ResidentPipeline, StepConfig, build_masters

    a, b = _data(11, frames), _data(12, frames)
    n, h, w = a.lights.shape
    masters = build_masters(a.bias_frames, a.dark_frames, a.flat_frames)
    pipe = ResidentPipeline(n, h, w, masters, StepConfig())
    try:
        raw = torch.from_numpy(a.lights.view(np.int16)).cuda()
        pipe.step_device_fused(raw.data_ptr(), a.truth_matrices)
        eager_a = pipe.stack.download_maps("full", include_dq=False)
        raw_b = torch.from_numpy(b.lights.view(np.int16)).cuda()
        pipe.step_device_fused(raw_b.data_ptr(), a.truth_matrices)
        eager_b = pipe.stack.download_maps("full", include_dq=False)

        kernels = pipe.capture_graph(raw.data_ptr(), a.truth_matrices)
        assert kernels >= 4
        before = _lib.kernel_launches()
        pipe.launch_graph()
        assert _lib.kernel_launches() - before == kernels
        got_a = pipe.stack.download_maps("full", include_dq=False)
        for k in range(5):
            np.testing.assert_array_equal(got_a[k], eager_a[k], err_msg=f"map {k}")
        raw.copy_(raw_b)  # the graph reads the raw frames at every replay
        pipe.launch_graph()
        got_b = pipe.stack.download_maps("full", include_dq=False)
        for k in range(5):
            np.testing.assert_array_equal(got_b[k], eager_b[k], err_msg=f"map {k}")
        assert not np.array_equal(got_a[0], got_b[0])
        pipe.stack.destroy_step_graph()
        with pytest.raises(ValueError):
            pipe.launch_graph()
    finally:
        pipe.close()


def test_graph_capture_rejects_unsupported(native):
    import torch

    from glass_gb300.pipeline import ResidentPipeline, StepConfig, build_masters

    a = _data(13)
    n, h, w = a.lights.shape
    masters = build_masters(a.bias_frames, a.dark_frames, a.flat_frames)
    pipe = ResidentPipeline(n, h, w, masters, StepConfig(interpolation="nearest"))
    try:
        raw = torch.from_numpy(a.lights.view(np.int16)).cuda()
        with pytest.raises(ValueError):
            pipe.capture_graph(raw.data_ptr(), a.truth_matrices)
        with pytest.raises(ValueError):
            pipe.stack.capture_step_graph(raw.data_ptr(), a.truth_matrices, pipe._calib_params(),
                                          weighting="median")
    finally:
        pipe.close()
