"""Launch-shape autotuner: the choice is recorded per problem shape, and the
outputs do not depend on it (only launch shapes are tuned)."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data():
    from glass_gb300.synthetic import StackConfig, generate

    cfg = StackConfig(frames=6, height=144, width=176, stars=50, max_shift=4.0, max_rotation_deg=0.2,
                      calibration_frames=3, seed=21)
    return generate(cfg)


def test_autotune_records_choices_and_preserves_results(native):
    import torch

    from glass_gb300 import _lib
    from glass_gb300.pipeline import DEFAULT_REFINE, ResidentPipeline, StepConfig, build_masters

    d = _data()
    n, h, w = d.lights.shape
    masters = build_masters(d.bias_frames, d.dark_frames, d.flat_frames)
    pipe = ResidentPipeline(n, h, w, masters, StepConfig(refine=dict(DEFAULT_REFINE)))
    raw = torch.from_numpy(d.lights.view(np.int16)).cuda()
    try:
        _lib.autotune_set_enabled(False)
        _lib.autotune_clear()
        pipe.step_device_fused(raw.data_ptr(), d.truth_matrices)
        fixed = pipe.stack.download_maps("full", include_dq=False)
        pipe.calibrate_device(raw.data_ptr())
        refined_fixed = pipe.refine(d.truth_matrices, 0)
        assert _lib.autotune_entries() == []

        _lib.autotune_set_enabled(True)
        pipe.step_device_fused(raw.data_ptr(), d.truth_matrices)
        tuned = pipe.stack.download_maps("full", include_dq=False)
        pipe.calibrate_device(raw.data_ptr())
        refined_tuned = pipe.refine(d.truth_matrices, 0)
        entries = {e["kernel"]: e for e in _lib.autotune_entries()}
        assert "fused_warp_integrate tile" in entries and "metric_partials bands" in entries
        assert entries["fused_warp_integrate tile"]["choice"] in {"128x1", "64x2", "32x4"}
        assert entries["metric_partials bands"]["candidates"] == 3
        assert all(e["ms"] > 0.0 for e in entries.values())
        for k in range(5):
            np.testing.assert_array_equal(tuned[k], fixed[k], err_msg=f"map {k}")
        # the band split changes the float64 summation order only
        np.testing.assert_allclose(refined_tuned, refined_fixed, rtol=0, atol=1e-6)
        _lib.autotune_clear()
        assert _lib.autotune_entries() == []
    finally:
        _lib.autotune_set_enabled(True)
        pipe.close()
