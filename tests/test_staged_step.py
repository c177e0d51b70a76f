"""Staged ingest: the end-to-end step that uploads the whole raw stack on the
copy stream up front and runs the per-frame stages (calibrate, catalogs,
registration, refinement, quality, warp) chunk by chunk while later chunks
are still in flight.

It must give the batched step's answers: the same registrations (status,
inliers) and quality decisions, refined matrices within 1e-6 px of each
other (the registration-quality sums are reduced over a CTA count that
depends on the frames sharing a launch), the same zero-weight frames and
count maps, and masters within 1e-5 of the batched ones relative to their
range; a second staged step reproduces the first bit for bit, also when its
upload was started (prefetched) behind the previous step's integration.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(frames=40):
    from glass_gb300.synthetic import StackConfig, generate

    cfg = StackConfig(frames=frames, height=192, width=224, stars=90, hot_pixel_fraction=1e-4,
                      cosmic_ray_density=1e-4, max_shift=5.0, max_rotation_deg=0.2, calibration_frames=3, seed=21)
    return generate(cfg)


def _pipe(data):
    from glass_gb300.pipeline import ResidentPipeline, StepConfig, build_masters

    n, h, w = data.lights.shape
    masters = build_masters(data.bias_frames, data.dark_frames, data.flat_frames)
    return ResidentPipeline(n, h, w, masters, StepConfig(refine_method="gradient", star_max_stars=200))


def test_staged_step_matches_batched_step(native):
    import torch

    from glass_gb300.adjoint import registration_rms_px

    data = _data()
    n, h, w = data.lights.shape
    pinned = torch.from_numpy(data.lights.view(np.int16)).pin_memory().numpy().view(np.uint16)
    a, b = _pipe(data), _pipe(data)
    try:
        maps_a = a.step_host(pinned, register=True, staged=False)
        assert [len(c) for c in b.frame_chunks(2)] == [20, 20]
        assert [len(c) for c in b.frame_chunks(3)] == [13, 14, 13]
        b.staged_chunks = 2  # chunked processing, the second half still in flight
        maps_b = b.step_host(pinned, register=True, staged=True)
        reg_a = {r["frame"]: r for r in a.last_registration}
        reg_b = {r["frame"]: r for r in b.last_registration}
        assert sorted(reg_a) == sorted(reg_b) == list(range(1, n))
        for k in reg_a:
            assert (reg_a[k]["status"], reg_a[k]["inliers"]) == (reg_b[k]["status"], reg_b[k]["inliers"]), k
        ref_a = {r["frame"]: r for r in a.last_refinement}
        ref_b = {r["frame"]: r for r in b.last_refinement}
        assert sorted(ref_a) == sorted(ref_b) and len(ref_a) >= n - 2
        for k in ref_a:
            assert registration_rms_px([ref_a[k]["matrix"]], [ref_b[k]["matrix"]], h, w) < 1e-6, k
        np.testing.assert_array_equal(a._accepted, b._accepted)
        wa, wb = a.stack.device_frame_weights(), b.stack.device_frame_weights()
        np.testing.assert_array_equal(wa <= 0, wb <= 0)
        np.testing.assert_allclose(wa, wb, rtol=1e-5)
        for k in (2, 3, 4):  # coverage, low, high
            assert np.mean(maps_a[k] == maps_b[k]) > 0.999, k
        fin = np.isfinite(maps_a[0]) & np.isfinite(maps_b[0])
        span = float(np.nanmax(maps_a[0]) - np.nanmin(maps_a[0]))
        assert np.max(np.abs(maps_a[0][fin] - maps_b[0][fin])) <= 1e-5 * span

        again = b.step_host(pinned, register=True, staged=True, prefetch=pinned)
        for k in range(5):
            np.testing.assert_array_equal(again[k], maps_b[k], err_msg=f"map {k}")
        # the prefetched upload serves the next step, which skips its own
        assert b._prefetched == pinned.ctypes.data
        third = b.step_host(pinned, register=True, staged=True)
        assert b._prefetched is None
        for k in range(5):
            np.testing.assert_array_equal(third[k], maps_b[k], err_msg=f"map {k}")
    finally:
        a.close()
        b.close()


def test_staged_upload_needs_pinned_memory(native):
    data = _data(frames=10)
    p = _pipe(data)
    try:
        with pytest.raises(ValueError):
            p.upload_raw(np.ascontiguousarray(data.lights))  # pageable
        with pytest.raises(ValueError):
            p.calibrate_staged([0])  # nothing staged yet
    finally:
        p.close()
