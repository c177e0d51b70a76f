"""GPU parity of the fused uint16 decode + calibration kernel (bit-exact)."""

from __future__ import annotations

import ast

import numpy as np
import pytest

from oracle import calibration as ocal

pytestmark = pytest.mark.gpu


def _case_args(g, spec):
    return (g["bias"] if spec["bias"] else None, g["dark"] if spec["dark"] else None,
            g["flat"] if spec["flat"] else None)


def test_calibrate_tile_matches_reference_golden(native, golden_calibration):
    g = golden_calibration
    for k, spec in enumerate(ast.literal_eval(str(s)) for s in g["_specs"]):
        bias, dark, flat = _case_args(g, spec)
        out = native.calibrate_tile_f32(g["light"].astype(np.float32), bias, dark, flat, spec["t_light"],
                                        spec["t_dark"], spec["policy"])
        np.testing.assert_array_equal(out, g[f"case{k}/out"], err_msg=str(spec))


def test_resident_u16_calibration_matches_reference_golden(native, golden_calibration):
    g = golden_calibration
    light = g["light"]
    h, w = light.shape
    for k, spec in enumerate(ast.literal_eval(str(s)) for s in g["_specs"]):
        bias, dark, flat = _case_args(g, spec)
        s = native.ResidentCalibratedStack(3, h, w)
        s.set_calibration_masters(bias, dark, flat)
        raw = np.stack([light, light[::-1], light[:, ::-1]])
        s.calibrate_frames_u16([2, 0, 1], raw, spec["t_light"], spec["t_dark"], spec["policy"])
        out = s.download_frame(2)
        np.testing.assert_array_equal(out, g[f"case{k}/out"], err_msg=str(spec))
        expected0 = ocal.calibrate_light(light[::-1], bias, dark, flat, spec["t_light"], spec["t_dark"],
                                         **_policy_kwargs(spec["policy"]))
        np.testing.assert_array_equal(s.download_frame(0), expected0)
        s.close()


def _policy_kwargs(policy):
    return {
        "master_dark_includes_bias": policy.get("master_dark_includes_bias", True),
        "dark_scaling_enabled": policy.get("dark_scaling_enabled", True),
        "flat_floor": policy.get("flat_floor", 1.0e-6),
        "pedestal": policy.get("pedestal", 0.0),
    }


@pytest.mark.parametrize("shape", [(64, 96), (7, 13), (1, 1)])
def test_fits_big_endian_bzero_path(native, shape):
    rng = np.random.default_rng(17)
    n = 6
    h, w = shape
    values = rng.integers(0, 65536, size=(n, h, w)).astype(np.uint16)
    bias = (300 + rng.standard_normal((h, w))).astype(np.float32)
    dark = (310 + rng.standard_normal((h, w))).astype(np.float32)
    flat = rng.uniform(0.9, 1.1, (h, w)).astype(np.float32)
    s = native.ResidentCalibratedStack(n, h, w)
    s.set_calibration_masters(bias, dark, flat)
    raws = [ocal.encode_fits_u16be(values[i]) for i in range(n)]
    released = []
    s.calibrate_frames_fits_u16be_bzero_host_async_multistream_callback_release_timed(
        np.arange(n), raws, np.full(n, 300.0), np.full(n, 150.0), 2, 2, released.append, {"pedestal": 100.0})
    assert sorted(released) == list(range(n))
    for i in range(n):
        expected = ocal.calibrate_light(values[i], bias, dark, flat, 300.0, 150.0, pedestal=100.0)
        np.testing.assert_array_equal(s.download_frame(i), expected)
    assert s.loaded_count == n


def test_many_frames_through_pinned_lanes(native):
    rng = np.random.default_rng(23)
    n, h, w = 19, 40, 56
    raw = rng.integers(0, 4096, size=(n, h, w)).astype(np.uint16)
    bias = np.full((h, w), 100.0, np.float32)
    s = native.ResidentCalibratedStack(n, h, w)
    s.set_calibration_masters(bias, None, None)
    pinned = native.host_pinned_empty_u8(raw.nbytes).view(np.uint16).reshape(raw.shape)
    pinned[...] = raw
    s.calibrate_frames_u16(np.arange(n), pinned, 1.0, None)
    tiles = s.download_frames_tile(np.arange(n), 3, 5, 50, 33)
    np.testing.assert_array_equal(tiles, (raw.astype(np.float32) - bias)[:, 5:33, 3:50])


def test_winsorized_masters_match_oracle(native):
    """Master frames by winsorized sigma clipping (the reference's hardened
    winsorized master path) equal the oracle's integration of the decoded
    calibration frames; a hot streak in one frame is rejected."""
    from glass_gb300.pipeline import build_masters
    from oracle.integration import weighted_integrate_stack

    rng = np.random.default_rng(21)
    bias = rng.integers(480, 520, size=(7, 24, 40)).astype(np.uint16)
    bias[2, 5, 3:9] = 9000  # a cosmic-ray streak in one bias frame
    m = build_masters(bias, None, None, method="winsorized")
    exp, *_ = weighted_integrate_stack(bias.astype(np.float32), None, "winsorized_sigma", 3.0, 3.0, 3, 0.5)
    np.testing.assert_allclose(m.bias, exp, rtol=2e-7, atol=0)
    assert float(m.bias[5, 5]) < 530.0
    mean = build_masters(bias, None, None)
    assert float(mean.bias[5, 5]) > 1000.0
    with pytest.raises(ValueError):
        build_masters(bias, None, None, method="median")
