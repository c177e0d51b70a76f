"""Grid local normalisation (the resident grid_mean_std mode).

CPU: the oracle's coefficient rules and the per-tile apply are pinned to the
reference (golden vectors from resident_cuda.py:_grid_local_norm_coefficients
and cpu/local_norm.py:apply_grid_normalization, bit-exact), and a normalised
frame's tiles carry the reference frame's mean and std.

GPU: tile statistics equal to the oracle's float32 values (valid counts
exact; means and stds within one float32 ulp: float-float device sums vs
NumPy float64 sums), the apply bit-exact against the reference's output, and
the device-only sequence (statistics -> coefficients -> apply, zero weight
for a frame without paired pixels) equal to the oracle's sequence.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import local_norm as oln

from .conftest import GOLDEN


@pytest.fixture(scope="module")
def golden_ln():
    return np.load(GOLDEN / "local_norm.npz", allow_pickle=False)


def test_oracle_coefficients_match_reference(golden_ln):
    g = golden_ln
    stats = {k: g[f"coeff/{k}"] for k in ("source_mean", "source_std", "reference_mean", "reference_std",
                                          "valid_pixels")}
    scales, offsets = oln.grid_coefficients(stats, 1.0e-6)
    np.testing.assert_array_equal(scales, g["coeff/scales"])
    np.testing.assert_array_equal(offsets, g["coeff/offsets"])


def test_oracle_apply_matches_reference(golden_ln):
    g = golden_ln
    for name in [str(n) for n in g["_apply_names"]]:
        th, tw = (int(v) for v in g[f"apply/{name}/tile"])
        got = oln.apply_grid(g[f"apply/{name}/data"], g[f"apply/{name}/scales"], g[f"apply/{name}/offsets"], th, tw)
        np.testing.assert_array_equal(got, g[f"apply/{name}/out"], err_msg=name)


def _frames(seed, n=4, h=300, w=420):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    base = 800.0 + 0.4 * xx + 0.2 * yy
    frames = []
    for k in range(n):
        gain = rng.uniform(0.8, 1.2)
        grad = rng.uniform(-0.3, 0.3)
        f = gain * base + grad * xx + rng.uniform(-100, 100) + rng.normal(0, 10, (h, w))
        frames.append(f.astype(np.float32))
    frames = np.stack(frames)
    if n > 2:
        frames[1, :, :17] = np.nan  # a warped frame's empty border
        frames[2, 5:9, 40:300] = np.nan
    return frames


def test_oracle_normalised_tiles_follow_the_reference():
    frames = _frames(1)
    out, w = oln.normalize_frames(frames, 0, np.ones(4, np.float32), tile=64)
    for k in (1, 2, 3):
        st = oln.pair_grid_stats(out[k], out[0], 64, 64)
        ok = st["valid_pixels"] > 0
        np.testing.assert_allclose(st["source_mean"][ok], st["reference_mean"][ok], rtol=1e-5)
        np.testing.assert_allclose(st["source_std"][ok], st["reference_std"][ok], rtol=1e-4)
    assert np.all(w == 1.0)


# ---- GPU ---------------------------------------------------------------------------

def _stack(native, frames):
    s = native.ResidentCalibratedStack(frames.shape[0], frames.shape[1], frames.shape[2])
    for k in range(frames.shape[0]):
        s.upload_calibrated_frame(k, frames[k])
    return s


def _ulps(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))


@pytest.mark.gpu
@pytest.mark.parametrize("tile", [64, 100, 256])
def test_gpu_pair_stats_match_oracle(native, tile):
    frames = _frames(2)
    s = _stack(native, frames)
    try:
        got = s.frame_pair_grid_stats_batch(0, [1, 2, 3], tile, tile)
    finally:
        s.close()
    for pos, k in enumerate((1, 2, 3)):
        exp = oln.pair_grid_stats(frames[k], frames[0], tile, tile)
        fr = got["frames"][pos]
        np.testing.assert_array_equal(fr["valid_pixels"], exp["valid_pixels"])
        for key in ("source_mean", "source_std", "reference_mean", "reference_std"):
            assert _ulps(fr[key], exp[key]).max() <= 1, (k, key)


@pytest.mark.gpu
def test_gpu_apply_matches_reference(native, golden_ln):
    g = golden_ln
    for name in [str(n) for n in g["_apply_names"]]:
        data = g[f"apply/{name}/data"]
        th, tw = (int(v) for v in g[f"apply/{name}/tile"])
        s = _stack(native, data[None])
        try:
            s.apply_grid_normalization_frame(0, g[f"apply/{name}/scales"], g[f"apply/{name}/offsets"], th, tw)
            got = s.download_frame(0)
        finally:
            s.close()
        np.testing.assert_array_equal(got, g[f"apply/{name}/out"], err_msg=name)


@pytest.mark.gpu
def test_gpu_local_normalize_matches_oracle_sequence(native):
    frames = _frames(3, n=5)
    frames[4] = np.nan  # no paired pixel: weight 0, frame untouched
    s = _stack(native, frames)
    try:
        s.compute_frame_weights("prior", np.ones(5, np.float32), 1.0e-6, download=False)
        scales, offsets = s.local_normalize_grid(0, [1, 2, 3, 4], tile=128, download=True)
        got = np.stack([s.download_frame(k) for k in range(5)])
        weights = s.device_frame_weights()
    finally:
        s.close()
    exp, w_exp = oln.normalize_frames(frames, 0, np.ones(5, np.float32), tile=128)
    for k in range(1, 4):
        st = oln.pair_grid_stats(frames[k], frames[0], 128, 128)
        sc, of = oln.grid_coefficients(st, 1.0e-6)
        assert _ulps(scales[k - 1], sc).max() <= 1 and _ulps(offsets[k - 1], of).max() <= 1
    # where the coefficients agree the frames agree bit for bit
    np.testing.assert_array_equal(np.isnan(got), np.isnan(exp))
    fin = np.isfinite(exp)
    assert _ulps(got[fin], exp[fin]).max() <= 2
    assert np.all(np.isnan(got[4]))
    np.testing.assert_array_equal(weights, w_exp)
    assert weights[4] == 0.0


@pytest.mark.gpu
def test_gpu_global_normalization(native):
    frames = _frames(4, n=1)
    s = _stack(native, frames)
    try:
        s.apply_global_normalization_frame(0, 1.25, -30.5)
        got = s.download_frame(0)
    finally:
        s.close()
    exp = frames[0] * np.float32(1.25) + np.float32(-30.5)
    np.testing.assert_array_equal(got, exp)
