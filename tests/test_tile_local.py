"""Tile-local weighted integration (the reference's
integrate_tile_local_mean / integrate_tile_local_sigma_clip).

CPU: the oracle with every multiplier 1 equals plain per-frame weighting,
and a multiplier of 0 removes the target frames inside its tile.
GPU: maps bit-exact against the oracle (float32 frame-order arithmetic on
both sides), argument rules as the reference's.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import tile_local as otl

EXTENTS = np.array([[0, 0, 40, 30], [40, 0, 96, 30], [10, 30, 70, 64]], dtype=np.int32)
MULTS = np.array([0.5, 2.0, 0.0], dtype=np.float32)


def _stack(seed, n=9, h=64, w=96):
    rng = np.random.default_rng(seed)
    data = rng.normal(500.0, 12.0, (n, h, w)).astype(np.float32)
    data[2, 5:9, 5:9] = np.float32(5000.0)
    data[4, 40:44, 20:24] = np.float32(-900.0)
    data[6, :, :3] = np.nan
    weights = rng.uniform(0.5, 1.5, n).astype(np.float32)
    weights[7] = 0.0
    target = np.zeros(n, dtype=bool)
    target[[1, 2, 5]] = True
    return data, weights, target


def test_oracle_unit_multipliers_equal_plain_weighting():
    data, weights, target = _stack(1)
    m1, w1 = otl.integrate_tile_local(data, weights, target, EXTENTS, np.ones(3, np.float32), "mean")
    m0, w0 = otl.integrate_tile_local(data, weights, np.zeros_like(target), EXTENTS, MULTS, "mean")
    np.testing.assert_array_equal(m1, m0)
    np.testing.assert_array_equal(w1, w0)


def test_oracle_zero_multiplier_drops_targets_in_tile():
    data, weights, target = _stack(2)
    _, w = otl.integrate_tile_local(data, weights, target, EXTENTS, MULTS, "mean")
    inside = w[40:60, 20:60]  # tile 2 (multiplier 0)
    expect = np.float32(0.0)
    for f in range(data.shape[0]):
        if not target[f] and weights[f] > 0:
            expect = np.float32(expect + weights[f])
    # frame 6 is NaN only in columns 0-2, outside this window
    np.testing.assert_array_equal(inside, np.full_like(inside, expect))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mean", "sigma", "winsorized"])
def test_gpu_tile_local_matches_oracle(native, mode):
    data, weights, target = _stack(3)
    n, h, w = data.shape
    s = native.ResidentCalibratedStack(n, h, w)
    try:
        for k in range(n):
            s.upload_calibrated_frame(k, data[k])
        if mode == "mean":
            got = s.integrate_tile_local_mean(target, EXTENTS, MULTS, weights)[:2]
        else:
            got = s.integrate_tile_local_sigma_clip(target, EXTENTS, MULTS, weights, 2.5, 2.5,
                                                    winsorize=mode == "winsorized")[:5]
    finally:
        s.close()
    exp = otl.integrate_tile_local(data, weights, target, EXTENTS, MULTS, mode, 2.5, 2.5)
    for k, (g, e) in enumerate(zip(got, exp)):
        np.testing.assert_array_equal(g, e, err_msg=f"{mode} map {k}")


@pytest.mark.gpu
def test_gpu_tile_local_arguments(native):
    data, weights, target = _stack(4)
    s = native.ResidentCalibratedStack(*data.shape)
    try:
        for k in range(data.shape[0]):
            s.upload_calibrated_frame(k, data[k])
        with pytest.raises(ValueError):  # no target frame
            s.integrate_tile_local_mean(np.zeros(data.shape[0], bool), EXTENTS, MULTS)
        with pytest.raises(ValueError):  # overlapping tiles
            s.integrate_tile_local_mean(target, np.array([[0, 0, 10, 10], [5, 5, 20, 20]]), [1.0, 1.0])
        with pytest.raises(ValueError):  # outside the image
            s.integrate_tile_local_mean(target, np.array([[0, 0, 97, 10]]), [1.0])
        with pytest.raises(ValueError):  # negative multiplier
            s.integrate_tile_local_mean(target, EXTENTS, [1.0, -1.0, 1.0])
        with pytest.raises(ValueError):
            s.integrate_tile_local_sigma_clip(target, EXTENTS, MULTS, low_sigma=0.0)
    finally:
        s.close()
