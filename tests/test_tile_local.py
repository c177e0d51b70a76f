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


# ---- pinned to the reference: tests/golden/tile_local.npz holds the
# reference test's own CPU expectation (`_expected_tile_local_sigma`,
# tests/test_cuda_resident_stack.py:523-583 of the reference) on seeded stacks
# with NaNs, a zero weight and non-overlapping tiles; "mean" is that
# expectation with no rejection.  Tolerances are the reference test's:
# 1e-6 for the mean (:518-519), 2e-5 for the clipped maps (:634-639).
def _golden_cases():
    from .conftest import GOLDEN

    g = np.load(GOLDEN / "tile_local.npz", allow_pickle=False)
    for name in (str(n) for n in g["_names"]):
        yield name, g


def _close(got, exp, tol, tag):
    np.testing.assert_allclose(np.asarray(got, np.float64), np.asarray(exp, np.float64), rtol=tol, atol=tol,
                               err_msg=tag)


def test_oracle_tile_local_matches_reference_expectation():
    n = 0
    for name, g in _golden_cases():
        args = (g[f"{name}/frames"], g[f"{name}/weights"], g[f"{name}/target"], g[f"{name}/extents"],
                g[f"{name}/multipliers"])
        m, w = otl.integrate_tile_local(*args, "mean")
        _close(m, g[f"{name}/mean/master"], 1e-6, name + " mean master")
        _close(w, g[f"{name}/mean/weight"], 1e-6, name + " mean weight")
        for mode in ("sigma", "winsorized"):
            got = otl.integrate_tile_local(*args, mode, 3.0, 1.0)
            for key, arr in zip(("master", "weight", "coverage", "low", "high"), got):
                _close(arr, g[f"{name}/{mode}/{key}"], 2e-5, f"{name} {mode} {key}")
        n += 1
    assert n == 8


@pytest.mark.gpu
def test_gpu_tile_local_matches_reference_expectation(native):
    for name, g in _golden_cases():
        frames = g[f"{name}/frames"]
        s = native.ResidentCalibratedStack(*frames.shape)
        try:
            for k in range(frames.shape[0]):
                s.upload_calibrated_frame(k, frames[k])
            args = (g[f"{name}/target"], g[f"{name}/extents"], g[f"{name}/multipliers"], g[f"{name}/weights"])
            m, w = s.integrate_tile_local_mean(*args)[:2]
            _close(m, g[f"{name}/mean/master"], 1e-6, name + " mean master")
            _close(w, g[f"{name}/mean/weight"], 1e-6, name + " mean weight")
            for mode in ("sigma", "winsorized"):
                got = s.integrate_tile_local_sigma_clip(*args, 3.0, 1.0, winsorize=mode == "winsorized")[:5]
                for key, arr in zip(("master", "weight", "coverage", "low", "high"), got):
                    _close(arr, g[f"{name}/{mode}/{key}"], 2e-5, f"{name} {mode} {key}")
        finally:
            s.close()
