"""Deterministic grid star catalogs (the resident triangle path's batch
catalog): the oracle against the reference tests' known answers
(tests/test_gpu_star_detect.py:186-238 of the reference), then the CUDA path
(gg_stack_star_grid_catalog through the drop-in shim) against the oracle:
candidate counts, kept counts, positions and values bit-exact; centroids within
1 float32 ulp of the oracle's float64 sums (the same sums in the same order,
so normally identical)."""

from __future__ import annotations

import numpy as np
import pytest

from oracle.catalog import grid_catalog, local_maxima


def _five_peaks():
    image = np.zeros((32, 32), dtype=np.float32)
    image[6, 6] = 50.0
    image[7, 7] = 49.0
    image[24, 6] = 48.0
    image[6, 24] = 47.0
    image[24, 24] = 46.0
    return image


def test_oracle_grid_known_answer():
    """Reference test :186-202: 2 x 2 grid, 2 per cell, 4 kept, separation 4."""
    r = grid_catalog(_five_peaks(), 10.0, 2, 2, 2, 4, 4.0)
    assert r["count"] == 4  # (7, 7) is not a local maximum: its neighbour (6, 6) is brighter
    assert r["stored_count"] == 4
    assert {(int(x), int(y)) for x, y in zip(r["x"], r["y"])} == {(6, 6), (24, 6), (6, 24), (24, 24)}
    assert list(r["flux"]) == [50.0, 48.0, 47.0, 46.0]


def test_oracle_grid_second_frame_known_answer():
    """Reference test :205-238, second frame."""
    image = np.zeros((32, 32), dtype=np.float32)
    image[5, 5] = 60.0
    image[20, 8] = 42.0
    image[9, 23] = 41.0
    image[22, 22] = 40.0
    r = grid_catalog(image, 10.0, 2, 2, 2, 4, 4.0)
    assert r["count"] == 4 and r["stored_count"] == 4
    assert [(int(x), int(y)) for x, y in zip(r["x"], r["y"])] == [(5, 5), (8, 20), (23, 9), (22, 22)]


def test_oracle_local_maximum_rule():
    """Interior, finite, above threshold, not below any neighbour (reference
    test :24-42 with its NaN and border pixels)."""
    image = np.zeros((8, 9), dtype=np.float32)
    image[2, 3] = 10.0
    image[5, 6] = 20.0
    image[1, 1] = 4.0
    image[4, 4] = np.nan
    image[0, 3] = 100.0
    assert sorted((y, x) for _, y, x in local_maxima(image, 5.0)) == [(2, 3), (5, 6)]


def test_oracle_order_ties_and_separation():
    """Equal values are ordered by y then x; the separation scan keeps the
    first of two close candidates in that order."""
    image = np.zeros((16, 16), dtype=np.float32)
    image[4, 9] = 30.0
    image[4, 6] = 30.0
    image[9, 2] = 30.0
    r = grid_catalog(image, 1.0, 1, 1, 8, 8, 3.5)
    assert [(int(x), int(y)) for x, y in zip(r["x"], r["y"])] == [(6, 4), (2, 9)]


def _star_field(rng, h, w, stars, nan_patch=False):
    img = rng.normal(100.0, 3.0, (h, w)).astype(np.float32)
    yy, xx = np.mgrid[0:h, 0:w]
    for _ in range(stars):
        x, y = rng.uniform(2, w - 3), rng.uniform(2, h - 3)
        img += (rng.uniform(200, 5000) * np.exp(-((xx - x) ** 2 + (yy - y) ** 2) / (2 * 1.3 ** 2))).astype(np.float32)
    if nan_patch:
        img[h // 3:h // 3 + 5, w // 2:w // 2 + 7] = np.nan
    return img


@pytest.fixture
def stack_of(native):
    made = []

    def make(frames):
        s = native.ResidentCalibratedStack(len(frames), frames[0].shape[0], frames[0].shape[1])
        for k, f in enumerate(frames):
            s.upload_calibrated_frame(k, f)
        made.append(s)
        return s

    yield make
    for s in made:
        s.close()


def _check(got, exp):
    assert got["count"] == exp["count"]
    assert got["stored_count"] == exp["stored_count"]
    np.testing.assert_array_equal(got["flux"], exp["flux"])
    for key in ("x", "y"):
        g, e = np.asarray(got[key], np.float32), np.asarray(exp[key], np.float32)
        assert np.all(np.abs(g - e) <= np.spacing(np.maximum(np.abs(e), 1.0)))


@pytest.mark.gpu
def test_gpu_grid_known_answers(stack_of):
    s = stack_of([_five_peaks()])
    r = s.star_grid_top_nms_candidates(0, 10.0, 2, 2, 2, 4, 4.0)
    assert r["count"] == 4 and r["stored_count"] == 4
    assert {(int(x), int(y)) for x, y in zip(r["x"], r["y"])} == {(6, 6), (24, 6), (6, 24), (24, 24)}


@pytest.mark.gpu
@pytest.mark.parametrize("case", [
    # (h, w, stars, threshold, cols, rows, K, max_out, sep, radius, global_mean)
    (256, 320, 60, 150.0, 4, 3, 8, 40, 6.0, 0, False),
    (256, 320, 60, 150.0, 4, 3, 8, 40, 6.0, 4, False),
    (256, 320, 60, 150.0, 4, 3, 8, 40, 6.0, 3, True),
    (300, 257, 200, 120.0, 8, 8, 48, 500, 2.0, 8, False),
    (400, 400, 30, 101.0, 3, 1, 700, 300, 0.0, 2, False),   # noise peaks: compaction in every cell
    (512, 512, 400, 120.0, 24, 16, 48, 400, 4.0, 3, False),  # 18,432 kept keys: the global-memory sort
])
def test_gpu_grid_catalog_matches_oracle(stack_of, case):
    h, w, stars, thr, cols, rows, k, mo, sep, radius, gmean = case
    rng = np.random.default_rng(h * 7 + w + stars)
    frames = [_star_field(rng, h, w, stars, nan_patch=(i == 1)) for i in range(3)]
    s = stack_of(frames)
    got = s.star_grid_top_nms_candidates_batch_deterministic_centroid([0, 1, 2], thr, cols, rows, k, mo, sep,
                                                                       radius, gmean)
    for i, g in enumerate(got):
        assert g["frame_index"] == i
        _check(g, grid_catalog(frames[i], thr, cols, rows, k, mo, sep, radius, gmean))


@pytest.mark.gpu
def test_gpu_batch_equals_single_calls_and_repeats(stack_of):
    """Batch results equal single-frame calls (reference test :205-238), and
    a dense field gives the same catalog on every call (reference :241-268)."""
    rng = np.random.default_rng(20260513)
    image = rng.normal(0.0, 0.01, size=(192, 192)).astype(np.float32)
    for index in range(900):
        image[2 + (index * 53) % 188, 2 + (index * 37) % 188] = np.float32(1000.0 + index)
    second = _star_field(np.random.default_rng(5), 192, 192, 50)
    s = stack_of([image, second])
    batch = s.star_grid_top_nms_candidates_batch_deterministic([0, 1], 100.0, 12, 12, 4, 64, 8.0)
    for i in range(2):
        single = s.star_grid_top_nms_candidates_deterministic(i, 100.0, 12, 12, 4, 64, 8.0)
        for key in ("x", "y", "flux"):
            np.testing.assert_array_equal(batch[i][key], single[key])
    first = batch[0]
    for _ in range(3):
        again = s.star_grid_top_nms_candidates_batch_deterministic([0], 100.0, 12, 12, 4, 64, 8.0)[0]
        for key in ("x", "y", "flux"):
            np.testing.assert_array_equal(again[key], first[key])
    _check(first, grid_catalog(image, 100.0, 12, 12, 4, 64, 8.0))


@pytest.mark.gpu
def test_gpu_grid_catalog_rejects_bad_arguments(stack_of):
    s = stack_of([np.zeros((16, 16), np.float32)])
    with pytest.raises(ValueError):
        s.star_grid_top_nms_candidates(0, 1.0, 0, 2, 2, 4, 1.0)
    with pytest.raises(ValueError):
        s.star_grid_top_nms_candidates(0, 1.0, 2, 2, 2, 4, -1.0)
    with pytest.raises(ValueError):
        s.star_grid_top_nms_candidates(0, 1.0, 2, 2, 5000, 4, 1.0)
