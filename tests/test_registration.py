"""Triangle-asterism registration: the oracle is pinned to the reference's
estimate_triangle_asterism_transform, _local_triangle_descriptors and the
descriptor-list similarity fallback (golden vectors from
src/glass/cpu/registration.py and src/glass_cuda.py), and the GPU must agree.

GPU bar: descriptors (values, vertex order, areas) bit-exact; inlier counts,
status and the set of star pairs exact; matrices within 1e-9 absolute
(the 2x2 SVD is evaluated in closed form, so the last bits differ); rms
within 1e-9 relative + 1e-12 absolute.  The affine model (golden from the
reference estimator with transform_model="affine") has the same bar except
matrices within 1e-8 absolute: the device solves the centred normal
equations where the reference's lstsq goes through an SVD, and 3-point fits
of thin triangles are less well conditioned than Procrustes fits.
"""

from __future__ import annotations

import ast

import numpy as np
import pytest

from oracle import registration as oreg
from oracle import stars as ostars

from .conftest import GOLDEN


@pytest.fixture(scope="module")
def golden_reg():
    return np.load(GOLDEN / "registration.npz", allow_pickle=False)


@pytest.fixture(scope="module")
def golden_affine():
    return np.load(GOLDEN / "registration_affine.npz", allow_pickle=False)


def _names(g, key):
    return [str(n) for n in g[key]]


def _params(g, name):
    return ast.literal_eval(str(g[f"{name}/params"]))


# ---- oracle pinning (CPU) -----------------------------------------------------------
def test_oracle_estimator_matches_reference(golden_reg):
    g = golden_reg
    names = _names(g, "_names")
    assert len(names) >= 20
    for name in names:
        res = oreg.estimate_triangle_asterism_transform(g[f"{name}/ref"], g[f"{name}/mov"], **_params(g, name))
        assert res["inliers"] == int(g[f"{name}/inliers"]), name
        assert res["status"] == str(g[f"{name}/status"]), name
        assert [tuple(p) for p in res["pairs"]] == [tuple(p) for p in g[f"{name}/pairs"].tolist()], name
        np.testing.assert_array_equal(res["matrix"], g[f"{name}/matrix"], err_msg=name)
        np.testing.assert_array_equal(res["rms_px"], g[f"{name}/rms_px"], err_msg=name)
        warn = [str(w) for w in g[f"{name}/warnings"]]
        for key, field in (("reference_descriptors", "reference_descriptor_count"),
                           ("moving_descriptors", "moving_descriptor_count"), ("descriptor_matches",
                                                                                "descriptor_matches")):
            found = [w for w in warn if w.startswith(f"triangle_asterism_{key}=")]
            if found:
                assert res[field] == int(found[0].split("=")[1]), (name, key)


def test_oracle_affine_estimator_matches_reference(golden_affine):
    g = golden_affine
    names = _names(g, "_names")
    assert len(names) >= 15
    for name in names:
        res = oreg.estimate_triangle_asterism_transform(g[f"{name}/ref"], g[f"{name}/mov"], transform_model="affine",
                                                        **_params(g, name))
        assert res["inliers"] == int(g[f"{name}/inliers"]), name
        assert res["status"] == str(g[f"{name}/status"]), name
        assert [tuple(p) for p in res["pairs"]] == [tuple(p) for p in g[f"{name}/pairs"].tolist()], name
        np.testing.assert_allclose(res["matrix"], g[f"{name}/matrix"], rtol=0, atol=1e-12, err_msg=name)
        np.testing.assert_allclose(res["rms_px"], g[f"{name}/rms_px"], rtol=1e-12, atol=1e-15, err_msg=name)


def test_oracle_affine_fit_recovers_shear():
    rng = np.random.default_rng(3)
    mov = rng.uniform(0.0, 1000.0, (12, 2))
    lin = np.array([[1.003, 0.002], [-0.004, 0.998]])
    ref = mov @ lin.T + np.array([4.0, -9.0])
    m = oreg.fit_affine(mov, ref)
    np.testing.assert_allclose(m[:2, :2], lin, atol=1e-12)
    np.testing.assert_allclose(m[:2, 2], [4.0, -9.0], atol=1e-9)
    assert oreg.fit_affine(mov[:2], ref[:2]) is None


def test_oracle_descriptors_match_reference(golden_reg):
    g = golden_reg
    for name in _names(g, "_desc_names"):
        p = _params(g, name)
        desc = oreg.local_triangle_descriptors(g[f"{name}/points"], p["max_points"], p["neighbors"],
                                               p["max_descriptors"])
        np.testing.assert_array_equal(np.asarray([d[0] for d in desc]).reshape(-1, 2), g[f"{name}/descriptors"])
        np.testing.assert_array_equal(np.asarray([d[1] for d in desc]).reshape(-1, 3), g[f"{name}/indices"])
        np.testing.assert_array_equal(np.asarray([d[2] for d in desc]), g[f"{name}/areas"])


def test_oracle_descriptor_list_similarity_matches_reference(golden_reg):
    g = golden_reg
    for name in _names(g, "_list_names"):
        res = oreg.similarity_from_descriptors(g[f"{name}/ref"], g[f"{name}/mov"], g[f"{name}/ref_desc"],
                                               g[f"{name}/ref_idx"], g[f"{name}/mov_desc"], g[f"{name}/mov_idx"],
                                               float(g[f"{name}/tolerance_px"]), 0.1)
        assert res["inliers"] == int(g[f"{name}/inliers"])
        assert res["best_candidate_index"] == int(g[f"{name}/best_candidate_index"])
        np.testing.assert_array_equal(res["matrix"].astype(np.float32), g[f"{name}/matrix32"])
        np.testing.assert_array_equal(res["rms_px"], g[f"{name}/rms_px"])


def test_oracle_fit_recovers_known_similarity():
    """registration.py:140-162 on an exact similarity (closed-form check)."""
    rng = np.random.default_rng(5)
    mov = rng.uniform(0, 100, (7, 2))
    t = np.deg2rad(12.0)
    lin = 1.03 * np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
    ref = mov @ lin.T + np.array([4.0, -9.0])
    m = oreg.fit_similarity(mov, ref)
    np.testing.assert_allclose(m[:2, :2], lin, atol=1e-12)
    np.testing.assert_allclose(m[:2, 2], [4.0, -9.0], atol=1e-10)
    assert oreg.fit_similarity(mov[:1], ref[:1]) is None
    assert oreg.fit_similarity(np.ones((4, 2)), ref[:4]) is None


# ---- GPU parity -----------------------------------------------------------------------
def _check_result(name, got, g, matrix_atol=1e-9):
    assert got["inliers"] == int(g[f"{name}/inliers"]), name
    assert got["status"] == str(g[f"{name}/status"]), name
    exp_pairs = sorted(tuple(p) for p in g[f"{name}/pairs"].tolist())
    assert sorted(got["pairs"]) == exp_pairs, name
    np.testing.assert_allclose(got["matrix"], g[f"{name}/matrix"], rtol=0, atol=matrix_atol, err_msg=name)
    np.testing.assert_allclose(got["rms_px"], g[f"{name}/rms_px"], rtol=1e-9, atol=1e-12, err_msg=name)


@pytest.mark.gpu
def test_gpu_descriptors_match_reference(native, golden_reg):
    g = golden_reg
    for name in _names(g, "_desc_names"):
        p = _params(g, name)
        pts = g[f"{name}/points"]
        got = native.triangle_asterism_descriptors_f32(pts[:, 0], pts[:, 1], p["max_points"], p["neighbors"],
                                                       p["max_descriptors"])
        # the module API takes float32 catalogs: compare with the oracle on those
        pts32 = pts.astype(np.float32).astype(np.float64)
        desc = oreg.local_triangle_descriptors(pts32, p["max_points"], p["neighbors"], p["max_descriptors"])
        assert got["count"] == len(desc), name
        np.testing.assert_array_equal(got["indices"], np.asarray([d[1] for d in desc], np.int32).reshape(-1, 3))
        np.testing.assert_array_equal(got["descriptors"],
                                      np.asarray([d[0] for d in desc], np.float64).reshape(-1, 2).astype(np.float32))


@pytest.mark.gpu
def test_gpu_descriptors_float64_exact(native, golden_reg):
    """float64 catalogs through the C ABI: bit-exact against the reference."""
    import ctypes

    from glass_gb300 import _lib

    g = golden_reg
    for name in _names(g, "_desc_names"):
        p = _params(g, name)
        pts = np.ascontiguousarray(g[f"{name}/points"], dtype=np.float64)
        cap = 2000
        desc = np.zeros((cap, 2))
        idx = np.zeros((cap, 3), np.int32)
        areas = np.zeros(cap)
        count = ctypes.c_int64()
        _lib.call("gg_triangle_descriptors", _lib.ptr(pts), ctypes.c_int64(len(pts)),
                  ctypes.c_int32(p["max_points"]), ctypes.c_int32(p["neighbors"]),
                  ctypes.c_int32(p["max_descriptors"]), _lib.ptr(desc), _lib.ptr(idx), _lib.ptr(areas),
                  ctypes.c_int64(cap), ctypes.byref(count))
        n = int(count.value)
        np.testing.assert_array_equal(desc[:n], g[f"{name}/descriptors"], err_msg=name)
        np.testing.assert_array_equal(idx[:n], g[f"{name}/indices"], err_msg=name)
        np.testing.assert_array_equal(areas[:n], g[f"{name}/areas"], err_msg=name)


# Catalogs with an exact symmetry (a square grid maps onto itself under
# several similarities): every symmetric solution has the same pair count and
# an rms of ~1e-16, so the winner is decided by last-bit differences of the
# rms, which depend on how the 2x2 SVD is evaluated.  Both sides must find a
# perfect solution; which one is not pinned.
_EXACT_TIES = {"grid"}


@pytest.mark.gpu
def test_gpu_estimator_matches_reference(native, golden_reg):
    g = golden_reg
    for name in _names(g, "_names"):
        got = native.estimate_triangle_asterism_transform(g[f"{name}/ref"], g[f"{name}/mov"], **_params(g, name))
        if name in _EXACT_TIES:
            assert got["inliers"] == int(g[f"{name}/inliers"]), name
            assert got["status"] == str(g[f"{name}/status"]), name
            assert got["rms_px"] < 1e-9 and float(g[f"{name}/rms_px"]) < 1e-9, name
            lin = got["matrix"][:2, :2]
            np.testing.assert_allclose(lin @ lin.T, np.eye(2), atol=1e-9)
            continue
        _check_result(name, got, g)


@pytest.mark.gpu
def test_gpu_descriptor_list_similarity_matches_reference(native, golden_reg):
    g = golden_reg
    for name in _names(g, "_list_names"):
        ref, mov = g[f"{name}/ref"], g[f"{name}/mov"]
        got = native.estimate_similarity_from_triangle_descriptors_f32(
            ref[:, 0], ref[:, 1], mov[:, 0], mov[:, 1], g[f"{name}/ref_desc"], g[f"{name}/ref_idx"],
            g[f"{name}/mov_desc"], g[f"{name}/mov_idx"], float(g[f"{name}/tolerance_px"]), 0.1)
        assert got["inliers"] == int(g[f"{name}/inliers"]), name
        assert got["best_candidate_index"] == int(g[f"{name}/best_candidate_index"]), name
        assert got["status"] == str(g[f"{name}/status"]), name
        np.testing.assert_allclose(np.asarray(got["matrix"], np.float32), g[f"{name}/matrix32"], rtol=1e-6,
                                   atol=1e-4, err_msg=name)
        np.testing.assert_allclose(got["rms_px"], g[f"{name}/rms_px"], rtol=1e-9, atol=1e-12, err_msg=name)


def _field(rng, h, w, stars, shift=(0.0, 0.0), noise=8.0):
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.full((h, w), 600.0)
    for x0, y0, flux in stars:
        img += flux * np.exp(-((xx - x0 - shift[0]) ** 2 + (yy - y0 - shift[1]) ** 2) / (2 * 1.3 ** 2))
    return (img + noise * rng.standard_normal((h, w))).astype(np.float32)


@pytest.mark.gpu
def test_gpu_stack_registration_from_device_catalogs(native):
    """detect_stars -> device catalogs -> registration, against the oracle run
    on the oracle's own detections of the same frames."""
    rng = np.random.default_rng(17)
    h, w, n = 160, 192, 4
    stars = [(rng.uniform(12, w - 12), rng.uniform(12, h - 12), rng.uniform(800, 20000)) for _ in range(70)]
    shifts = [(0.0, 0.0), (3.25, -2.5), (-6.0, 4.75), (1.5, 7.0)]
    frames = [_field(rng, h, w, stars, s) for s in shifts]
    s = native.ResidentCalibratedStack(n, h, w)
    try:
        for k in range(n):
            s.upload_calibrated_frame(k, frames[k])
        cats = s.detect_stars(list(range(n)), threshold_sigma=5.0, max_stars=120)
        got = s.register_frames_triangle(0, [1, 2, 3, 0], tolerance_px=2.0)
    finally:
        s.close()
    ref_cat = ostars.detect_stars(frames[0], threshold_sigma=5.0, max_stars=120)
    for pos, k in enumerate([1, 2, 3, 0]):
        cat = ostars.detect_stars(frames[k], threshold_sigma=5.0, max_stars=120)
        assert len(cat) == cats[k].size
        exp = oreg.estimate_triangle_asterism_transform([(c[0], c[1]) for c in ref_cat],
                                                        [(c[0], c[1]) for c in cat], tolerance_px=2.0)
        assert got[pos]["inliers"] == exp["inliers"], k
        assert got[pos]["status"] == exp["status"] == "ok", k
        np.testing.assert_allclose(got[pos]["matrix"], exp["matrix"], rtol=0, atol=1e-8)
        np.testing.assert_allclose(got[pos]["matrix"][:2, 2], shifts[0][0] - np.asarray(shifts[k]), atol=0.1)


@pytest.mark.gpu
def test_gpu_catalog_shape_filter_skips_streaks(native):
    """Streaks brighter than every star fill an unfiltered top-80 catalog;
    the eccentricity filter keeps the round stars and registration works."""
    rng = np.random.default_rng(23)
    h, w = 200, 240
    stars = [(rng.uniform(12, w - 12), rng.uniform(12, h - 12), rng.uniform(800, 9000)) for _ in range(90)]
    shifts = [(0.0, 0.0), (2.5, -1.75)]
    frames = []
    for sh in shifts:
        img = _field(rng, h, w, stars, sh)
        for _ in range(120):  # streaks 3-6 px long, 1 px wide
            x0, y0 = rng.integers(5, w - 12), rng.integers(5, h - 12)
            length = int(rng.integers(3, 7))
            img[y0, x0:x0 + length] += np.float32(rng.uniform(40000, 60000))
        frames.append(img)
    s = native.ResidentCalibratedStack(2, h, w)
    try:
        for k in range(2):
            s.upload_calibrated_frame(k, frames[k])
        cats = s.detect_stars([0, 1], threshold_sigma=5.0, max_stars=400, catalog_max_eccentricity=0.8)
        got = s.register_frames_triangle(0, [1], tolerance_px=2.0)[0]
    finally:
        s.close()
    first80 = cats[0][:80]
    assert np.count_nonzero(first80["eccentricity"] > 0.8) > 20  # the raw ranking is polluted
    assert got["status"] == "ok" and got["inliers"] >= 40
    np.testing.assert_allclose(got["matrix"][:2, 2], -np.asarray(shifts[1]), atol=0.1)


@pytest.mark.gpu
def test_gpu_affine_estimator_matches_reference(native, golden_affine):
    g = golden_affine
    for name in _names(g, "_names"):
        got = native.estimate_triangle_asterism_transform(g[f"{name}/ref"], g[f"{name}/mov"], transform_model="affine",
                                                          **_params(g, name))
        assert got["transform_model"] == "affine"
        _check_result(name, got, g, matrix_atol=1e-8)


@pytest.mark.gpu
def test_gpu_registration_argument_errors(native):
    with pytest.raises(ValueError):
        native.estimate_triangle_asterism_transform(np.zeros((5, 2)), np.zeros((5, 2)),
                                                    transform_model="homography")
    with pytest.raises(ValueError):
        native.estimate_triangle_asterism_transform(np.zeros((5, 2)), np.zeros((5, 2)), max_candidates=5000)
    with pytest.raises(ValueError):
        native.estimate_triangle_asterism_transform(np.zeros((5, 2)), np.zeros((5, 2)), max_stars=81)
    with pytest.raises(ValueError):
        native.triangle_asterism_descriptors_f32([0, 1, 2], [0, 1], 80, 5, 10)
    with pytest.raises(IndexError):
        native.estimate_similarity_from_triangle_descriptors_f32([0, 10, 0], [0, 0, 10], [0, 10, 0], [0, 0, 10],
                                                                 [[1.0, 1.0]], [[0, 1, 5]], [[1.0, 1.0]],
                                                                 [[0, 1, 2]])
    s = native.ResidentCalibratedStack(2, 16, 16)
    try:
        with pytest.raises(RuntimeError):
            s.register_frames_triangle(0, [1])  # no catalogs yet
        with pytest.raises(IndexError):
            s.register_frames_triangle(0, [2])
    finally:
        s.close()
