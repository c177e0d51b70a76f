"""Star detection: the oracle is pinned to the reference's detect_stars
(golden vectors from src/glass/cpu/star_detect.py), and the GPU detector must
return the same star list.

GPU bar: same stars in the same order (count and ordering exact); positions,
flux and the derived moments within 1e-9 relative - both sides sum float64
moments, only the summation order differs.
"""

from __future__ import annotations

import ast

import numpy as np
import pytest

from oracle import stars as ostars

from .conftest import GOLDEN

FIELDS = ("x", "y", "flux", "peak", "fwhm_px", "eccentricity", "snr", "sharpness", "npix")


@pytest.fixture(scope="module")
def golden_stars():
    return np.load(GOLDEN / "stars.npz", allow_pickle=False)


def _params(g, name):
    return ast.literal_eval(str(g[f"{name}/params"]))


def test_oracle_matches_reference_detect_stars(golden_stars):
    g = golden_stars
    names = [str(n) for n in g["_names"]]
    assert len(names) >= 10
    for name in names:
        found = ostars.detect_stars(g[f"{name}/image"], **_params(g, name))
        assert len(found) == len(g[f"{name}/x"]), name
        for fi, field in enumerate(FIELDS):
            got = np.asarray([np.nan if s[fi] is None else s[fi] for s in found], dtype=np.float64)
            np.testing.assert_array_equal(got, g[f"{name}/{field}"], err_msg=f"{name} {field}")


@pytest.mark.gpu
def test_gpu_detect_stars_matches_reference(native, golden_stars):
    g = golden_stars
    gpu_fields = ("x", "y", "flux", "peak", "fwhm", "eccentricity", "snr", "sharpness", "npix")
    for name in [str(n) for n in g["_names"]]:
        params = _params(g, name)
        got = native.detect_stars_f32(g[f"{name}/image"], **params)
        assert got.size == len(g[f"{name}/x"]), f"{name}: {got.size} stars vs {len(g[name + '/x'])}"
        for gf, rf in zip(gpu_fields, FIELDS):
            exp = g[f"{name}/{rf}"]
            np.testing.assert_allclose(got[gf].astype(np.float64), exp, rtol=1e-9, atol=1e-12,
                                       err_msg=f"{name} {rf}")


@pytest.mark.gpu
def test_gpu_detect_stars_batch_and_info(native):
    rng = np.random.default_rng(8)
    n, h, w = 3, 72, 96
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    frames = []
    for k in range(n):
        img = np.full((h, w), 900.0)
        for _ in range(15):
            x0, y0 = rng.uniform(4, w - 5), rng.uniform(4, h - 5)
            img += rng.uniform(500, 9000) * np.exp(-((xx - x0) ** 2 + (yy - y0) ** 2) / (2 * 1.2 ** 2))
        frames.append((img + 12.0 * rng.standard_normal((h, w))).astype(np.float32))
    s = native.ResidentCalibratedStack(n, h, w)
    for k in range(n):
        s.upload_calibrated_frame(k, frames[k])
    cats, info = s.detect_stars([2, 0, 1], threshold_sigma=5.0, max_stars=12, with_info=True)
    for pos, k in enumerate([2, 0, 1]):
        exp = ostars.detect_stars(frames[k], threshold_sigma=5.0, max_stars=12)
        med, _rms, mad, noise = ostars.robust_background(frames[k])
        assert info[pos]["median"] == np.float32(med)
        assert info[pos]["mad"] == np.float32(mad)
        assert cats[pos].size == len(exp)
        np.testing.assert_allclose(cats[pos]["x"], [e[0] for e in exp], rtol=1e-9)
        np.testing.assert_allclose(cats[pos]["flux"], [e[2] for e in exp], rtol=1e-9)
    s.close()


@pytest.mark.gpu
def test_gpu_median_mad_exact_on_large_and_adversarial_frames(native):
    """Frames larger than the sample the order statistics start from: a sky
    frame (the sample's band settles both statistics in one pass), a frame
    whose sampled pixels differ from all the others, and
    a frame of heavy ties with NaNs (both fall back to the three-pass radix
    select).  Median and MAD must equal the oracle's exactly."""
    rng = np.random.default_rng(31)
    h, w = 256, 384
    sky = (1000.0 + 31.0 * rng.standard_normal((h, w))).astype(np.float32)
    sky[rng.random((h, w)) < 1e-3] = 40000.0
    # the sampled pixels (32768 evenly spaced positions) hold small values,
    # every other pixel 1000: the sample's band misses the true middle ranks
    n_pix, n_sample = h * w, 32768
    sampled = ((2 * np.arange(n_sample, dtype=np.int64) + 1) * n_pix) // (2 * n_sample)
    alternating = np.full(n_pix, 1000.0, dtype=np.float32)
    alternating[sampled] = rng.normal(0.0, 1.0, n_sample).astype(np.float32)
    alternating = alternating.reshape(h, w)
    ties = rng.integers(0, 4, (h, w)).astype(np.float32) * 10.0
    ties[rng.random((h, w)) < 0.1] = np.nan
    frames = [sky, alternating, ties]
    s = native.ResidentCalibratedStack(len(frames), h, w)
    try:
        for k, f in enumerate(frames):
            s.upload_calibrated_frame(k, f)
        _cats, info = s.detect_stars([0, 1, 2], threshold_sigma=5.0, max_stars=20, with_info=True)
        for k, f in enumerate(frames):
            med, _rms, mad, _noise = ostars.robust_background(f)
            assert info[k]["median"] == np.float32(med), k
            assert info[k]["mad"] == np.float32(mad), k
            assert info[k]["valid_pixels"] == int(np.isfinite(f).sum())
    finally:
        s.close()


# ---- background mesh (this project's extension; the oracle is the spec) ----------

def _gradient_field(seed, h=192, w=256, n=40):
    """Stars on a sky with a steep gradient (300 -> 2300 ADU across the frame)."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img = 300.0 + 2000.0 * xx / (w - 1) + 150.0 * np.sin(yy / 40.0)
    pos = []
    for _ in range(n):
        x0, y0 = rng.uniform(6, w - 7), rng.uniform(6, h - 7)
        img += rng.uniform(150, 4000) * np.exp(-((xx - x0) ** 2 + (yy - y0) ** 2) / (2 * 1.3 ** 2))
        pos.append((x0, y0))
    img += 8.0 * rng.standard_normal((h, w))
    return img.astype(np.float32), np.asarray(pos)


def test_oracle_mesh_background_tracks_gradient():
    img, pos = _gradient_field(1)
    bg, nz = ostars.background_mesh(img, 32)
    assert bg.shape == (6, 8)
    # cell medians follow the sky (the gradient inside a 32-px cell, 250 ADU,
    # sets its MAD: the noise estimate is local but not gradient-free)
    assert np.all(np.diff(bg, axis=1) > 100.0)
    assert np.all(nz < 130.0)
    glob = ostars.detect_stars(img, threshold_sigma=5.0, max_stars=500)
    mesh = ostars.detect_stars(img, threshold_sigma=5.0, max_stars=500, mesh_cell=32)

    def matched(cat):
        got = np.asarray([(s[0], s[1]) for s in cat]).reshape(-1, 2)
        if got.size == 0:
            return 0
        d = np.sqrt(((pos[:, None, :] - got[None]) ** 2).sum(-1)).min(axis=1)
        return int(np.count_nonzero(d < 1.0))

    # the global threshold (median + 5 MAD-sigma of the whole gradient) sits
    # above most stars; the mesh finds every one of them
    assert matched(mesh) == len(pos) and matched(glob) < len(pos) // 2
    # every mesh detection is a real star (no sky-gradient peaks)
    got = np.asarray([(s[0], s[1]) for s in mesh])
    d = np.sqrt(((got[:, None, :] - pos[None]) ** 2).sum(-1)).min(axis=1)
    assert np.all(d < 2.0)


def test_oracle_mesh_value_interpolates_between_centres():
    mesh = np.array([[0.0, 10.0], [20.0, 30.0]])
    # centres at (cell - 1) / 2 = 7.5 and 23.5 for cell 16; clamped outside
    assert ostars.mesh_value(mesh, 16, 0, 0) == 0.0
    assert ostars.mesh_value(mesh, 16, 31, 31) == 30.0
    assert abs(ostars.mesh_value(mesh, 16, 15.5, 7.5) - 5.0) < 1e-12
    assert abs(ostars.mesh_value(mesh, 16, 15.5, 15.5) - 15.0) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("cell", [16, 32, 64])
def test_gpu_mesh_detection_matches_oracle(native, cell):
    frames = [_gradient_field(s)[0] for s in (2, 3)]
    frames[1][10:40, 200:230] = np.nan  # a masked patch: one cell partly, others fully
    h, w = frames[0].shape
    s = native.ResidentCalibratedStack(2, h, w)
    try:
        for k in range(2):
            s.upload_calibrated_frame(k, frames[k])
        cats = s.detect_stars([0, 1], threshold_sigma=5.0, max_stars=300, mesh_cell=cell)
    finally:
        s.close()
    gpu_fields = ("x", "y", "flux", "peak", "fwhm", "eccentricity", "snr", "sharpness", "npix")
    for k in range(2):
        exp = ostars.detect_stars(frames[k], threshold_sigma=5.0, max_stars=300, mesh_cell=cell)
        assert cats[k].size == len(exp), (k, cats[k].size, len(exp))
        for j, gf in enumerate(gpu_fields):
            e = np.asarray([np.nan if s_[j] is None else s_[j] for s_ in exp], dtype=np.float64)
            np.testing.assert_allclose(cats[k][gf].astype(np.float64), e, rtol=1e-9, atol=1e-12,
                                       err_msg=f"frame {k} {gf}")


@pytest.mark.gpu
def test_gpu_mesh_detection_arguments(native):
    img = _gradient_field(4)[0]
    s = native.ResidentCalibratedStack(1, *img.shape)
    try:
        s.upload_calibrated_frame(0, img)
        with pytest.raises(ValueError):
            s.detect_stars([0], mesh_cell=4)
        with pytest.raises(ValueError):
            s.detect_stars([0], mesh_cell=128)
        with pytest.raises(ValueError):
            s.detect_stars([0], mesh_cell=32, background=300.0)
    finally:
        s.close()
