"""Gauss-Newton registration refinement on resident frames.

CPU: a float64 restatement of the accumulation (per-sample Jacobian from the
PyTorch reference sampler's autograd position gradient) and of the solve
(model projection, centred parameters) converges to the known transform of a
synthetic pair, which pins the algorithm the device kernels implement.

GPU (libglass_gb300.so): the normal-equation sums of one accumulation pass
match the float64 restatement (every entry within 2e-5 of its Cauchy-Schwarz
scale sqrt(H_ii H_jj), resp. sqrt(H_ii sum r^2); counts exact); the full
refinement recovers known similarity / affine transforms to 0.005 px RMS from
starts 0.3-0.6 px off with cosmic rays in the moving frame and a photometric
change, and a batch gives the same answers as single calls.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from .test_adjoint import _field, _similarity, _stars
from .torch_warp_reference import value_and_position_gradient

def _theta_of(matrix):
    inv = np.linalg.inv(np.asarray(matrix, dtype=np.float64))
    return inv[:2].reshape(-1)


def _matrix_of(theta):
    inv = np.vstack([np.asarray(theta, dtype=np.float64).reshape(2, 3), [0.0, 0.0, 1.0]])
    m = np.linalg.inv(inv)
    m[2] = (0.0, 0.0, 1.0)
    return m


def gn_sums_reference(ref, mov, theta, alpha, beta, stride, interp="lanczos3", row_stride=None):
    """float64 J^T J (upper, 36), J^T r (8), sum r^2, count over all valid
    samples of the grid (every row_stride-th row, default stride, and every
    stride-th column)."""
    h, w = ref.shape
    ys, xs = np.mgrid[0:h:row_stride or stride, 0:w:stride].astype(np.float64)
    sx = theta[0] * xs + theta[1] * ys + theta[2]
    sy = theta[3] * xs + theta[4] * ys + theta[5]
    o, ox, oy = (t.numpy() for t in value_and_position_gradient(torch.tensor(mov, dtype=torch.float64),
                                                                torch.tensor(sx), torch.tensor(sy), interp))
    if interp == "bilinear":
        valid = (sx >= 0) & (sx <= w - 1) & (sy >= 0) & (sy <= h - 1)
    else:
        valid = (sx >= 2) & (sx < w - 3) & (sy >= 2) & (sy < h - 3)
    a = ref[ys.astype(int), xs.astype(int)].astype(np.float64)
    valid &= np.isfinite(a) & np.isfinite(o)
    r = o - alpha * a - beta
    cx, cy, ir = (w - 1) / 2.0, (h - 1) / 2.0, 2.0 / max(w, h)
    xt, yt = (xs - cx) * ir, (ys - cy) * ir
    J = np.stack([ox * xt, ox * yt, ox, oy * xt, oy * yt, oy, -a, -np.ones_like(a)], axis=-1)[valid]
    rv = r[valid]
    H = J.T @ J
    out = np.zeros(48)
    out[:36] = H[np.triu_indices(8)]
    out[36:44] = J.T @ rv
    out[44] = rv @ rv
    out[45] = rv.size
    return out


def _projection(model):
    P = np.zeros((8, 8))
    if model == "affine":
        return np.eye(8)
    cols = [np.eye(8)[2], np.eye(8)[5]]
    if model == "similarity":
        cols += [np.eye(8)[0] + np.eye(8)[4], -np.eye(8)[1] + np.eye(8)[3]]
    cols += [np.eye(8)[6], np.eye(8)[7]]
    P = np.stack(cols, axis=1)
    return P


def gn_step_reference(sums, theta, alpha, beta, model, h, w):
    """One float64 Gauss-Newton update from the sums (the solve kernel's math)."""
    H = np.zeros((8, 8))
    H[np.triu_indices(8)] = sums[:36]
    H = H + np.triu(H, 1).T
    g = sums[36:44]
    P = _projection(model)
    A = P.T @ H @ P
    d = np.linalg.solve(A, -P.T @ g)
    dt = P @ d
    cx, cy, ir = (w - 1) / 2.0, (h - 1) / 2.0, 2.0 / max(w, h)
    t = np.array(theta, dtype=np.float64)
    t[0] += dt[0] * ir
    t[1] += dt[1] * ir
    t[2] += dt[2] - (dt[0] * cx + dt[1] * cy) * ir
    t[3] += dt[3] * ir
    t[4] += dt[4] * ir
    t[5] += dt[5] - (dt[3] * cx + dt[4] * cy) * ir
    return t, alpha + dt[6], beta + dt[7]


def gn_masked_sums_reference(ref, mov, theta, alpha, beta, sigma, stride, clip=5.0, shift=1.0):
    """The device accumulation with its mask, float64: (sums, robust sigma).
    The robust sigma is 1.4826 * median |r| over the valid samples (the
    device reads the median from a log histogram, within a few per cent)."""
    h, w = ref.shape
    ys, xs = np.mgrid[0:h:stride, 0:w:stride].astype(np.float64)
    sx = theta[0] * xs + theta[1] * ys + theta[2]
    sy = theta[3] * xs + theta[4] * ys + theta[5]
    o, ox, oy = (t.numpy() for t in value_and_position_gradient(torch.tensor(mov, dtype=torch.float64),
                                                                torch.tensor(sx), torch.tensor(sy)))
    valid = (sx >= 2) & (sx < w - 3) & (sy >= 2) & (sy < h - 3)
    yi, xi = ys.astype(int), xs.astype(int)
    a = ref[yi, xi].astype(np.float64)
    r = o - alpha * a - beta
    valid &= np.isfinite(r)
    rp = np.pad(ref.astype(np.float64), 1, mode="edge")
    ga = 0.5 * np.maximum(np.abs(rp[yi + 1, xi + 2] - rp[yi + 1, xi]), np.abs(rp[yi + 2, xi + 1] - rp[yi, xi + 1]))
    ga[(xi == 0) | (xi == w - 1) | (yi == 0) | (yi == h - 1)] = 0.0
    gb = np.maximum(np.abs(ox), np.abs(oy))
    allow = clip * sigma + shift * np.minimum(abs(alpha) * ga, gb)
    keep = valid & (np.abs(r) <= allow) & (gb <= 2.0 * abs(alpha) * ga + 3.0 * sigma)
    robust = 1.4826 * float(np.median(np.abs(r[valid])))
    cx, cy, ir = (w - 1) / 2.0, (h - 1) / 2.0, 2.0 / max(w, h)
    xt, yt = (xs - cx) * ir, (ys - cy) * ir
    J = np.stack([ox * xt, ox * yt, ox, oy * xt, oy * yt, oy, -a, -np.ones_like(a)], axis=-1)[keep]
    rv = r[keep]
    out = np.zeros(48)
    out[:36] = (J.T @ J)[np.triu_indices(8)]
    out[36:44] = J.T @ rv
    out[44] = rv @ rv
    out[45] = rv.size
    return out, robust


def gn_refine_reference(ref, mov, matrix, model="similarity", stride=2, stats_passes=3, iterations=8):
    """The device refinement's sequence in float64: statistics passes on a
    grid twice as coarse (beta from the kept mean, robust sigma), then
    Gauss-Newton steps."""
    h, w = ref.shape
    theta, alpha, beta, sigma = _theta_of(matrix), 1.0, 0.0, np.inf
    for _ in range(stats_passes):
        sums, robust = gn_masked_sums_reference(ref, mov, theta, alpha, beta, sigma, 2 * stride)
        beta += -sums[43] / sums[45]
        sigma = robust
    for _ in range(iterations):
        sums, robust = gn_masked_sums_reference(ref, mov, theta, alpha, beta, sigma, stride)
        theta, alpha, beta = gn_step_reference(sums, theta, alpha, beta, model, h, w)
        sigma = robust
    return _matrix_of(theta), alpha, beta, sigma


def _rms(est, truth, h, w):
    from glass_gb300.adjoint import registration_rms_px

    return registration_rms_px([est], [truth], h, w)


def _pair(seed, h, w, truth, gain=1.0, offset=0.0, cosmic=0):
    rng = np.random.default_rng(seed)
    stars = _stars(rng, h, w, int(h * w / 500))
    ref = _field(rng, h, w, stars)
    mov = (_field(rng, h, w, stars, truth) * np.float32(gain) + np.float32(offset)).astype(np.float32)
    for _ in range(cosmic):
        y, x = rng.integers(2, h - 3), rng.integers(2, w - 3)
        mov[y:y + 2, x:x + int(rng.integers(1, 4))] += np.float32(rng.uniform(5000, 60000))
    return ref, mov


# ---- CPU ---------------------------------------------------------------------------

@pytest.mark.parametrize("model", ["similarity", "affine"])
def test_reference_gauss_newton_converges(model):
    h, w = 96, 112
    truth = _similarity(0.004, 1.0005, 3.2, -1.9)
    ref, mov = _pair(1, h, w, truth, gain=0.9, offset=40.0)
    start = _similarity(0.0055, 1.0, 3.2 + 0.4, -1.9 - 0.25)
    theta, alpha, beta = _theta_of(start), 1.0, 0.0
    for _ in range(6):
        sums = gn_sums_reference(ref, mov, theta, alpha, beta, 1)
        theta, alpha, beta = gn_step_reference(sums, theta, alpha, beta, model, h, w)
    assert _rms(start, truth, h, w) > 0.3
    assert _rms(_matrix_of(theta), truth, h, w) < 0.02
    assert abs(alpha - 0.9) < 0.01


def test_reference_masked_refine_rejects_cosmic_rays():
    """With cosmic rays in the moving frame the masked sequence still lands
    within 0.005 px (without the gradient-consistency test the rays' Lanczos
    ringing biases it by about 0.025 px on this pair)."""
    h, w = 256, 288
    truth = _similarity(0.004, 1.0, 5.3, -2.2)
    start = _similarity(0.0052, 1.0, 5.3 + 0.45, -2.2 - 0.35)
    ref, mov = _pair(4, h, w, truth, gain=0.85, offset=60.0, cosmic=40)
    m, alpha, _, sigma = gn_refine_reference(ref, mov, start, iterations=5)
    assert _rms(m, truth, h, w) < 0.005
    assert abs(alpha - 0.85) < 0.005
    assert 5.0 < sigma < 9.0  # noise of the difference of two frames (5 ADU each, scaled)


# ---- GPU ---------------------------------------------------------------------------

def _stack(native, frames):
    n, (h, w) = len(frames), frames[0].shape
    s = native.ResidentCalibratedStack(n, h, w)
    for k, f in enumerate(frames):
        s.upload_calibrated_frame(k, f)
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("interp", ["bilinear", "lanczos3"])
def test_gpu_normal_equations_scaled(native, interp):
    h, w = 120, 136
    ref, mov = _pair(2, h, w, _similarity(0.003, 1.0, 2.6, -3.1), gain=1.1, offset=-30.0)
    _, mov2 = _pair(3, h, w, _similarity(-0.002, 1.0, -1.4, 0.8))
    thetas = [_theta_of(_similarity(0.0035, 1.0, 2.9, -3.3)), _theta_of(_similarity(-0.002, 1.0, -1.2, 0.7))]
    phot = [(1.05, -20.0, np.inf), (1.0, 5.0, np.inf)]
    s = _stack(native, [ref, mov, mov2])
    try:
        got = s.gradient_normal_equations(0, [1, 2], thetas, phot, interpolation=interp, sample_stride=2)
    finally:
        s.close()
    for k, m in enumerate((mov, mov2)):
        exp = gn_sums_reference(ref, m, thetas[k], phot[k][0], phot[k][1], 2, interp)
        assert got[k, 45] == exp[45]
        H = np.zeros((8, 8))
        H[np.triu_indices(8)] = exp[:36]
        d = np.sqrt(np.diag(H + np.triu(H, 1).T))
        scale_h = np.outer(d, d)[np.triu_indices(8)]
        assert np.all(np.abs(got[k, :36] - exp[:36]) <= 2e-5 * scale_h), k
        scale_g = d * np.sqrt(exp[44])
        assert np.all(np.abs(got[k, 36:44] - exp[36:44]) <= 2e-5 * scale_g), k
        assert abs(got[k, 44] - exp[44]) <= 2e-5 * exp[44]
        np.testing.assert_array_equal(got[k, 46:], 0.0)


@pytest.mark.gpu
def test_gpu_normal_equations_whole_rows(native):
    """The whole-row grid (every column of every 5th row) sums the same
    samples as the restatement on that grid."""
    h, w = 120, 136
    ref, mov = _pair(2, h, w, _similarity(0.003, 1.0, 2.6, -3.1), gain=1.1, offset=-30.0)
    theta = _theta_of(_similarity(0.0035, 1.0, 2.9, -3.3))
    s = _stack(native, [ref, mov])
    try:
        got = s.gradient_normal_equations(0, [1], [theta], [(1.05, -20.0, np.inf)], sample_stride=1, row_stride=5)[0]
    finally:
        s.close()
    exp = gn_sums_reference(ref, mov, theta, 1.05, -20.0, 1, row_stride=5)
    assert got[45] == exp[45]
    H = np.zeros((8, 8))
    H[np.triu_indices(8)] = exp[:36]
    d = np.sqrt(np.diag(H + np.triu(H, 1).T))
    assert np.all(np.abs(got[:36] - exp[:36]) <= 2e-5 * np.outer(d, d)[np.triu_indices(8)])
    assert np.all(np.abs(got[36:44] - exp[36:44]) <= 2e-5 * d * np.sqrt(exp[44]))


@pytest.mark.gpu
@pytest.mark.parametrize("model", ["similarity", "affine"])
def test_gpu_gradient_refine_recovers_truth(native, model):
    h, w = 256, 288
    truths = [_similarity(0.004, 1.0, 5.3, -2.2), _similarity(-0.003, 1.0004, -3.7, 4.1)]
    starts = [_similarity(0.0052, 1.0, 5.3 + 0.45, -2.2 - 0.35), _similarity(-0.0045, 1.0, -3.7 - 0.3, 4.1 + 0.5)]
    ref, mov1 = _pair(4, h, w, truths[0], gain=0.85, offset=60.0, cosmic=40)
    _, mov2 = _pair(4, h, w, truths[1], cosmic=40)
    s = _stack(native, [ref, mov1, mov2])
    try:
        res = s.refine_matrix_gradient_batch_to_reference(0, [1, 2], np.stack(starts), model=model)
        single = s.refine_matrix_gradient_batch_to_reference(0, [2], starts[1][None], model=model)
    finally:
        s.close()
    for k in range(2):
        before, after = _rms(starts[k], truths[k], h, w), _rms(res[k]["matrix"], truths[k], h, w)
        assert before > 0.3
        assert res[k]["ok"], res[k]
        assert after < 0.005, (k, before, after, res[k])
    assert abs(res[0]["alpha"] - 0.85) < 0.02
    np.testing.assert_allclose(single[0]["matrix"], res[1]["matrix"], rtol=0, atol=1e-6)


@pytest.mark.gpu
def test_gpu_gradient_refine_whole_rows_recovers_truth(native):
    """Whole rows (every column of every 4th row; the statistics passes on
    every 8th row) land as close as the square grid."""
    h, w = 256, 288
    truth = _similarity(0.004, 1.0, 5.3, -2.2)
    start = _similarity(0.0052, 1.0, 5.3 + 0.45, -2.2 - 0.35)
    ref, mov = _pair(4, h, w, truth, gain=0.85, offset=60.0, cosmic=40)
    s = _stack(native, [ref, mov])
    try:
        res = s.refine_matrix_gradient_batch_to_reference(0, [1], start[None], sample_stride=1, row_stride=4)[0]
    finally:
        s.close()
    assert res["ok"], res
    assert _rms(res["matrix"], truth, h, w) < 0.005, res
    assert res["samples"] <= (h // 4) * w
    assert abs(res["alpha"] - 0.85) < 0.02


@pytest.mark.gpu
@pytest.mark.parametrize("gain,offset", [(0.5, 900.0), (2.0, -700.0)])
def test_gpu_gradient_refine_large_photometric_ratio(native, gain, offset):
    """A thin-cloud frame against a clear reference (and the reverse): the
    photometric start (value-distribution quantiles) puts alpha near the
    gain before the masked passes, so star pixels are not clipped away."""
    h, w = 256, 288
    truth = _similarity(0.003, 1.0, 3.2, -1.7)
    start = _similarity(0.0038, 1.0, 3.2 + 0.4, -1.7 - 0.3)
    ref, mov = _pair(9, h, w, truth, gain=gain, offset=offset, cosmic=40)
    s = _stack(native, [ref, mov])
    try:
        res = s.refine_matrix_gradient_batch_to_reference(0, [1], start[None])
    finally:
        s.close()
    assert res[0]["ok"], res[0]
    # 0.5 px start -> under 0.01 px (unscaled cosmic rays weigh more against
    # the scaled stars than at gain 1)
    assert _rms(res[0]["matrix"], truth, h, w) < 0.01, res[0]
    assert abs(res[0]["alpha"] - gain) < 0.02 * gain


@pytest.mark.gpu
def test_gpu_gradient_refine_arguments(native):
    h, w = 64, 64
    s = _stack(native, [np.zeros((h, w), np.float32), np.zeros((h, w), np.float32)])
    try:
        eye = np.eye(3)[None]
        with pytest.raises(ValueError):
            s.refine_matrix_gradient_batch_to_reference(0, [1], eye, model="projective")
        with pytest.raises(ValueError):
            s.refine_matrix_gradient_batch_to_reference(0, [1], eye, sample_stride=0)
        with pytest.raises(ValueError):
            s.refine_matrix_gradient_batch_to_reference(0, [1], eye, row_stride=-1)
        with pytest.raises(ValueError):
            s.refine_matrix_gradient_batch_to_reference(0, [1], eye, row_stride=5000)
        with pytest.raises(ValueError):
            s.refine_matrix_gradient_batch_to_reference(0, [1], np.array([[[1, 0, 0], [0, 1, 0], [1e-3, 0, 1.0]]]))
        with pytest.raises(IndexError):
            s.refine_matrix_gradient_batch_to_reference(0, [5], eye)
        # a blank frame pair has no gradient information: the system is singular
        res = s.refine_matrix_gradient_batch_to_reference(0, [1], eye)
        assert not res[0]["ok"]
        np.testing.assert_array_equal(res[0]["matrix"], np.eye(3))
    finally:
        s.close()


def test_gradient_sample_grid_targets_sample_count():
    from glass_gb300.pipeline import DEFAULT_GRADIENT_REFINE, gradient_sample_grid

    p = dict(DEFAULT_GRADIENT_REFINE)
    assert gradient_sample_grid(p, 2048, 2048) == (3, 3)  # 466k samples: the square grid holds
    cols, rows = gradient_sample_grid(p, 6422, 9600)  # 9600 x 6422 frame: whole rows
    assert (cols, rows) == (1, 62)
    assert 0.9e6 < -(-6422 // rows) * 9600 <= 1.0e6
    assert gradient_sample_grid(dict(p, target_samples=None), 6422, 9600) == (3, 3)
    assert gradient_sample_grid(dict(p, sample_stride=5), 512, 512) == (5, 5)
    assert gradient_sample_grid(dict(p, target_samples=1), 6422, 9600) == (1, 4096)
