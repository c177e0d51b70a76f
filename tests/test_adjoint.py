"""Adjoint of the affine warp and gradient-based registration refinement.

CPU: the float64 PyTorch reference (tests/torch_warp_reference.py) is pinned
to the float64 oracle (oracle/adjoint.py): same forward, autograd gradient of
the parameters equal to central finite differences, autograd gradient of the
source equal to the oracle's transpose.  The float64 oracle forward is pinned
to the reference-semantics warp oracle (oracle/warp.py) within float32
rounding.

GPU (through libglass_gb300.so): forward within the Lanczos3 warp tolerance
of the float64 oracle; parameter gradient within 2e-4 of the gradient norm of
both the PyTorch reference and the float64 central differences (float32 per
pixel, float64 across blocks); source gradient within 1e-5 relative of the
oracle transpose (float32 atomics); refinement recovers a known similarity to
0.02 px RMS from a 0.5 px start with cosmic rays in the moving frame.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import adjoint as oadj
from oracle import warp as owarp

from .torch_warp_reference import warp_affine_reference


def _field(rng, h, w, stars, matrix=None, sky=1000.0, noise=5.0, fwhm=3.0):
    """Gaussian stars at reference positions mapped into this frame by inv(matrix)."""
    xs, ys, peaks = stars[:, 0], stars[:, 1], stars[:, 2]
    if matrix is not None:
        inv = np.linalg.inv(matrix)
        pts = inv @ np.vstack([xs, ys, np.ones_like(xs)])
        xs, ys = pts[0] / pts[2], pts[1] / pts[2]
    sig = fwhm / 2.3548
    img = np.full((h, w), sky, dtype=np.float64)
    yy, xx = np.mgrid[0:h, 0:w]
    for x, y, p in zip(xs, ys, peaks):
        x0, y0 = int(x), int(y)
        ya, yb, xa, xb = max(0, y0 - 12), min(h, y0 + 13), max(0, x0 - 12), min(w, x0 + 13)
        if ya >= yb or xa >= xb:
            continue
        img[ya:yb, xa:xb] += p * np.exp(-0.5 * ((xx[ya:yb, xa:xb] - x) ** 2 + (yy[ya:yb, xa:xb] - y) ** 2) / sig**2)
    img += rng.normal(0.0, noise, img.shape)
    return img.astype(np.float32)


def _stars(rng, h, w, n):
    return np.column_stack([rng.uniform(-10, w + 10, n), rng.uniform(-10, h + 10, n), rng.uniform(300, 20000, n)])


def _similarity(angle, scale, dx, dy):
    c, s = scale * np.cos(angle), scale * np.sin(angle)
    return np.array([[c, -s, dx], [s, c, dy], [0.0, 0.0, 1.0]])


def _theta(h, w):
    m = _similarity(0.004, 1.0007, 1.37, -0.62)
    inv = np.linalg.inv(m)
    return np.array([inv[0, 0], inv[0, 1], inv[0, 2], inv[1, 0], inv[1, 1], inv[1, 2]])


def _inner_grad(rng, h, w, theta, margin=6.0):
    """Random incoming gradient on output pixels whose samples stay `margin` px inside."""
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float64)
    sx = theta[0] * xs + theta[1] * ys + theta[2]
    sy = theta[3] * xs + theta[4] * ys + theta[5]
    inner = (sx > margin) & (sx < w - 1 - margin) & (sy > margin) & (sy < h - 1 - margin)
    return np.where(inner, rng.normal(0.0, 1.0, (h, w)), 0.0)


def _reference_grads(img, theta, g, interp):
    src = torch.tensor(img, dtype=torch.float64, requires_grad=True)
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    out = warp_affine_reference(src, th, interp)
    (out * torch.tensor(g)).sum().backward()
    return out.detach().numpy(), src.grad.numpy(), th.grad.numpy()


# ---- CPU: pin the float64 references ----------------------------------------------

@pytest.mark.parametrize("interp", ["bilinear", "lanczos3"])
def test_oracle_f64_forward_matches_reference_warp(interp):
    rng = np.random.default_rng(3)
    h, w = 48, 56
    img = _field(rng, h, w, _stars(rng, h, w, 12))
    theta = _theta(h, w)
    inv = np.array([[theta[0], theta[1], theta[2]], [theta[3], theta[4], theta[5]], [0, 0, 1.0]])
    exp, cov = owarp.warp_matrix(img, np.linalg.inv(inv), interp, fill=0.0)
    got = oadj.warp_affine_f64(img, theta, interp, fill=0.0)
    ok = cov > 0
    np.testing.assert_array_equal(np.isfinite(got) & (got != 0), ok & (exp != 0))
    np.testing.assert_allclose(got[ok], exp[ok], rtol=2e-6, atol=2e-6 * float(np.abs(img).max()))


@pytest.mark.parametrize("interp", ["bilinear", "lanczos3"])
def test_torch_reference_forward_matches_oracle(interp):
    rng = np.random.default_rng(4)
    h, w = 40, 44
    img = _field(rng, h, w, _stars(rng, h, w, 10)).astype(np.float64)
    if interp == "lanczos3":
        img[rng.integers(0, h, 6), rng.integers(0, w, 6)] = np.nan
    theta = _theta(h, w)
    got = warp_affine_reference(torch.tensor(img), torch.tensor(theta), interp, fill=-7.0).numpy()
    exp = oadj.warp_affine_f64(img, theta, interp, fill=-7.0)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(exp))
    fin = np.isfinite(exp)
    np.testing.assert_allclose(got[fin], exp[fin], rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("interp,rtol", [("lanczos3", 1e-6), ("bilinear", 2e-3)])
def test_torch_reference_theta_grad_matches_central_differences(interp, rtol):
    """Lanczos3 is C1 in the sample position; bilinear has kinks at integer
    positions, which the finite differences straddle for a few pixels."""
    rng = np.random.default_rng(5)
    h, w = 40, 48
    img = _field(rng, h, w, _stars(rng, h, w, 10)).astype(np.float64)
    theta = _theta(h, w)
    g = _inner_grad(rng, h, w, theta)
    _, _, gt = _reference_grads(img, theta, g, interp)
    fd = oadj.fd_theta_gradient(img, theta, g, interp, step_px=1e-4 if interp == "lanczos3" else 1e-6)
    assert np.linalg.norm(gt - fd) <= rtol * np.linalg.norm(fd), (gt, fd)


@pytest.mark.parametrize("interp", ["bilinear", "lanczos3"])
def test_torch_reference_source_grad_is_oracle_transpose(interp):
    rng = np.random.default_rng(6)
    h, w = 36, 40
    img = _field(rng, h, w, _stars(rng, h, w, 8)).astype(np.float64)
    if interp == "lanczos3":
        img[rng.integers(0, h, 5), rng.integers(0, w, 5)] = np.inf
    theta = _theta(h, w)
    g = rng.normal(0.0, 1.0, (h, w))
    out, gs, _ = _reference_grads(img, theta, np.where(np.isfinite(oadj.warp_affine_f64(img, theta, interp)), g, 0),
                                  interp)
    gz = np.where(np.isfinite(out), g, 0.0)
    exp = oadj.adjoint_source(img, theta, gz, interp)
    np.testing.assert_allclose(gs, exp, rtol=1e-12, atol=1e-12)
    # dot-product test on a finite source with the same non-finite pattern
    s = np.where(np.isfinite(img), rng.normal(0.0, 1.0, img.shape), img)
    lhs = float(np.nansum(gz * oadj.warp_affine_f64(s, theta, interp, fill=0.0)))
    rhs = float(np.sum(np.where(np.isfinite(s), exp * s, 0.0)))
    assert abs(lhs - rhs) <= 1e-10 * max(1.0, abs(lhs))


def test_matrix_theta_round_trip():
    from glass_gb300.adjoint import matrix_from_theta, registration_rms_px, theta_from_matrix

    m = _similarity(0.01, 0.999, 3.5, -2.25)
    np.testing.assert_allclose(matrix_from_theta(theta_from_matrix(m)), m, rtol=0, atol=1e-12)
    shifted = m.copy()
    shifted[0, 2] += 0.3
    assert abs(registration_rms_px([shifted], [m], 100, 100) - 0.3 / 0.999) < 1e-6
    with pytest.raises(ValueError):
        theta_from_matrix(np.array([[1, 0, 0], [0, 1, 0], [1e-3, 0, 1.0]]))


# ---- GPU ---------------------------------------------------------------------------

def _device(img):
    return torch.tensor(img, dtype=torch.float32, device="cuda")


@pytest.mark.gpu
@pytest.mark.parametrize("interp", ["bilinear", "lanczos3"])
def test_gpu_forward_matches_oracle(native, interp):
    from glass_gb300.adjoint import warp_affine

    rng = np.random.default_rng(7)
    h, w = 96, 120
    img = _field(rng, h, w, _stars(rng, h, w, 25))
    if interp == "lanczos3":
        img[rng.integers(0, h, 10), rng.integers(0, w, 10)] = np.nan
    theta = _theta(h, w)
    got = warp_affine(_device(img), torch.tensor(theta), interp, fill=float("nan")).cpu().numpy()
    exp = oadj.warp_affine_f64(img, theta, interp)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(exp))
    fin = np.isfinite(exp)
    tol = 3e-6 * float(np.nanmax(np.abs(img)))
    np.testing.assert_allclose(got[fin], exp[fin], rtol=1e-5, atol=tol)


@pytest.mark.gpu
@pytest.mark.parametrize("interp", ["bilinear", "lanczos3"])
@pytest.mark.parametrize("with_nan", [False, True])
def test_gpu_adjoint_matches_references(native, interp, with_nan):
    from glass_gb300.adjoint import warp_affine

    if with_nan and interp == "bilinear":
        pytest.skip("a non-finite bilinear tap makes the output NaN (no gradient)")
    rng = np.random.default_rng(8)
    h, w = 96, 112
    img = _field(rng, h, w, _stars(rng, h, w, 25))
    if with_nan:
        img[rng.integers(0, h, 12), rng.integers(0, w, 12)] = np.nan
    theta = _theta(h, w)
    g = _inner_grad(rng, h, w, theta)
    exp_out = oadj.warp_affine_f64(img, theta, interp)
    g = np.where(np.isfinite(exp_out), g, 0.0)
    src = _device(img).requires_grad_(True)
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    out = warp_affine(src, th, interp)
    out.backward(torch.tensor(g, dtype=torch.float32, device="cuda"))
    got_src = src.grad.cpu().numpy().astype(np.float64)
    got_theta = th.grad.numpy()

    _, ref_src, ref_theta = _reference_grads(img.astype(np.float64), theta, g, interp)
    # compare in pixel units: linear parameters scaled by the image size
    px = np.array([1.0 / w, 1.0 / w, 1.0, 1.0 / w, 1.0 / w, 1.0])
    assert np.linalg.norm((got_theta - ref_theta) * px) <= 2e-4 * np.linalg.norm(ref_theta * px), (got_theta,
                                                                                                 ref_theta)
    if interp == "lanczos3":
        fd = oadj.fd_theta_gradient(img, theta, g, interp)
        assert np.linalg.norm((got_theta - fd) * px) <= 2e-4 * np.linalg.norm(fd * px), (got_theta, fd)
    exp_src = oadj.adjoint_source(img, theta, g, interp)
    np.testing.assert_allclose(got_src, exp_src, rtol=1e-5, atol=1e-6 * float(np.abs(exp_src).max()))
    np.testing.assert_allclose(ref_src, exp_src, rtol=1e-9, atol=1e-12)


@pytest.mark.gpu
def test_gpu_adjoint_argument_errors(native):
    from glass_gb300.adjoint import warp_affine

    img = torch.zeros((16, 16), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError):
        warp_affine(img, torch.tensor([1.0, 0, 0, 0, 1, float("nan")]))
    with pytest.raises(ValueError):
        warp_affine(img, torch.zeros(5, dtype=torch.float64))
    with pytest.raises(ValueError):
        warp_affine(img.double(), torch.zeros(6, dtype=torch.float64))
    with pytest.raises(ValueError):
        warp_affine(img, torch.zeros(6, dtype=torch.float64), interpolation="nearest")


@pytest.mark.gpu
@pytest.mark.parametrize("loss", ["ncc", "ssd"])
def test_gpu_refine_recovers_known_similarity(native, loss):
    from glass_gb300.adjoint import RefineConfig, refine_affine, registration_rms_px

    rng = np.random.default_rng(9)
    h, w = 192, 224
    stars = _stars(rng, h, w, 90)
    truth = _similarity(0.003, 1.0, 4.3, -2.7)
    ref = _field(rng, h, w, stars)
    mov = _field(rng, h, w, stars, truth)
    for _ in range(25):  # cosmic-ray hits in the moving frame only
        y, x = rng.integers(2, h - 3), rng.integers(2, w - 3)
        mov[y:y + 2, x:x + int(rng.integers(1, 4))] += np.float32(rng.uniform(5000, 60000))
    start = _similarity(0.0045, 1.0, 4.3 + 0.35, -2.7 - 0.3)
    before = registration_rms_px([start], [truth], h, w)
    out = refine_affine(_device(ref), _device(mov), start, RefineConfig(model="similarity", loss=loss))
    after = registration_rms_px([out.matrix], [truth], h, w)
    assert before > 0.25
    assert after < 0.02, (before, after, out.history[-3:])
    assert out.ncc_after > out.ncc_before
    assert 0.0 < out.masked_fraction < 0.1
