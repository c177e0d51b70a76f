"""Gradient registration by L-BFGS on the masked NCC of star regions
(glass_gb300.adjoint.refine_affine_lbfgs), the optimiser and loss checked on
the CPU with the float64 PyTorch restatement of the warp standing in for the
device adjoint, then on the GPU through AffineWarp (the hand-written
adjoint): from a catalog-grade start (~0.05 px) to a few thousandths of a
pixel of the true affine map."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from glass_gb300.adjoint import LbfgsConfig, refine_affine_lbfgs, registration_rms_px

from .torch_warp_reference import warp_affine_reference


def _pair(seed=3, size=192):
    rng = np.random.default_rng(seed)
    h = w = size
    n = int(30 * h * w / 128 ** 2)
    xy = np.column_stack([rng.uniform(-10, w + 10, n), rng.uniform(-10, h + 10, n)])
    peak = np.exp(rng.uniform(np.log(500), np.log(20000), n))
    sig = 2.5 / 2.3548
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)

    def render(fwd):
        pos = xy @ fwd[:2, :2].T + fwd[:2, 2]
        img = np.full((h, w), 1000.0)
        for (x, y), p in zip(pos, peak):
            img += p * np.exp(-((xx - x) ** 2 + (yy - y) ** 2) / (2 * sig ** 2))
        return (rng.poisson(img) + rng.normal(0, 5, (h, w))).astype(np.float32)

    fwd = np.eye(3)
    fwd[:2, :2] += rng.normal(0, 1e-3, (2, 2))
    fwd[:2, 2] = rng.uniform(-0.5, 0.5, 2)
    truth = np.linalg.inv(fwd)
    start = truth.copy()
    start[0, 2] += 0.04
    start[1, 2] -= 0.03
    start[0, 0] += 2e-4
    return render(np.eye(3)), render(fwd), truth, start


def test_lbfgs_refine_with_reference_warp_cpu():
    ref, mov, truth, start = _pair()
    h, w = ref.shape
    before = registration_rms_px([start], [truth], h, w)
    out = refine_affine_lbfgs(torch.from_numpy(ref), torch.from_numpy(mov), start, LbfgsConfig(iterations=20),
                              warp_fn=lambda src, th: warp_affine_reference(src, th, "lanczos3", float("nan")))
    after = registration_rms_px([out.matrix], [truth], h, w)
    assert out.evaluations <= 20
    assert out.ncc_after >= out.ncc_before
    assert before > 0.04 and after < 0.01, (before, after)


@pytest.mark.gpu
def test_lbfgs_refine_through_the_device_adjoint(native):
    ref, mov, truth, start = _pair(seed=11, size=256)
    h, w = ref.shape
    out = refine_affine_lbfgs(torch.from_numpy(ref).cuda(), torch.from_numpy(mov).cuda(), start,
                              LbfgsConfig(iterations=20))
    after = registration_rms_px([out.matrix], [truth], h, w)
    assert out.evaluations <= 20
    assert after < 0.01, after
