"""Float64 PyTorch restatement of the affine warp, differentiated by autograd.

Test infrastructure: the reference gradient that the hand-written device
adjoint is compared with.  Same sampling rules as oracle/adjoint.py
(engine/warp.py:99-152; Lanczos3 renormalised over finite taps), written with
differentiable torch operations so that autograd yields d out / d source and
d out / d theta.  The cell indices floor(sx), floor(sy) and the validity mask
are piecewise constant and carry no gradient.
"""

from __future__ import annotations

import torch


def _lanczos3(d: torch.Tensor) -> torch.Tensor:
    return torch.where(d.abs() >= 3.0, torch.zeros_like(d), torch.sinc(d) * torch.sinc(d / 3.0))


def sample_reference(src: torch.Tensor, sx: torch.Tensor, sy: torch.Tensor, interpolation: str = "lanczos3",
                     fill: float = 0.0) -> torch.Tensor:
    """Samples `src` at float64 positions (sx, sy) (any shape)."""
    src = src.double()
    h, w = src.shape
    with torch.no_grad():
        if interpolation == "bilinear":
            valid = (sx >= 0) & (sx <= w - 1) & (sy >= 0) & (sy <= h - 1)
        else:
            valid = (sx >= 2) & (sx < w - 3) & (sy >= 2) & (sy < h - 3)
        x0 = torch.floor(torch.where(valid, sx, torch.full_like(sx, 2.0))).long()
        y0 = torch.floor(torch.where(valid, sy, torch.full_like(sy, 2.0))).long()
    tx = sx - x0.double()
    ty = sy - y0.double()
    flat = src.reshape(-1)
    if interpolation == "bilinear":
        x1 = torch.clamp(x0 + 1, max=w - 1)
        y1 = torch.clamp(y0 + 1, max=h - 1)
        out = ((1 - ty) * ((1 - tx) * flat[y0 * w + x0] + tx * flat[y0 * w + x1])
               + ty * ((1 - tx) * flat[y1 * w + x0] + tx * flat[y1 * w + x1]))
        return torch.where(valid, out, torch.full_like(out, fill))
    num = torch.zeros_like(sx)
    den = torch.zeros_like(sx)
    for j in range(6):
        wy = _lanczos3(ty - (j - 2))
        yy = torch.clamp(y0 - 2 + j, 0, h - 1)
        for i in range(6):
            wx = _lanczos3(tx - (i - 2))
            xx = torch.clamp(x0 - 2 + i, 0, w - 1)
            v = flat[yy * w + xx]
            fin = torch.isfinite(v)
            wt = wx * wy
            num = num + torch.where(fin, wt * torch.where(fin, v, torch.zeros_like(v)), torch.zeros_like(v))
            den = den + torch.where(fin, wt, torch.zeros_like(wt))
    ok = valid & (den.abs() > 1.0e-12)
    safe = torch.where(ok, den, torch.ones_like(den))
    return torch.where(ok, num / safe, torch.full_like(num, fill))


def warp_affine_reference(src: torch.Tensor, theta: torch.Tensor, interpolation: str = "lanczos3",
                          fill: float = 0.0) -> torch.Tensor:
    theta = theta.double()
    h, w = src.shape
    ys, xs = torch.meshgrid(torch.arange(h, dtype=torch.float64, device=src.device),
                            torch.arange(w, dtype=torch.float64, device=src.device), indexing="ij")
    sx = theta[0] * xs + theta[1] * ys + theta[2]
    sy = theta[3] * xs + theta[4] * ys + theta[5]
    return sample_reference(src, sx, sy, interpolation, fill)


def value_and_position_gradient(src: torch.Tensor, sx: torch.Tensor, sy: torch.Tensor,
                                interpolation: str = "lanczos3"):
    """(O, dO/dsx, dO/dsy) at every position, float64 (each output depends
    only on its own position, so the gradient of sum(O) is per position)."""
    px = sx.detach().double().clone().requires_grad_(True)
    py = sy.detach().double().clone().requires_grad_(True)
    out = sample_reference(src.detach(), px, py, interpolation)
    out.sum().backward()
    return out.detach(), px.grad, py.grad
