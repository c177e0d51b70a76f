"""Oracle: float64 affine warp, its central finite differences and its transpose.

Test infrastructure only.  The warp follows the sampling rules of
src/glass/engine/warp.py:99-152 and tests/test_gpu_warp_vs_cpu.py:66-128
(bilinear: valid for sx in [0, W-1], sy in [0, H-1], x1 = min(x0 + 1, W - 1);
Lanczos3: valid for sx in [2, W-3), sy in [2, H-3), a 6 x 6 window of taps at
x0-2..x0+3, non-finite taps skipped and the weights renormalised, weight sum
|D| <= 1e-12 invalid) evaluated entirely in float64 from the six parameters
theta of the inverse map (output -> source): sx = t0 x + t1 y + t2,
sy = t3 x + t4 y + t5.  The reference has no adjoint; the gradients here are
the float64 yardsticks the device adjoint is checked against:
  - fd_theta_gradient: central differences of L = sum(g * warp(theta));
  - adjoint_source: the transpose of the (linear in the source) warp applied
    to g, so <g, W s> = <W^T g, s>.
"""

from __future__ import annotations

import numpy as np

from oracle.warp import lanczos3_weight


def _coords(theta, height: int, width: int):
    t = np.asarray(theta, dtype=np.float64).reshape(6)
    ys, xs = np.mgrid[0:height, 0:width].astype(np.float64)
    return t[0] * xs + t[1] * ys + t[2], t[3] * xs + t[4] * ys + t[5]


def _taps(image: np.ndarray, theta, interpolation: str):
    """-> (valid mask, list of (flat source index, weight) per tap, x0, y0)."""
    h, w = image.shape
    sx, sy = _coords(theta, h, w)
    if interpolation == "bilinear":
        valid = (sx >= 0) & (sx <= w - 1) & (sy >= 0) & (sy <= h - 1)
    elif interpolation == "lanczos3":
        valid = (sx >= 2) & (sx < w - 3) & (sy >= 2) & (sy < h - 3)
    else:
        raise ValueError("interpolation must be bilinear or lanczos3")
    sxv = np.where(valid, sx, 2.0)
    syv = np.where(valid, sy, 2.0)
    x0 = np.floor(sxv).astype(np.int64)
    y0 = np.floor(syv).astype(np.int64)
    tx, ty = sxv - x0, syv - y0
    taps = []
    if interpolation == "bilinear":
        x1 = np.minimum(x0 + 1, w - 1)
        y1 = np.minimum(y0 + 1, h - 1)
        for yy, wy in ((y0, 1.0 - ty), (y1, ty)):
            for xx, wx in ((x0, 1.0 - tx), (x1, tx)):
                taps.append((yy * w + xx, wy * wx))
    else:
        for j in range(6):
            wy = lanczos3_weight(ty - (j - 2))
            yy = np.clip(y0 - 2 + j, 0, h - 1)
            for i in range(6):
                wx = lanczos3_weight(tx - (i - 2))
                xx = np.clip(x0 - 2 + i, 0, w - 1)
                taps.append((yy * w + xx, wy * wx))
    return valid, taps


def warp_affine_f64(image, theta, interpolation: str = "lanczos3", fill: float = np.nan) -> np.ndarray:
    img = np.asarray(image, dtype=np.float64)
    valid, taps = _taps(img, theta, interpolation)
    flat = img.ravel()
    if interpolation == "bilinear":
        acc = np.zeros(img.shape)
        for idx, wt in taps:
            acc += wt * flat[idx]
        ok = valid
        out = acc
    else:
        num = np.zeros(img.shape)
        den = np.zeros(img.shape)
        for idx, wt in taps:
            v = flat[idx]
            fin = np.isfinite(v)
            num += np.where(fin, wt * np.where(fin, v, 0.0), 0.0)
            den += np.where(fin, wt, 0.0)
        ok = valid & (np.abs(den) > 1.0e-12)
        out = np.divide(num, den, out=np.zeros_like(num), where=ok)
    return np.where(ok, out, fill)


def fd_theta_gradient(image, theta, grad_out, interpolation: str = "lanczos3", step_px: float = 1.0e-4):
    """Central differences of sum(grad_out * warp) over the six parameters.

    The linear parameters are stepped by step_px / max(H, W) so that every
    step moves the sample points by at most about step_px pixels."""
    img = np.asarray(image, dtype=np.float64)
    g = np.asarray(grad_out, dtype=np.float64)
    t = np.asarray(theta, dtype=np.float64).reshape(6)
    scale = float(max(img.shape))
    steps = np.array([step_px / scale, step_px / scale, step_px, step_px / scale, step_px / scale, step_px])
    out = np.zeros(6)
    for q in range(6):
        tp, tm = t.copy(), t.copy()
        tp[q] += steps[q]
        tm[q] -= steps[q]
        lp = warp_affine_f64(img, tp, interpolation, 0.0)
        lm = warp_affine_f64(img, tm, interpolation, 0.0)
        out[q] = float(np.sum(g * (lp - lm))) / (2.0 * steps[q])
    return out


def adjoint_source(image, theta, grad_out, interpolation: str = "lanczos3") -> np.ndarray:
    """W^T g for the warp at the given source (its non-finite pattern fixes W)."""
    img = np.asarray(image, dtype=np.float64)
    g = np.asarray(grad_out, dtype=np.float64)
    valid, taps = _taps(img, theta, interpolation)
    flat = img.ravel()
    out = np.zeros(img.size)
    if interpolation == "bilinear":
        ok = valid.copy()
        for idx, _ in taps:
            ok &= np.isfinite(flat[idx])  # a non-finite tap makes the output NaN
        for idx, wt in taps:
            np.add.at(out, idx[ok], (g * wt)[ok])
    else:
        den = np.zeros(img.shape)
        for idx, wt in taps:
            den += np.where(np.isfinite(flat[idx]), wt, 0.0)
        ok = valid & (np.abs(den) > 1.0e-12)
        scale = np.divide(g, den, out=np.zeros_like(g), where=ok)
        for idx, wt in taps:
            sel = ok & np.isfinite(flat[idx])
            np.add.at(out, idx[sel], (scale * wt)[sel])
    return out.reshape(img.shape)
