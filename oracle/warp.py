"""Oracle: matrix warps (nearest / bilinear / Lanczos3) of one frame.

Restates, vectorised over pixels but with the per-pixel arithmetic and
summation order of the reference:
  - src/glass/engine/warp.py:155-227 (_warp_tile_matrix: float64 source
    coordinates from the float64 inverse, validity ranges, fill/coverage)
  - src/glass/engine/warp.py:87-119 (nearest / bilinear sampling, float32)
  - tests/test_gpu_warp_vs_cpu.py:66-128 (Lanczos3 with non-finite taps
    skipped, renormalisation, optional overshoot clamp; float64 weights with
    sinc(v) = 1 for |v| < 1e-6) - the behaviour the reference CUDA kernels
    (warp_kernels.cu:388-777) implement and are tested against.
  - src/glass/cpu/warp.py:6-22 (integer translation).
"""

from __future__ import annotations

import numpy as np

_F32 = np.float32


def _sinc(v: np.ndarray) -> np.ndarray:
    out = np.ones_like(v)
    big = np.abs(v) >= 1.0e-6
    pix = np.pi * v[big]
    out[big] = np.sin(pix) / pix
    return out


def lanczos3_weight(d: np.ndarray) -> np.ndarray:
    d = np.asarray(d, dtype=np.float64)
    w = _sinc(d) * _sinc(d / 3.0)
    return np.where(np.abs(d) >= 3.0, 0.0, w)


def source_coordinates(matrix, height: int, width: int):
    """float64 source coordinates of every output pixel (engine/warp.py:168-191).

    The matrix is used as given, promoted to float64: the reference's matrix
    entry points pass float32 matrices, its translation helpers float64 shifts.
    """
    transform = np.asarray(matrix, dtype=np.float64)
    inverse = np.linalg.inv(transform)
    ys, xs = np.mgrid[0:height, 0:width].astype(np.float64)
    denom = inverse[2, 0] * xs + inverse[2, 1] * ys + inverse[2, 2]
    ok = np.abs(denom) > 1.0e-12
    sx = np.divide(inverse[0, 0] * xs + inverse[0, 1] * ys + inverse[0, 2], denom, out=np.full_like(xs, np.nan),
                   where=ok)
    sy = np.divide(inverse[1, 0] * xs + inverse[1, 1] * ys + inverse[1, 2], denom, out=np.full_like(ys, np.nan),
                   where=ok)
    return sx, sy


def warp_matrix(data, matrix, interpolation: str = "bilinear", fill: float = 0.0, clamping_threshold: float = -1.0):
    """-> (warped float32, coverage float32)."""
    image = np.asarray(data, dtype=_F32)
    h, w = image.shape
    out = np.full((h, w), fill, dtype=_F32)
    cov = np.zeros((h, w), dtype=_F32)
    sx, sy = source_coordinates(matrix, h, w)
    valid = np.isfinite(sx) & np.isfinite(sy)
    if interpolation in ("nearest", "bilinear"):
        valid &= (sx >= 0.0) & (sx <= w - 1) & (sy >= 0.0) & (sy <= h - 1)
    elif interpolation == "lanczos3":
        valid &= (sx >= 2.0) & (sx < w - 3) & (sy >= 2.0) & (sy < h - 3)
    else:
        raise ValueError(f"unsupported warp interpolation: {interpolation}")
    vx = sx[valid]
    vy = sy[valid]
    if vx.size == 0:
        return out, cov
    if interpolation == "nearest":
        sampled = image[np.rint(vy).astype(np.int64), np.rint(vx).astype(np.int64)].astype(_F32)
        ok = np.ones(vx.shape, dtype=bool)
    elif interpolation == "bilinear":
        x0 = np.floor(vx).astype(np.int64)
        y0 = np.floor(vy).astype(np.int64)
        x1 = np.minimum(x0 + 1, w - 1)
        y1 = np.minimum(y0 + 1, h - 1)
        tx = (vx - x0).astype(_F32)
        ty = (vy - y0).astype(_F32)
        top = image[y0, x0] * (_F32(1.0) - tx) + image[y0, x1] * tx
        bottom = image[y1, x0] * (_F32(1.0) - tx) + image[y1, x1] * tx
        sampled = (top * (_F32(1.0) - ty) + bottom * ty).astype(_F32)
        ok = np.ones(vx.shape, dtype=bool)
    else:
        x0 = np.floor(vx).astype(np.int64)
        y0 = np.floor(vy).astype(np.int64)
        wsum = np.zeros(vx.shape)
        acc = np.zeros(vx.shape)
        vmin = np.full(vx.shape, np.inf)
        vmax = np.full(vx.shape, -np.inf)
        for j in range(-2, 4):
            yy = y0 + j
            wy = lanczos3_weight(vy - yy)
            for i in range(-2, 4):
                xx = x0 + i
                v = image[yy, xx].astype(np.float64)
                fin = np.isfinite(v)
                wgt = wy * lanczos3_weight(vx - xx)
                acc = np.where(fin, acc + np.where(fin, v, 0.0) * wgt, acc)
                wsum = np.where(fin, wsum + wgt, wsum)
                vmin = np.where(fin, np.minimum(vmin, v), vmin)
                vmax = np.where(fin, np.maximum(vmax, v), vmax)
        ok = np.abs(wsum) > 1.0e-12
        value = np.divide(acc, wsum, out=np.zeros_like(acc), where=ok)
        if clamping_threshold >= 0.0:
            rng = vmax - vmin
            has = vmin <= vmax
            clamped = np.minimum(vmax + clamping_threshold * rng, np.maximum(vmin - clamping_threshold * rng, value))
            value = np.where(has, clamped, value)
        sampled = value.astype(_F32)
    rows, cols = np.nonzero(valid)
    out[rows[ok], cols[ok]] = sampled[ok]
    cov[rows[ok], cols[ok]] = 1.0
    return out, cov


def warp_translation(data, dx: float, dy: float, fill: float = 0.0):
    """cpu/warp.py:6-22 + coverage (glass_cuda.py:539-562)."""
    image = np.asarray(data, dtype=_F32)
    h, w = image.shape
    out = np.full_like(image, fill)
    cov = np.zeros_like(image)
    ix, iy = int(round(dx)), int(round(dy))
    sx0, sx1, dx0, dx1 = max(0, -ix), min(w, w - ix), max(0, ix), min(w, w + ix)
    sy0, sy1, dy0, dy1 = max(0, -iy), min(h, h - iy), max(0, iy), min(h, h + iy)
    if sx0 < sx1 and sy0 < sy1:
        out[dy0:dy1, dx0:dx1] = image[sy0:sy1, sx0:sx1]
        cov[dy0:dy1, dx0:dx1] = 1.0
    return out, cov
