"""Oracle: tile-local weighted integration.

Restates glass_integrate_resident_tile_local_weighted_mean_f32_kernel and
glass_integrate_resident_tile_local_sigma_clip_f32_kernel
(cpp/cuda/integration_kernels.cu:1658-1711, 3622-3796; argument rules
native_bindings.cpp:12998-13100): per pixel, the weight of a target frame is
multiplied by the multiplier of the tile whose half-open extent contains the
pixel (1 outside every tile); a sample takes part when its weight is > 0 and
finite and it is finite.  float32 arithmetic in frame order with one rounding
per operation (the reference's CUDA build may fuse a += b * c into one
fused multiply-add, which this restatement does not do).
"""

from __future__ import annotations

import numpy as np

_F32 = np.float32


def _multiplier_map(h: int, w: int, extents, multipliers) -> np.ndarray:
    mult = np.ones((h, w), dtype=_F32)
    done = np.zeros((h, w), dtype=bool)
    for (x0, y0, x1, y1), m in zip(np.asarray(extents).reshape(-1, 4), np.asarray(multipliers, dtype=_F32)):
        sl = (slice(y0, y1), slice(x0, x1))
        mult[sl] = np.where(done[sl], mult[sl], m)
        done[sl] = True
    return mult


def integrate_tile_local(stack, weights, target_mask, extents, multipliers, mode: str = "mean",
                         low_sigma: float = 3.0, high_sigma: float = 3.0):
    """mode "mean" -> (master, weight); "sigma" / "winsorized" -> (master,
    weight, coverage, low, high), all float32."""
    data = np.asarray(stack, dtype=_F32)
    n, h, w = data.shape
    wts = np.ones(n, dtype=_F32) if weights is None else np.asarray(weights, dtype=_F32)
    tgt = np.asarray(target_mask).astype(bool)
    mult = _multiplier_map(h, w, extents, multipliers)
    eff = [np.where(tgt[f], wts[f] * mult, wts[f]).astype(_F32) for f in range(n)]
    take = [(eff[f] > 0) & np.isfinite(eff[f]) & np.isfinite(data[f]) for f in range(n)]
    zero = np.zeros((h, w), dtype=_F32)
    lo_t = np.full((h, w), -np.inf, dtype=_F32)
    hi_t = np.full((h, w), np.inf, dtype=_F32)
    ok = np.ones((h, w), dtype=bool)
    ls, hs = _F32(low_sigma), _F32(high_sigma)
    if mode != "mean":
        mean, count = zero.copy(), zero.copy()
        for f in range(n):
            mean = np.where(take[f], mean + data[f], mean)
            count = np.where(take[f], count + _F32(1.0), count)
        ok = count > 0
        mean = np.where(ok, mean / np.where(ok, count, _F32(1.0)), zero).astype(_F32)
        var = zero.copy()
        for f in range(n):
            d = (data[f] - mean).astype(_F32)
            var = np.where(take[f], var + d * d, var)
        safe = np.where(ok, count, _F32(1.0))
        center, scale = mean, np.sqrt(var / safe).astype(_F32)
        lo_t = (center - ls * scale).astype(_F32)
        hi_t = (center + hs * scale).astype(_F32)
        if mode == "winsorized":
            wm = zero.copy()
            for f in range(n):
                wm = np.where(take[f], wm + np.clip(data[f], lo_t, hi_t), wm)
            wm = (wm / safe).astype(_F32)
            wv = zero.copy()
            for f in range(n):
                d = (np.clip(data[f], lo_t, hi_t) - wm).astype(_F32)
                wv = np.where(take[f], wv + d * d, wv)
            center, scale = wm, np.sqrt(wv / safe).astype(_F32)
            lo_t = (center - ls * scale).astype(_F32)
            hi_t = (center + hs * scale).astype(_F32)
    s, ws, cov, lowc, highc = zero.copy(), zero.copy(), zero.copy(), zero.copy(), zero.copy()
    for f in range(n):
        t = take[f] & ok
        v = data[f]
        if mode != "mean":
            is_low = t & (v < lo_t)
            is_high = t & ~is_low & (v > hi_t)
            lowc = np.where(is_low, lowc + _F32(1.0), lowc)
            highc = np.where(is_high, highc + _F32(1.0), highc)
            t = t & ~is_low & ~is_high
        s = np.where(t, s + v * eff[f], s)
        ws = np.where(t, ws + eff[f], ws)
        cov = np.where(t, cov + _F32(1.0), cov)
    master = np.where(ws > 0, s / np.where(ws > 0, ws, _F32(1.0)), zero).astype(_F32)
    if mode == "mean":
        return master, ws
    return master, ws, cov, lowc, highc
