"""Oracle: rejection statistics and weighted integration.

Restates, operation for operation, the NumPy arithmetic of
  - src/glass/cpu/integration.py:36-118  (weighted_integrate_stack)
  - src/glass/engine/rejection.py:31-66  (center_and_scale dispatch)
  - src/glass/engine/rejection.py:215-240 (all-valid winsorized sigma)
  - src/glass/engine/rejection.py:242-297 (deterministic winsorized sigma)
  - src/glass/engine/rejection.py:299-366 (percentile helpers)
  - src/glass/engine/rejection.py:323-349 (frame-axis std)
The dtypes and rounding points are the reference's (float32 arrays, float64
sums, NEP 50 scalar promotion); only the code organisation is this file's.

Also defines linear-fit clipping, which the reference lacks, in float64
(`linear_fit_clip_reference`), as the specification the CUDA kernel follows.
"""

from __future__ import annotations

import numpy as np

_F32 = np.float32


def _percentile_count(sorted_stack: np.ndarray, count: np.ndarray, fraction: float) -> np.ndarray:
    """rejection.py:299-321 - per-pixel count, value = lo*(1-t) + hi*t in float32."""
    n = np.maximum(count, 1).astype(np.int64)
    pos = (n - 1).astype(_F32) * _F32(fraction)
    lo_idx = np.floor(pos).astype(np.int64)
    hi_idx = np.minimum(lo_idx + 1, n - 1).astype(np.int64)
    t = (pos - lo_idx.astype(_F32)).astype(_F32)
    lo_val = np.take_along_axis(sorted_stack, lo_idx[None], axis=0)[0].astype(_F32)
    hi_val = np.take_along_axis(sorted_stack, hi_idx[None], axis=0)[0].astype(_F32)
    out = (lo_val * (_F32(1.0) - t) + hi_val * t).astype(_F32)
    return np.where(count > 0, out, _F32(0.0)).astype(_F32)


def _percentile_all(sorted_stack: np.ndarray, percent: float) -> np.ndarray:
    """rejection.py:352-366 - whole-stack frame count, value = lo + (hi-lo)*f."""
    frames = int(sorted_stack.shape[0])
    if frames == 1:
        return np.asarray(sorted_stack[0], dtype=_F32)
    pos = (_F32(percent) / _F32(100.0)) * _F32(frames - 1)
    lo = int(np.floor(pos))
    hi = int(np.ceil(pos))
    f = _F32(pos - lo)
    lo_val = np.asarray(sorted_stack[lo], dtype=_F32)
    if hi == lo:
        return lo_val
    hi_val = np.asarray(sorted_stack[hi], dtype=_F32)
    return (lo_val + (hi_val - lo_val) * f).astype(_F32)


def _std_valid(data: np.ndarray, valid: np.ndarray, count: np.ndarray) -> np.ndarray:
    """rejection.py:323-349 - float64 std with the mean rounded to float32."""
    n64 = count.astype(np.float64)
    d64 = data.astype(np.float64)
    total = np.sum(np.where(valid, d64, 0.0), axis=0, dtype=np.float64)
    mean = np.divide(total, n64, out=np.zeros_like(total), where=count > 0).astype(_F32)
    dev = d64 - mean[None].astype(np.float64)
    ss = np.sum(np.where(valid, dev * dev, 0.0), axis=0, dtype=np.float64)
    var = np.divide(ss, n64, out=np.zeros_like(ss), where=count > 0)
    return np.sqrt(var).astype(_F32)


def winsorized_all_valid(stack: np.ndarray, low_sigma: float, high_sigma: float):
    """rejection.py:219-240 - used when every sample of the stack is valid."""
    data = np.asarray(stack, dtype=_F32)
    ordered = np.sort(data, axis=0)
    med = _percentile_all(ordered, 50.0)
    q25 = _percentile_all(ordered, 25.0)
    q75 = _percentile_all(ordered, 75.0)
    scale1 = ((q75 - q25) / _F32(1.349)).astype(_F32)
    std_all = np.std(data, axis=0, dtype=np.float64).astype(_F32)
    scale1 = np.where(scale1 > 0, scale1, std_all)
    lo = med - _F32(low_sigma) * scale1
    hi = med + _F32(high_sigma) * scale1
    clipped = np.clip(data, lo[None], hi[None])
    center = np.mean(clipped, axis=0, dtype=np.float64).astype(_F32)
    scale = np.std(clipped, axis=0, dtype=np.float64).astype(_F32)
    scale = np.where(scale > 0, scale, scale1)
    return center.astype(_F32), scale.astype(_F32)


def winsorized_masked(stack: np.ndarray, valid: np.ndarray, low_sigma: float, high_sigma: float):
    """rejection.py:242-297 - per-pixel valid counts (the general case)."""
    data = np.asarray(stack, dtype=_F32)
    ok = np.asarray(valid, dtype=bool) & np.isfinite(data)
    count = np.sum(ok, axis=0).astype(np.int64)
    ordered = np.sort(np.where(ok, data, np.inf), axis=0)
    med = _percentile_count(ordered, count, 0.5)
    q25 = _percentile_count(ordered, count, 0.25)
    q75 = _percentile_count(ordered, count, 0.75)
    std_fb = _std_valid(data, ok, count)
    scale1 = ((q75 - q25) / _F32(1.349)).astype(_F32)
    scale1 = np.where((scale1 > 0) & np.isfinite(scale1), scale1, std_fb).astype(_F32)
    lo = (med - _F32(low_sigma) * scale1).astype(_F32)
    hi = (med + _F32(high_sigma) * scale1).astype(_F32)
    clipped = np.clip(data, lo[None], hi[None])
    n64 = count.astype(np.float64)
    wsum = np.sum(np.where(ok, clipped, _F32(0.0)).astype(np.float64), axis=0, dtype=np.float64)
    wmean = np.divide(wsum, n64, out=np.zeros_like(wsum), where=count > 0).astype(_F32)
    dev = clipped.astype(np.float64) - wmean[None].astype(np.float64)
    ss = np.sum(np.where(ok, dev * dev, 0.0), axis=0, dtype=np.float64)
    var = np.divide(ss, n64, out=np.zeros_like(ss), where=count > 0)
    scale = np.sqrt(var).astype(_F32)
    scale = np.where((scale > 0) & np.isfinite(scale), scale, scale1).astype(_F32)
    has = count > 0
    return (np.where(has, wmean, _F32(0.0)).astype(_F32), np.where(has, scale, _F32(0.0)).astype(_F32))


def center_and_scale(stack: np.ndarray, valid: np.ndarray, method: str, low_sigma: float, high_sigma: float):
    """rejection.py:31-66 (sigma_clip / winsorized_sigma / mad)."""
    if method == "winsorized_sigma" and bool(np.all(valid)) and bool(np.all(np.isfinite(stack))):
        return winsorized_all_valid(stack, low_sigma, high_sigma)
    masked = np.where(valid, stack, np.nan)
    if method in ("sigma", "sigma_clip"):
        center = np.nanmedian(masked, axis=0)
        scale = np.nanstd(masked, axis=0)
    elif method in ("mad", "median_sigma"):
        center = np.nanmedian(masked, axis=0)
        scale = _F32(1.4826) * np.nanmedian(np.abs(masked - center[None]), axis=0)
    elif method == "winsorized_sigma":
        center, scale = winsorized_masked(stack, valid, low_sigma, high_sigma)
    else:
        raise ValueError(f"unsupported rejection statistics method: {method}")
    return (np.nan_to_num(center, nan=0.0).astype(_F32), np.nan_to_num(scale, nan=0.0).astype(_F32))


def _guarded_masks(valid, low, high, min_samples, max_reject_fraction):
    """cpu/integration.py:84-99 - cancel rejections the guard does not allow."""
    rejected = low | high
    if np.any(rejected):
        total = np.sum(valid, axis=0)
        nrej = np.sum(rejected, axis=0)
        remaining = total - nrej
        frac = np.divide(nrej, np.maximum(total, 1), out=np.zeros_like(total, dtype=_F32), where=total > 0)
        allowed = (remaining >= int(min_samples)) & (frac <= _F32(max_reject_fraction))
        low = low & allowed[None]
        high = high & allowed[None]
    return low, high


def linear_fit_clip_reference(column: np.ndarray, low_sigma: float, high_sigma: float,
                              iterations: int = 5) -> tuple[int, int]:
    """Linear-fit clipping of one pixel's valid samples, in float64.

    The reference has no linear-fit clipping; this is the definition the CUDA
    kernel implements.  Fit v = a + b*(r - c) (r = rank within the kept range,
    c = (n-1)/2) to the sorted kept samples, sigma = mean |v - fit|, walk in
    from both ends rejecting v < fit - k_lo*sigma / v > fit + k_hi*sigma, keep
    ties of the first kept value, repeat until stable.  Returns the kept rank
    range [lo, hi) of the sorted column.
    """
    y = np.sort(np.asarray(column, dtype=np.float64))
    lo, hi = 0, y.size
    for _ in range(int(iterations)):
        n = hi - lo
        if n < 3:
            break
        seg = y[lo:hi]
        c = 0.5 * (n - 1)
        r = np.arange(n, dtype=np.float64) - c
        a0 = float(np.sum(seg)) / n
        b = float(np.sum(r * seg)) / (n * (n * n - 1) / 12.0)
        fit = a0 + b * r
        sigma = float(np.sum(np.abs(seg - fit))) / n
        new_lo, new_hi = lo, hi
        while new_lo < hi and y[new_lo] < (a0 + b * ((new_lo - lo) - c)) - low_sigma * sigma:
            new_lo += 1
        while new_hi > new_lo and y[new_hi - 1] > (a0 + b * ((new_hi - 1 - lo) - c)) + high_sigma * sigma:
            new_hi -= 1
        if new_hi <= new_lo:
            break
        while new_lo > lo and y[new_lo - 1] == y[new_lo]:
            new_lo -= 1
        while new_hi < hi and y[new_hi] == y[new_hi - 1]:
            new_hi += 1
        if new_lo == lo and new_hi == hi:
            break
        lo, hi = new_lo, new_hi
    return lo, hi


def weighted_integrate_stack(stack, weights=None, rejection="none", low_sigma=3.0, high_sigma=3.0,
                             min_samples=3, max_reject_fraction=0.5, coverage=None,
                             linear_fit_iterations=5):
    """cpu/integration.py:36-118 -> (master, weight_map, coverage, low, high), all float32.

    rejection: "none" | "sigma_clip" | "winsorized_sigma" | "linear_fit" (the
    last one is this project's definition, see linear_fit_clip_reference).
    """
    frames = np.asarray(stack, dtype=_F32)
    if frames.ndim != 3:
        raise ValueError("stack must have shape (frame_count, height, width)")
    if min_samples < 1:
        raise ValueError("min_samples must be at least 1")
    if not 0.0 <= max_reject_fraction <= 1.0:
        raise ValueError("max_reject_fraction must be between 0 and 1")
    n, h, w = frames.shape
    fw = np.ones(n, dtype=_F32) if weights is None else np.asarray(weights, dtype=_F32)
    if fw.shape != (n,):
        raise ValueError("weights must have shape (frame_count,)")
    if coverage is None:
        valid = np.isfinite(frames)
    else:
        cov = np.asarray(coverage, dtype=_F32)
        valid = (cov > 0.5) & np.isfinite(frames)
    valid = valid & np.isfinite(fw)[:, None, None] & (fw[:, None, None] > 0)
    low_map = np.zeros((h, w), dtype=_F32)
    high_map = np.zeros((h, w), dtype=_F32)
    if rejection in ("sigma_clip", "winsorized_sigma"):
        center, scale = center_and_scale(frames, valid, rejection, low_sigma, high_sigma)
        lt = center - _F32(low_sigma) * scale
        ht = center + _F32(high_sigma) * scale
        low = valid & (frames < lt[None])
        high = valid & (frames > ht[None])
        low, high = _guarded_masks(valid, low, high, min_samples, max_reject_fraction)
        low_map = np.sum(low, axis=0).astype(_F32)
        high_map = np.sum(high, axis=0).astype(_F32)
        valid = valid & ~(low | high)
    elif rejection == "linear_fit":
        low = np.zeros_like(valid)
        high = np.zeros_like(valid)
        for y in range(h):
            for x in range(w):
                ok = valid[:, y, x]
                col = frames[ok, y, x].astype(np.float64)
                if col.size == 0:
                    continue
                lo, hi = linear_fit_clip_reference(col, low_sigma, high_sigma, linear_fit_iterations)
                ordered = np.sort(col)
                vlo, vhi = ordered[lo], ordered[hi - 1]
                low[:, y, x] = ok & (frames[:, y, x] < vlo)
                high[:, y, x] = ok & (frames[:, y, x] > vhi)
        low, high = _guarded_masks(valid, low, high, min_samples, max_reject_fraction)
        low_map = np.sum(low, axis=0).astype(_F32)
        high_map = np.sum(high, axis=0).astype(_F32)
        valid = valid & ~(low | high)
    elif rejection != "none":
        raise ValueError(f"unsupported rejection mode: {rejection}")
    eff = np.where(valid, fw[:, None, None], 0.0).astype(np.float64)
    wsum = np.sum(np.where(valid, frames, 0.0).astype(np.float64) * eff, axis=0)
    wmap = np.sum(eff, axis=0)
    cov_map = np.sum(valid, axis=0).astype(_F32)
    master = np.divide(wsum, wmap, out=np.zeros_like(wsum), where=wmap > 0)
    return master.astype(_F32), wmap.astype(_F32), cov_map, low_map, high_map


def dq_map(master, weight, coverage=None, low=None, high=None, geometric=None, active_frame_count=0):
    """resident_cuda.py:3110-3297 - int16 DQ bits (contracts.py:77-88)."""
    m = np.asarray(master, dtype=_F32)
    w = np.asarray(weight, dtype=_F32)
    dq = np.zeros(m.shape, dtype=np.int16)
    invalid = ~np.isfinite(m) | ~np.isfinite(w) | (w <= 0)
    if coverage is not None:
        c = np.asarray(coverage, dtype=_F32)
        bad = ~np.isfinite(c) | (c <= 0.5)
        dq[bad] |= 64
        invalid |= bad
    if geometric is not None:
        g = np.asarray(geometric, dtype=_F32)
        bad = ~np.isfinite(g) | (g <= 0.5)
        dq[bad] |= 64
        invalid |= bad
        if active_frame_count > 0:
            partial = np.isfinite(g) & (g > 0.5) & (g < float(active_frame_count) - 0.5)
            dq[partial] |= 64
    dq[invalid] |= 1
    if low is not None:
        lo = np.asarray(low, dtype=_F32)
        dq[np.isfinite(lo) & (lo > 0)] |= 256
    if high is not None:
        hi = np.asarray(high, dtype=_F32)
        dq[np.isfinite(hi) & (hi > 0)] |= 512
    return dq

