"""Oracle: the light-stack step evaluated entirely in float64.

Test infrastructure.  The other oracle modules restate the reference's
arithmetic with its float32 rounding points (bit-exact parity targets); this
one evaluates the same definitions with every operation in float64 and no
intermediate float32 rounding, so that the error of each float32 output map
of the device path can be stated against exact-as-practical values:
  - calibration   cpu/calibration.py:51-76 (dark scaled by exposure, bias,
                  flat floored), float64;
  - warp          Lanczos3 / bilinear through oracle.adjoint.warp_affine_f64
                  (engine/warp.py:99-152 sampling, float64 weights and sums);
  - weights       simple SNR |mean| / std of a frame's finite samples
                  (resident_cuda.py:1948-1956), float64;
  - integration   winsorized sigma clipping (engine/rejection.py:242-297:
                  median, IQR / 1.349 with the standard-deviation fallback,
                  winsorize, mean / std of the clipped column with the first
                  scale as fallback), the reject thresholds and the
                  min-samples / max-fraction guard of cpu/integration.py:36-118,
                  weighted mean; float64 throughout.
"""

from __future__ import annotations

import numpy as np

from oracle.adjoint import warp_affine_f64


def calibrate_f64(raw, bias=None, dark=None, flat=None, dark_scale=1.0, flat_floor=1.0e-6):
    out = np.asarray(raw, dtype=np.float64).copy()
    if dark is not None:
        out -= np.asarray(dark, dtype=np.float64) * float(dark_scale)
    if bias is not None:
        out -= np.asarray(bias, dtype=np.float64)
    if flat is not None:
        out /= np.maximum(np.asarray(flat, dtype=np.float64), flat_floor)
    return out


def warp_frames_f64(frames, matrices, interpolation="lanczos3"):
    """Frames warped through affine moving -> reference matrices (NaN outside)."""
    out = np.empty_like(np.asarray(frames, dtype=np.float64))
    for k, (f, m) in enumerate(zip(frames, matrices)):
        inv = np.linalg.inv(np.asarray(m, dtype=np.float64))
        out[k] = warp_affine_f64(f, inv[:2].reshape(-1), interpolation, np.nan)
    return out


def simple_snr_weights_f64(frames, eps=1.0e-6):
    w = []
    for f in frames:
        v = np.asarray(f, dtype=np.float64)
        v = v[np.isfinite(v)]
        w.append(max(abs(v.mean()) / max(v.std(), eps), eps) if v.size else eps)
    return np.asarray(w, dtype=np.float64)


def _percentile(ordered, count, fraction):
    n = np.maximum(count, 1)
    pos = (n - 1) * fraction
    lo = np.floor(pos).astype(np.int64)
    hi = np.minimum(lo + 1, n - 1)
    t = pos - lo
    lv = np.take_along_axis(ordered, lo[None], axis=0)[0]
    hv = np.take_along_axis(ordered, hi[None], axis=0)[0]
    return np.where(count > 0, lv * (1.0 - t) + hv * t, 0.0)


def winsorized_integrate_f64(stack, weights, low_sigma=3.0, high_sigma=3.0, min_samples=3,
                             max_reject_fraction=0.5):
    """-> (master, weight, coverage, low, high) as float64 / int64 maps."""
    data = np.asarray(stack, dtype=np.float64)
    w = np.asarray(weights, dtype=np.float64)
    valid = np.isfinite(data) & np.isfinite(w)[:, None, None] & (w[:, None, None] > 0)
    count = valid.sum(axis=0)
    cnt = np.maximum(count, 1)
    ordered = np.sort(np.where(valid, data, np.inf), axis=0)
    med = _percentile(ordered, count, 0.5)
    q25 = _percentile(ordered, count, 0.25)
    q75 = _percentile(ordered, count, 0.75)
    zero = np.where(valid, data, 0.0)
    mean0 = zero.sum(axis=0) / cnt
    std0 = np.sqrt((np.where(valid, data - mean0, 0.0) ** 2).sum(axis=0) / cnt)
    s1 = (q75 - q25) / 1.349
    s1 = np.where((s1 > 0) & np.isfinite(s1), s1, std0)
    clipped = np.clip(data, (med - low_sigma * s1)[None], (med + high_sigma * s1)[None])
    m = np.where(valid, clipped, 0.0).sum(axis=0) / cnt
    s = np.sqrt((np.where(valid, clipped - m, 0.0) ** 2).sum(axis=0) / cnt)
    s = np.where((s > 0) & np.isfinite(s), s, s1)
    lt, ht = m - low_sigma * s, m + high_sigma * s
    low = valid & (data < lt[None])
    high = valid & (data > ht[None])
    rej = low | high
    nrej = rej.sum(axis=0)
    allowed = ((count - nrej) >= min_samples) & (nrej / cnt <= max_reject_fraction)
    low &= allowed[None]
    high &= allowed[None]
    kept = valid & ~(low | high)
    eff = np.where(kept, w[:, None, None], 0.0)
    wmap = eff.sum(axis=0)
    master = np.divide((np.where(kept, data, 0.0) * eff).sum(axis=0), wmap, out=np.zeros_like(wmap),
                       where=wmap > 0)
    return master, wmap, kept.sum(axis=0), low.sum(axis=0), high.sum(axis=0), s
