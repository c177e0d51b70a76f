"""Oracle (test infrastructure): deterministic grid star catalogs.

Restates the reference's resident grid catalog (the semantics of
cpp/cuda/star_detect_kernels.cu; only tests/, smoke() and bench.py's CPU legs
use this module):
  - local maxima: star_detect_kernels.cu:40-68 (interior pixel, finite, value >
    threshold, not below any of its 8 neighbours; tests/test_gpu_star_detect.py
    :8-21 states the same rule in NumPy);
  - candidate order: star_detect_kernels.cu:70-101 (larger value, then
    smaller y, then smaller x);
  - per-cell top-K with cells [cx*W//cols, (cx+1)*W//cols) x [...]:
    star_detect_kernels.cu:317-498;
  - flux-ordered merge and the greedy separation scan (squared float32
    distance < min_separation^2): :500-648;
  - windowed centroid (radius clamped to 1..8, window clipped to the frame,
    background = median of the finite window samples - the mean of the two
    middle ones, in float32, for an even count - or the given global mean;
    weights max(v - bg, 0) in float32, float64 sums, status 1 when moved):
    :650-742;
  - the frame's global mean of finite samples (float64 sum, float32 result):
    native_bindings.cpp:12400-12430.
Pure Python loops over candidates: small frames only.
"""

from __future__ import annotations

import numpy as np

_F32 = np.float32


def local_maxima(image, threshold: float) -> list[tuple[float, int, int]]:
    """All candidates as (value, y, x)."""
    img = np.asarray(image, dtype=_F32)
    h, w = img.shape
    if h < 3 or w < 3:
        return []
    core = img[1:-1, 1:-1]
    with np.errstate(invalid="ignore"):
        mask = np.isfinite(core) & (core > _F32(threshold))
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                if dx or dy:
                    mask &= ~(core < img[1 + dy:h - 1 + dy, 1 + dx:w - 1 + dx])
    ys, xs = np.nonzero(mask)
    return [(float(core[y, x]), int(y + 1), int(x + 1)) for y, x in zip(ys, xs)]


def _order(c):
    value, y, x = c
    return (-value, y, x)


def grid_catalog(image, threshold: float, grid_cols: int, grid_rows: int, candidates_per_cell: int,
                 max_output_candidates: int, min_separation_px: float, centroid_radius: int = 0,
                 global_mean_background: bool = False) -> dict:
    """-> {"count", "stored_count", "x", "y", "flux", "x_before", "y_before", "status"}."""
    img = np.asarray(image, dtype=_F32)
    h, w = img.shape
    cands = local_maxima(img, threshold)
    kept = []
    for cy in range(grid_rows):
        y0, y1 = cy * h // grid_rows, (cy + 1) * h // grid_rows
        for cx in range(grid_cols):
            x0, x1 = cx * w // grid_cols, (cx + 1) * w // grid_cols
            cell = [c for c in cands if y0 <= c[1] < y1 and x0 <= c[2] < x1]
            kept.extend(sorted(cell, key=_order)[:candidates_per_cell])
    kept.sort(key=_order)
    sep2 = _F32(min_separation_px) * _F32(min_separation_px)
    out = []
    for value, y, x in kept:
        if len(out) >= max_output_candidates:
            break
        fx, fy = _F32(x), _F32(y)
        clash = False
        for _, oy, ox in out:
            dx, dy = fx - _F32(ox), fy - _F32(oy)
            if _F32(dx * dx) + _F32(dy * dy) < sep2:
                clash = True
                break
        if not clash:
            out.append((value, y, x))
    xb = np.array([c[2] for c in out], dtype=_F32)
    yb = np.array([c[1] for c in out], dtype=_F32)
    flux = np.array([c[0] for c in out], dtype=_F32)
    xs, ys = xb.copy(), yb.copy()
    status = np.zeros(len(out), dtype=np.uint8)
    if centroid_radius > 0:
        bg_global = float("nan")
        if global_mean_background:
            finite = img[np.isfinite(img)].astype(np.float64)
            if finite.size:
                bg_global = float(_F32(finite.sum() / finite.size))
        r = min(max(int(centroid_radius), 1), 8)
        for i in range(len(out)):
            cx = int(np.floor(_F32(xb[i]) + _F32(0.5)))
            cy = int(np.floor(_F32(yb[i]) + _F32(0.5)))
            if not (0 <= cx < w and 0 <= cy < h):
                continue
            wx0, wx1 = max(0, cx - r), min(w - 1, cx + r)
            wy0, wy1 = max(0, cy - r), min(h - 1, cy + r)
            win = img[wy0:wy1 + 1, wx0:wx1 + 1]
            bg = _F32(bg_global) if np.isfinite(bg_global) else None
            if bg is None:
                samples = np.sort(win[np.isfinite(win)])
                if samples.size == 0:
                    continue
                m = samples.size
                bg = samples[m // 2] if m & 1 else _F32(_F32(0.5) * _F32(samples[m // 2 - 1] + samples[m // 2]))
            sw = sx = sy = 0.0
            for yy in range(wy0, wy1 + 1):
                for xx in range(wx0, wx1 + 1):
                    v = img[yy, xx]
                    if not np.isfinite(v):
                        continue
                    wt = max(_F32(v - bg), _F32(0.0))
                    if wt <= 0.0:
                        continue
                    sw += float(wt)
                    sx += float(xx) * float(wt)
                    sy += float(yy) * float(wt)
            if sw <= 0.0:
                continue
            xs[i], ys[i] = _F32(sx / sw), _F32(sy / sw)
            status[i] = 1
    return {"count": len(cands), "stored_count": len(out), "x": xs, "y": ys, "flux": flux, "x_before": xb,
            "y_before": yb, "status": status}
