"""Oracle: isolated cosmetic-defect detection (source DQ for light frames).

Restates src/glass/cpu/cosmetic.py:68-182 (detect_isolated_cosmetic_defects
with _global_robust_location_scale and _eight_neighbors) and :184-307
(star_protection_mask, detect_star_protected_cosmetic_defects), which the
resident path turns into invalid (NaN) samples without replacing them
(src/glass/engine/resident_source_dq.py:76-131, 825-925).  Returns boolean
masks instead of the reference's DQMask: (hot, cold, candidate_hot,
candidate_cold), plus the star-protected pixels for the protected variant.
"""

from __future__ import annotations

import warnings

import numpy as np

from oracle.stars import detect_stars, robust_background

_F32 = np.float32


def _eight_neighbors(image: np.ndarray) -> np.ndarray:
    padded = np.pad(image, 1, mode="edge")
    return np.stack([padded[0:-2, 0:-2], padded[0:-2, 1:-1], padded[0:-2, 2:], padded[1:-1, 0:-2],
                     padded[1:-1, 2:], padded[2:, 0:-2], padded[2:, 1:-1], padded[2:, 2:]], axis=0).astype(_F32)


def isolated_defects(data, hot_sigma=8.0, cold_sigma=8.0, structure_sigma=1.5, min_neighbor_support=2):
    """-> dict of boolean masks hot, cold, candidate_hot, candidate_cold and
    the scalars median, sigma (cpu/cosmetic.py:97-182)."""
    image = np.asarray(data, dtype=_F32)
    median, _rms, _mad, sigma = robust_background(image)
    finite_mask = np.isfinite(image)
    if not np.any(finite_mask):
        z = np.zeros(image.shape, dtype=bool)
        return {"hot": z, "cold": z, "candidate_hot": z, "candidate_cold": z, "median": 0.0, "sigma": 0.0}
    neighbors = _eight_neighbors(image)
    finite_neighbors = np.where(np.isfinite(neighbors), neighbors, np.nan)
    with np.errstate(all="ignore"), warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)  # all-NaN neighbourhoods
        local_median = np.nanmedian(finite_neighbors, axis=0).astype(_F32)
    local_median = np.where(np.isfinite(local_median), local_median, _F32(median))
    hot_limit = _F32(median + float(hot_sigma) * sigma)
    cold_limit = _F32(median - float(cold_sigma) * sigma)
    hot_delta = _F32(float(hot_sigma) * sigma)
    cold_delta = _F32(float(cold_sigma) * sigma)
    with np.errstate(invalid="ignore"):
        cand_hot = finite_mask & (image > hot_limit) & ((image - local_median) > hot_delta)
        cand_cold = finite_mask & (image < cold_limit) & ((local_median - image) > cold_delta)
        support_sigma = max(0.0, float(structure_sigma))
        hot_support = np.count_nonzero(finite_neighbors > _F32(median + support_sigma * sigma), axis=0)
        cold_support = np.count_nonzero(finite_neighbors < _F32(median - support_sigma * sigma), axis=0)
    required = max(0, int(min_neighbor_support))
    return {"hot": cand_hot & (hot_support < required), "cold": cand_cold & (cold_support < required),
            "candidate_hot": cand_hot, "candidate_cold": cand_cold, "median": float(median), "sigma": float(sigma)}


def star_protection_mask(shape, stars, radius_px=3.0, min_pixels=3, max_sharpness=0.95) -> np.ndarray:
    """cpu/cosmetic.py:184-222 for star tuples (x, y, flux, peak, fwhm, ecc,
    snr, sharpness, npix)."""
    height, width = int(shape[0]), int(shape[1])
    protected = np.zeros((height, width), dtype=bool)
    radius = max(0.0, float(radius_px))
    if radius <= 0.0:
        return protected
    r2 = radius * radius
    for s in stars:
        if int(s[8]) < int(min_pixels):
            continue
        if s[7] is not None and float(s[7]) > float(max_sharpness):
            continue
        cx, cy = float(s[0]), float(s[1])
        if not (np.isfinite(cx) and np.isfinite(cy)):
            continue
        x0, x1 = max(0, int(np.floor(cx - radius))), min(width, int(np.ceil(cx + radius)) + 1)
        y0, y1 = max(0, int(np.floor(cy - radius))), min(height, int(np.ceil(cy + radius)) + 1)
        if x1 <= x0 or y1 <= y0:
            continue
        yy, xx = np.ogrid[y0:y1, x0:x1]
        protected[y0:y1, x0:x1] |= (xx - cx) * (xx - cx) + (yy - cy) * (yy - cy) <= r2
    return protected


def star_protected_defects(data, hot_sigma=8.0, cold_sigma=8.0, structure_sigma=1.5, min_neighbor_support=2,
                           star_threshold_sigma=5.0, star_max_candidates=500, star_protection_radius_px=3.0,
                           star_min_pixels=3, star_max_sharpness=0.95):
    """cpu/cosmetic.py:225-307: the isolated detector with flags cleared
    inside the protection discs of compact catalog stars."""
    image = np.asarray(data, dtype=_F32)
    iso = isolated_defects(image, hot_sigma, cold_sigma, structure_sigma, min_neighbor_support)
    catalog = detect_stars(image, threshold_sigma=float(star_threshold_sigma), max_stars=int(star_max_candidates),
                           min_separation_px=max(2.0, float(star_protection_radius_px) * 0.5))
    protected = star_protection_mask(image.shape, catalog, star_protection_radius_px, star_min_pixels,
                                     star_max_sharpness)
    out = dict(iso)
    out["star_protected_hot"] = protected & iso["hot"]
    out["star_protected_cold"] = protected & iso["cold"]
    out["hot"] = iso["hot"] & ~protected
    out["cold"] = iso["cold"] & ~protected
    out["star_count"] = len(catalog)
    return out


def threshold_mask(frame, low_threshold, high_threshold, apply=True):
    """Threshold-only cosmetic mask of one frame, as
    ResidentCalibratedStack.apply_cosmetic_threshold_mask_frame /
    count_cosmetic_threshold_mask_frame do it on the device
    (cpp/src/native_bindings.cpp:3243-3400 over
    cpp/cuda/integration_kernels.cu:181-232): every sample is tested in the
    order non-finite, > high (hot), < low (cold), the thresholds compared as
    float32.  Returns (frame after the call, hot, cold, non-finite counts);
    with apply the three classes become NaN, otherwise the frame is returned
    unchanged."""
    x = np.asarray(frame, dtype=_F32)
    lo, hi = _F32(low_threshold), _F32(high_threshold)
    if np.isnan(lo) or np.isnan(hi) or lo > hi:
        raise ValueError("cosmetic thresholds must be finite-or-infinite values with low <= high")
    nonfinite = ~np.isfinite(x)
    with np.errstate(invalid="ignore"):
        hot = ~nonfinite & (x > hi)
        cold = ~nonfinite & ~hot & (x < lo)
    out = x.copy()
    if apply:
        out[nonfinite | hot | cold] = np.nan
    return out, int(hot.sum()), int(cold.sum()), int(nonfinite.sum())
