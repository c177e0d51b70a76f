"""Oracle: star detection.

Restates src/glass/cpu/star_detect.py:29-168 (robust_background,
_measure_candidate, _dedupe_stars, detect_stars) with the same NumPy
arithmetic; returns plain tuples instead of the reference's Star dataclass:
(x, y, flux, peak, fwhm, eccentricity, snr, sharpness, npix), fwhm /
eccentricity None when undefined.
"""

from __future__ import annotations

import numpy as np

_F32 = np.float32


def robust_background(data):
    """star_detect.py:29-42 -> (median, rms, mad, noise) as Python floats."""
    image = np.asarray(data, dtype=_F32)
    finite = image[np.isfinite(image)]
    if finite.size == 0:
        return 0.0, 0.0, 0.0, 1.0
    median = float(np.median(finite))
    rms = float(np.std(finite))
    mad = float(np.median(np.abs(finite - median)))
    noise = float(1.4826 * mad)
    if noise <= 0.0:
        noise = rms
    if noise <= 0.0:
        noise = 1.0
    return median, rms, mad, noise


def measure(image, x, y, background, noise, radius):
    """star_detect.py:45-100 for one candidate peak (x, y)."""
    h, w = image.shape
    y0, y1 = max(0, y - radius), min(h, y + radius + 1)
    x0, x1 = max(0, x - radius), min(w, x + radius + 1)
    patch = image[y0:y1, x0:x1]
    finite = np.isfinite(patch)
    if not np.any(finite):
        return None
    weights = np.where(finite, np.maximum(patch - _F32(background), 0.0), 0.0)
    flux = float(np.sum(weights, dtype=np.float64))
    if flux <= 0.0:
        return None
    yy, xx = np.mgrid[y0:y1, x0:x1]
    cx = float(np.sum(xx * weights, dtype=np.float64) / flux)
    cy = float(np.sum(yy * weights, dtype=np.float64) / flux)
    dx = xx - cx
    dy = yy - cy
    mxx = float(np.sum(dx * dx * weights, dtype=np.float64) / flux)
    myy = float(np.sum(dy * dy * weights, dtype=np.float64) / flux)
    mxy = float(np.sum(dx * dy * weights, dtype=np.float64) / flux)
    trace = max(mxx + myy, 0.0)
    root = float(np.sqrt(max((mxx - myy) * (mxx - myy) + 4.0 * mxy * mxy, 0.0)))
    major = max((trace + root) / 2.0, 0.0)
    minor = max((trace - root) / 2.0, 0.0)
    mean_sigma = float(np.sqrt(max((major + minor) / 2.0, 0.0)))
    fwhm = 2.354820045 * mean_sigma if mean_sigma > 0.0 else None
    ecc = float(np.sqrt(max(0.0, 1.0 - minor / major))) if major > 0.0 else None
    peak = float(max(float(image[y, x]) - background, 0.0))
    npix = int(np.count_nonzero(weights > 0.0))
    snr = flux / max(float(noise) * np.sqrt(max(npix, 1)), 1.0e-6)
    return (cx, cy, flux, peak, None if fwhm is None else float(fwhm), ecc, float(snr),
            float(peak / max(flux, 1.0e-6)), npix)


def _median_sorted(s: np.ndarray) -> float:
    n = s.size
    m = n // 2
    return float(s[m]) if n % 2 else float((s[m - 1] + s[m]) * 0.5)


def background_mesh(data, cell: int):
    """Background mesh, this project's definition (the reference thresholds
    against one global median / MAD): per cell of cell x cell pixels from the
    top-left corner, the float64 median of the finite pixels and the noise
    1.4826 * MAD (1 when the MAD is 0); NaN for a cell without finite pixels.
    -> (background [ny, nx], noise [ny, nx])."""
    image = np.asarray(data, dtype=_F32)
    h, w = image.shape
    ny, nx = -(-h // cell), -(-w // cell)
    bg = np.full((ny, nx), np.nan)
    nz = np.full((ny, nx), np.nan)
    for j in range(ny):
        for i in range(nx):
            v = image[j * cell:(j + 1) * cell, i * cell:(i + 1) * cell]
            v = np.sort(v[np.isfinite(v)].astype(np.float64))
            if v.size == 0:
                continue
            med = _median_sorted(v)
            mad = _median_sorted(np.sort(np.abs(v - med)))
            bg[j, i] = med
            nz[j, i] = 1.4826 * mad if mad > 0.0 else 1.0
    return bg, nz


def _mesh_axis(coord, cell: int, n: int):
    u = (np.asarray(coord, dtype=np.float64) + 0.5) / cell - 0.5
    fl = np.floor(u)
    lo, hi = fl < 0.0, fl >= n - 1
    i0 = np.where(lo, 0, np.where(hi, n - 1, fl)).astype(np.int64)
    f = np.where(lo | hi, 0.0, u - fl)
    return i0, np.minimum(i0 + 1, n - 1), f


def mesh_value(mesh: np.ndarray, cell: int, x, y):
    """Bilinear interpolation of a mesh between cell centres ((i + 0.5) *
    cell - 0.5), clamped at the first and last centre, float64."""
    ny, nx = mesh.shape
    i0, i1, fx = _mesh_axis(x, cell, nx)
    j0, j1, fy = _mesh_axis(y, cell, ny)
    top = (1.0 - fx) * mesh[j0, i0] + fx * mesh[j0, i1]
    bottom = (1.0 - fx) * mesh[j1, i0] + fx * mesh[j1, i1]
    return (1.0 - fy) * top + fy * bottom


def detect_stars(data, threshold_sigma=5.0, max_stars=500, background=None, noise=None, window_radius=4,
                 min_separation_px=2.0, mesh_cell: int = 0):
    """star_detect.py:121-168 -> list of star tuples, brightest first.

    mesh_cell > 0 (this project's extension): the threshold at each pixel is
    the interpolated mesh background + k * max(noise, 1e-6), compared in
    float64, and each star is measured against the interpolated background
    and noise at its peak."""
    image = np.asarray(data, dtype=_F32)
    h, w = image.shape
    if mesh_cell:
        bgm, nzm = background_mesh(image, mesh_cell)
        ys_, xs_ = np.mgrid[0:h, 0:w]
        bg_map = mesh_value(bgm, mesh_cell, xs_, ys_)
        nz_map = mesh_value(nzm, mesh_cell, xs_, ys_)
        thr_map = bg_map + float(threshold_sigma) * np.maximum(nz_map, 1.0e-6)
        if h < 3 or w < 3:
            return []
        core = image[1:-1, 1:-1]
        with np.errstate(invalid="ignore"):
            mask = np.isfinite(core) & (core.astype(np.float64) > thr_map[1:-1, 1:-1])
    else:
        median, _rms, _mad, est_noise = robust_background(image)
        bg = median if background is None else float(background)
        sigma = est_noise if noise is None else float(noise)
        threshold = bg + threshold_sigma * max(sigma, 1.0e-6)
        if h < 3 or w < 3:
            return []
        core = image[1:-1, 1:-1]
        mask = np.isfinite(core) & (core > threshold)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            if dx or dy:
                mask &= core >= image[1 + dy:h - 1 + dy, 1 + dx:w - 1 + dx]
    ys, xs = np.nonzero(mask)
    radius = max(1, int(window_radius))
    if mesh_cell:
        found = (measure(image, int(x + 1), int(y + 1), float(bg_map[y + 1, x + 1]), float(nz_map[y + 1, x + 1]),
                         radius) for y, x in zip(ys, xs))
    else:
        found = (measure(image, int(x + 1), int(y + 1), bg, sigma, radius) for y, x in zip(ys, xs))
    stars = [s for s in found if s is not None]
    if min_separation_px > 0.0 and len(stars) > 1:
        kept = []
        sep2 = float(min_separation_px * min_separation_px)
        for s in sorted(stars, key=lambda item: item[2], reverse=True):
            if all((s[0] - o[0]) ** 2 + (s[1] - o[1]) ** 2 >= sep2 for o in kept):
                kept.append(s)
        stars = kept
    stars.sort(key=lambda item: item[2], reverse=True)
    return stars[:max_stars]
