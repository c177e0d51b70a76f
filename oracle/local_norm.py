"""Oracle: grid local normalisation of registered frames to the reference frame.

Restates the resident path (the default of `glass run`, mode grid_mean_std,
tile 256; cli.py:476-479):
  - pair_grid_stats: per tile of tile_h x tile_w pixels from the top-left
    corner, the float64 sums of the source and reference pixels and of their
    squares over the pixels finite in both, then mean = sum / n and
    std = sqrt(max(sum2 / n - mean^2, 0)) in float64, stored as float32
    (cpp/cuda/local_norm_kernels.cu:220-300 + native_bindings.cpp:10745-10760);
  - grid_coefficients: empty tiles keep scale 1 / offset 0; a tile whose
    source or reference std is <= eps gets scale 1 and offset
    ref_mean - src_mean; otherwise scale = float32(ref_std / src_std) and
    offset = float32(ref_mean - src_mean * scale), all float32 arithmetic
    (src/glass/engine/resident_cuda.py:1897-1927);
  - apply_grid: out = data * scale + offset per tile, float32 multiply then
    float32 add (src/glass/cpu/local_norm.py:197-215; the reference's CUDA
    apply kernel, local_norm_kernels.cu:30-52, is compiled with fused
    multiply-adds and can differ from this by one rounding).
The float64 sums are NumPy's (pairwise); the device sums in float-float, so
the float32 statistics agree except when a value lies within ~1e-14 of a
float32 rounding boundary.
"""

from __future__ import annotations

import numpy as np

_F32 = np.float32


def grid_shape(height: int, width: int, tile_h: int, tile_w: int) -> tuple[int, int]:
    if tile_h <= 0 or tile_w <= 0:
        raise ValueError("tile dimensions must be positive")
    return -(-height // tile_h), -(-width // tile_w)


def pair_grid_stats(source, reference, tile_h: int, tile_w: int) -> dict:
    src = np.asarray(source, dtype=_F32)
    ref = np.asarray(reference, dtype=_F32)
    h, w = src.shape
    rows, cols = grid_shape(h, w, tile_h, tile_w)
    out = {k: np.zeros((rows, cols), dtype=_F32) for k in ("source_mean", "source_std", "reference_mean",
                                                           "reference_std")}
    out["valid_pixels"] = np.zeros((rows, cols), dtype=np.uint64)
    for gy in range(rows):
        for gx in range(cols):
            s = src[gy * tile_h:(gy + 1) * tile_h, gx * tile_w:(gx + 1) * tile_w]
            r = ref[gy * tile_h:(gy + 1) * tile_h, gx * tile_w:(gx + 1) * tile_w]
            ok = np.isfinite(s) & np.isfinite(r)
            n = int(np.count_nonzero(ok))
            out["valid_pixels"][gy, gx] = n
            if n == 0:
                continue
            sv = s[ok].astype(np.float64)
            rv = r[ok].astype(np.float64)
            inv = 1.0 / float(n)
            sm = float(np.sum(sv)) * inv
            rm = float(np.sum(rv)) * inv
            svar = max(float(np.sum(sv * sv)) * inv - sm * sm, 0.0)
            rvar = max(float(np.sum(rv * rv)) * inv - rm * rm, 0.0)
            out["source_mean"][gy, gx] = _F32(sm)
            out["source_std"][gy, gx] = _F32(np.sqrt(svar))
            out["reference_mean"][gy, gx] = _F32(rm)
            out["reference_std"][gy, gx] = _F32(np.sqrt(rvar))
    return out


def grid_coefficients(stats: dict, eps: float = 1.0e-6) -> tuple[np.ndarray, np.ndarray]:
    sm = np.asarray(stats["source_mean"], dtype=_F32)
    ss = np.asarray(stats["source_std"], dtype=_F32)
    rm = np.asarray(stats["reference_mean"], dtype=_F32)
    rs = np.asarray(stats["reference_std"], dtype=_F32)
    valid = np.asarray(stats["valid_pixels"], dtype=np.uint64)
    scales = np.ones_like(sm, dtype=_F32)
    offsets = np.zeros_like(sm, dtype=_F32)
    for row in range(sm.shape[0]):
        for col in range(sm.shape[1]):
            if int(valid[row, col]) == 0:
                continue
            if float(ss[row, col]) <= eps or float(rs[row, col]) <= eps:
                offsets[row, col] = _F32(rm[row, col] - sm[row, col])
                continue
            scale = _F32(rs[row, col] / ss[row, col])
            scales[row, col] = scale
            offsets[row, col] = _F32(rm[row, col] - sm[row, col] * scale)
    return scales, offsets


def apply_grid(data, scales, offsets, tile_h: int, tile_w: int) -> np.ndarray:
    src = np.asarray(data, dtype=_F32)
    sg = np.asarray(scales, dtype=_F32)
    og = np.asarray(offsets, dtype=_F32)
    h, w = src.shape
    if sg.shape != grid_shape(h, w, tile_h, tile_w) or og.shape != sg.shape:
        raise ValueError("coefficient grid shape does not match data shape and tile dimensions")
    out = np.empty_like(src)
    for gy in range(sg.shape[0]):
        for gx in range(sg.shape[1]):
            sl = (slice(gy * tile_h, (gy + 1) * tile_h), slice(gx * tile_w, (gx + 1) * tile_w))
            out[sl] = src[sl] * sg[gy, gx] + og[gy, gx]
    return out


def normalize_frames(frames, reference_index: int, weights, tile: int = 256, eps: float = 1.0e-6):
    """The resident sequence (resident_cuda.py:12920-13040): every frame with
    a positive weight except the reference is normalised to the reference,
    tile by tile; a frame without any paired finite pixel gets weight 0 and
    stays as it is.  -> (frames, weights)."""
    out = np.array(frames, dtype=_F32, copy=True)
    w = np.array(weights, dtype=_F32, copy=True)
    for k in range(out.shape[0]):
        if k == reference_index or not float(w[k]) > 0.0:
            continue
        stats = pair_grid_stats(out[k], out[reference_index], tile, tile)
        if int(np.sum(stats["valid_pixels"], dtype=np.uint64)) == 0:
            w[k] = 0.0
            continue
        scales, offsets = grid_coefficients(stats, eps)
        out[k] = apply_grid(out[k], scales, offsets, tile, tile)
    return out, w
