"""Oracle: alignment metrics and sub-pixel translation refinement.

Restates the reference's NumPy paths in src/glass_cuda.py:

- ``alignment_metrics``      matrix_alignment_metrics_f32 :706-768
- ``refine_translation``     refine_matrix_translation_with_metrics_f32 :771-900
- ``translation_ncc``        estimate_translation_subpixel_ncc_f32 :1175-1245
  with _translation_bilinear_ncc_score :1131-1172

The bilinear warp is ``oracle.warp.warp_matrix`` (the reference's warp
semantics, pinned separately).  Statistics are float64 like the reference.
"""

from __future__ import annotations

import numpy as np

from .warp import warp_matrix

_F32 = np.float32


def _stats(ref_valid: np.ndarray, warped_valid: np.ndarray, sampled: int, stride: int) -> dict:
    n = int(ref_valid.size)
    if n == 0:
        return {"valid_pixels": 0, "sampled_pixels": sampled, "sample_stride": stride, "rms": float("nan"),
                "mean_abs_diff": float("nan"), "ncc": float("nan")}
    diff = warped_valid - ref_valid
    rms = float(np.sqrt(np.mean(diff * diff)))
    mad = float(np.mean(np.abs(diff)))
    if n <= 1:
        ncc = float("nan")
    else:
        rc = ref_valid - float(np.mean(ref_valid))
        wc = warped_valid - float(np.mean(warped_valid))
        den = float(np.sqrt(np.sum(rc * rc) * np.sum(wc * wc)))
        ncc = float(np.sum(rc * wc) / den) if den > 0.0 else float("nan")
    return {"valid_pixels": n, "sampled_pixels": sampled, "sample_stride": stride, "rms": rms,
            "mean_abs_diff": mad, "ncc": ncc}


def alignment_metrics(reference, moving, matrix, sample_stride: int = 1) -> dict:
    """glass_cuda.py:706-768 (NumPy path)."""
    ref = np.asarray(reference, dtype=_F32)
    mov = np.asarray(moving, dtype=_F32)
    warped, coverage = warp_matrix(mov, np.asarray(matrix, dtype=np.float64), "bilinear", 0.0)
    s = max(1, int(sample_stride))
    rs = ref[::s, ::s].astype(np.float64)
    ws = warped[::s, ::s].astype(np.float64)
    valid = (coverage[::s, ::s] > 0.0) & np.isfinite(rs) & np.isfinite(ws)
    return _stats(rs[valid], ws[valid], int(rs.size), s)


def _arange32(start: float, stop: float, step: float) -> np.ndarray:
    return np.arange(start, stop, step, dtype=_F32)


def refine_translation(reference, moving, matrix, search_radius_px: float = 1.0, coarse_step_px: float = 0.25,
                       fine_radius_px: float = 0.25, fine_step_px: float = 0.0625, coarse_sample_stride: int = 4,
                       final_sample_stride: int = 1) -> dict:
    """glass_cuda.py:771-900 (NumPy path): coarse grid, then fine grid, key
    (rms, -ncc), first candidate wins ties."""
    base = np.asarray(matrix, dtype=_F32).reshape(3, 3)

    def score(dx, dy, stride):
        cand = np.array(base, copy=True)
        cand[0, 2] += _F32(dx)
        cand[1, 2] += _F32(dy)
        m = alignment_metrics(reference, moving, cand.astype(np.float64), stride)
        return (m["rms"], -m["ncc"]), m, cand

    offsets = _arange32(-float(search_radius_px), float(search_radius_px) + float(coarse_step_px) * 0.5,
                        float(coarse_step_px))
    best_key = None
    best_dx = best_dy = 0.0
    best_m = None
    best_mat = np.array(base, copy=True)
    coarse = 0
    for dx in offsets:
        for dy in offsets:
            key, m, cand = score(float(dx), float(dy), coarse_sample_stride)
            coarse += 1
            if best_key is None or key < best_key:
                best_key, best_dx, best_dy, best_m, best_mat = key, float(dx), float(dy), m, cand
    fine = 0
    if fine_radius_px > 0.0:
        fx = _arange32(best_dx - float(fine_radius_px), best_dx + float(fine_radius_px) + float(fine_step_px) * 0.5,
                       float(fine_step_px))
        fy = _arange32(best_dy - float(fine_radius_px), best_dy + float(fine_radius_px) + float(fine_step_px) * 0.5,
                       float(fine_step_px))
        best_key = None
        for dx in fx:
            for dy in fy:
                key, m, cand = score(float(dx), float(dy), final_sample_stride)
                fine += 1
                if best_key is None or key < best_key:
                    best_key, best_dx, best_dy, best_m, best_mat = key, float(dx), float(dy), m, cand
    elif final_sample_stride != coarse_sample_stride:
        _key, best_m, best_mat = score(best_dx, best_dy, final_sample_stride)
    return {"matrix": best_mat.astype(_F32), "dx_correction": best_dx, "dy_correction": best_dy,
            "metrics": best_m, "coarse_candidates": coarse, "fine_candidates": fine}


def translation_ncc(reference, moving, center_dx: float, center_dy: float, radius_steps: int, step: float,
                    sample_stride: int = 1) -> dict:
    """glass_cuda.py:1131-1245 (NumPy path), vectorised per candidate."""
    ref = np.asarray(reference, dtype=_F32)
    mov = np.asarray(moving, dtype=_F32)
    h, w = ref.shape
    s = max(1, int(sample_stride))
    ys, xs = np.mgrid[0:h:s, 0:w:s]
    best = (float(center_dx), float(center_dy), float("-inf"))
    count = 0
    for oy in range(-int(radius_steps), int(radius_steps) + 1):
        for ox in range(-int(radius_steps), int(radius_steps) + 1):
            dx = float(center_dx) + ox * float(step)
            dy = float(center_dy) + oy * float(step)
            sx = xs.astype(np.float64) - dx
            sy = ys.astype(np.float64) - dy
            ok = (sx >= 0.0) & (sx <= float(w - 1)) & (sy >= 0.0) & (sy <= float(h - 1))
            x0 = np.floor(np.where(ok, sx, 0.0)).astype(np.int64)
            y0 = np.floor(np.where(ok, sy, 0.0)).astype(np.int64)
            x1 = np.minimum(x0 + 1, w - 1)
            y1 = np.minimum(y0 + 1, h - 1)
            tx = (np.where(ok, sx, 0.0) - x0).astype(_F32)
            ty = (np.where(ok, sy, 0.0) - y0).astype(_F32)
            one = _F32(1.0)
            top = mov[y0, x0] * (one - tx) + mov[y0, x1] * tx
            bottom = mov[y1, x0] * (one - tx) + mov[y1, x1] * tx
            m = (top * (one - ty) + bottom * ty).astype(np.float64)
            r = ref[ys, xs].astype(np.float64)
            valid = ok & np.isfinite(r) & np.isfinite(m)
            count += 1
            rv, mv = r[valid], m[valid]
            if rv.size <= 1:
                score = float("-inf")
            else:
                rc = rv - float(np.mean(rv))
                mc = mv - float(np.mean(mv))
                den = float(np.sqrt(np.sum(rc * rc) * np.sum(mc * mc)))
                score = float(np.sum(rc * mc) / den) if den > 0.0 else float("-inf")
            if score > best[2]:
                best = (dx, dy, score)
    return {"dx": best[0], "dy": best[1], "score": best[2], "candidate_count": count}
