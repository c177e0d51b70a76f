"""Oracle: triangle-asterism star registration.

Restates src/glass/cpu/registration.py:106-475 (similarity and affine
models) with the same NumPy arithmetic:

- ``local_triangle_descriptors``  :273-303 (+ ``_ordered_triangle_by_sides``
  :242-270, ``_triangle_area`` :236-239)
- ``fit_similarity``              :140-162 (Procrustes through a 2x2 SVD)
- ``fit_affine``                  :106-119 (least squares of the 2n x 6 system)
- ``greedy_pairs`` / ``score``    :177-215
- ``estimate_triangle_asterism_transform`` :361-475
- ``similarity_from_descriptors`` the descriptor-list fallback of
  src/glass_cuda.py:2097-2140

Point lists are (n, 2) float64 arrays, brightest star first.  Results are
plain dicts with the StarRegistration fields (cpu/registration.py:11-20)
except the warning strings.
"""

from __future__ import annotations

from itertools import combinations

import numpy as np

_EDGES = ((0, 1), (1, 2), (2, 0))


def _norm(v) -> float:
    return float(np.linalg.norm(v))


def ordered_triangle(points: np.ndarray, raw: tuple[int, int, int]):
    """registration.py:242-270 -> (ordered global indices, descriptor) or None
    when degenerate."""
    tri = points[list(raw)]
    sides = np.asarray([_norm(tri[a] - tri[b]) for a, b in _EDGES], dtype=np.float64)
    short, mid, long_ = (float(v) for v in np.sort(sides))
    if short <= 1.0e-6 or mid <= 1.0e-6:
        return None
    a, b = _EDGES[int(np.argmax(sides))]
    c = 3 - a - b
    if _norm(tri[a] - tri[c]) < _norm(tri[b] - tri[c]):
        a, b = b, a
    order = (raw[a], raw[b], raw[c])
    return order, np.asarray([long_ / mid, mid / short], dtype=np.float64)


def triangle_area(tri: np.ndarray) -> float:
    """registration.py:236-239."""
    e1 = tri[1] - tri[0]
    e2 = tri[2] - tri[0]
    return abs(float(e1[0] * e2[1] - e1[1] * e2[0])) * 0.5


def local_triangle_descriptors(points, max_points: int, neighbors: int, max_descriptors: int):
    """registration.py:273-303 -> list of (descriptor[2], (i, j, k), area),
    area-descending (stable)."""
    pts = np.asarray(points, dtype=np.float64).reshape(-1, 2)[: max(0, int(max_points))]
    n = len(pts)
    if n < 3:
        return []
    k = min(n, max(3, int(neighbors)))
    seen: set[tuple[int, ...]] = set()
    out = []
    for anchor in range(n):
        dist = np.sqrt(np.sum((pts - pts[anchor]) ** 2, axis=1))
        near = [int(i) for i in np.argsort(dist, kind="stable")[:k]]
        for raw in combinations(near, 3):
            key = tuple(sorted(raw))
            if key in seen:
                continue
            seen.add(key)
            area = triangle_area(pts[list(raw)])
            if area < 2.0:
                continue
            got = ordered_triangle(pts, raw)
            if got is None:
                continue
            out.append((got[1], got[0], area))
    out.sort(key=lambda item: item[2], reverse=True)
    return out[: int(max_descriptors)]


def fit_similarity(moving: np.ndarray, reference: np.ndarray) -> np.ndarray | None:
    """registration.py:140-162; None where the reference raises ValueError."""
    if len(moving) < 2:
        return None
    mm = np.mean(moving, axis=0)
    rm = np.mean(reference, axis=0)
    mc = moving - mm
    rc = reference - rm
    variance = float(np.sum(mc * mc))
    if variance <= 1.0e-12:
        return None
    u, s, vt = np.linalg.svd(mc.T @ rc)
    rot = vt.T @ u.T
    if np.linalg.det(rot) < 0:
        vt[-1, :] *= -1
        rot = vt.T @ u.T
    lin = float(np.sum(s) / variance) * rot
    t = rm - mm @ lin.T
    return np.asarray([[lin[0, 0], lin[0, 1], t[0]], [lin[1, 0], lin[1, 1], t[1]], [0.0, 0.0, 1.0]],
                      dtype=np.float64)


def fit_affine(moving: np.ndarray, reference: np.ndarray) -> np.ndarray | None:
    """registration.py:106-119; None where the reference raises ValueError."""
    if len(moving) < 3:
        return None
    rows, rhs = [], []
    for (x, y), (rx, ry) in zip(moving, reference):
        rows.append([x, y, 1.0, 0.0, 0.0, 0.0])
        rows.append([0.0, 0.0, 0.0, x, y, 1.0])
        rhs.extend([rx, ry])
    p, *_ = np.linalg.lstsq(np.asarray(rows, dtype=np.float64), np.asarray(rhs, dtype=np.float64), rcond=None)
    return np.asarray([[p[0], p[1], p[2]], [p[3], p[4], p[5]], [0.0, 0.0, 1.0]], dtype=np.float64)


def fit_model(transform_model: str, moving: np.ndarray, reference: np.ndarray) -> np.ndarray | None:
    """registration.py:165-174 for the two models of the asterism estimator."""
    if transform_model == "similarity":
        return fit_similarity(moving, reference)
    if transform_model == "affine":
        return fit_affine(moving, reference)
    raise ValueError("triangle asterism registration supports similarity or affine transforms")


def apply_matrix(points: np.ndarray, matrix: np.ndarray) -> np.ndarray:
    """registration.py:46-51."""
    hom = np.hstack([points, np.ones((points.shape[0], 1), dtype=np.float64)])
    out = hom @ matrix.T
    w = out[:, 2:3]
    return np.divide(out[:, :2], w, out=out[:, :2].copy(), where=np.abs(w) > 1.0e-12)


def greedy_pairs(reference: np.ndarray, transformed: np.ndarray, tol: float):
    """registration.py:177-207 -> (pairs [(moving, reference)], rms)."""
    if len(reference) == 0 or len(transformed) == 0:
        return [], float("inf")
    d = transformed[:, None, :] - reference[None, :, :]
    dist = np.sqrt(np.sum(d * d, axis=2))
    cand = [(int(i), int(j)) for i, j in np.argwhere(dist <= tol)]
    if not cand:
        return [], float("inf")
    cand.sort(key=lambda p: float(dist[p[0], p[1]]))
    used_m: set[int] = set()
    used_r: set[int] = set()
    pairs, res = [], []
    for i, j in cand:
        if i in used_m or j in used_r:
            continue
        used_m.add(i)
        used_r.add(j)
        pairs.append((i, j))
        res.append(float(dist[i, j]))
    return pairs, float(np.sqrt(np.mean(np.square(res))))


def score(reference: np.ndarray, moving: np.ndarray, matrix: np.ndarray, tol: float):
    """registration.py:210-215."""
    return greedy_pairs(reference, apply_matrix(moving, matrix), tol)


def _failed(reason: str, ndesc=(0, 0), matches=0) -> dict:
    return {"matrix": np.eye(3), "inliers": 0, "rms_px": float("nan"), "status": "failed", "pairs": [],
            "reference_descriptor_count": ndesc[0], "moving_descriptor_count": ndesc[1],
            "descriptor_matches": matches, "reason": reason}


def estimate_triangle_asterism_transform(reference, moving, min_inliers: int = 6, tolerance_px: float = 3.0,
                                         max_stars: int = 80, neighbors: int = 5, descriptor_radius: float = 0.1,
                                         max_descriptors: int = 1200, max_candidates: int = 1500,
                                         transform_model: str = "similarity") -> dict:
    """registration.py:361-475 (similarity or affine fits)."""
    if transform_model not in ("similarity", "affine"):
        raise ValueError("triangle asterism registration supports similarity or affine transforms")
    ref = np.asarray(reference, dtype=np.float64).reshape(-1, 2)[: max(0, int(max_stars))]
    mov = np.asarray(moving, dtype=np.float64).reshape(-1, 2)[: max(0, int(max_stars))]
    if len(ref) < 3 or len(mov) < 3:
        return _failed("not enough stars")
    rdesc = local_triangle_descriptors(ref, max_stars, neighbors, max_descriptors)
    mdesc = local_triangle_descriptors(mov, max_stars, neighbors, max_descriptors)
    if not rdesc or not mdesc:
        return _failed("no descriptors", (len(rdesc), len(mdesc)))
    rvec = np.asarray([d[0] for d in rdesc], dtype=np.float64)
    matches = []
    for mdv, midx, _area in mdesc:
        dist = np.sqrt(np.sum((rvec - mdv) ** 2, axis=1))
        for r in np.nonzero(dist <= descriptor_radius)[0]:
            matches.append((float(dist[int(r)]), midx, rdesc[int(r)][1]))
    matches.sort(key=lambda item: item[0])
    matches = matches[: int(max_candidates)]
    best, best_pairs, best_rms, best_index = np.eye(3), [], float("inf"), -1
    for c, (_d, midx, ridx) in enumerate(matches):
        mt = mov[list(midx)]
        rt = ref[list(ridx)]
        for o, rto in enumerate((rt, rt[[1, 0, 2]])):
            m = fit_model(transform_model, mt, rto)
            if m is None:
                continue
            pairs, rms = score(ref, mov, m, tolerance_px)
            if len(pairs) > len(best_pairs) or (len(pairs) == len(best_pairs) and rms < best_rms):
                best, best_pairs, best_rms, best_index = m, pairs, rms, 2 * c + o
    for _ in range(3):
        if len(best_pairs) < 3:
            break
        m = fit_model(transform_model, mov[[p[0] for p in best_pairs]], ref[[p[1] for p in best_pairs]])
        if m is None:
            break
        pairs, rms = score(ref, mov, m, tolerance_px)
        if len(pairs) > len(best_pairs) or (len(pairs) == len(best_pairs) and rms <= best_rms):
            best, best_pairs, best_rms = m, pairs, rms
    return {"matrix": best, "inliers": len(best_pairs), "rms_px": best_rms if np.isfinite(best_rms) else float("nan"),
            "status": "ok" if len(best_pairs) >= min_inliers else "failed", "pairs": best_pairs,
            "reference_descriptor_count": len(rdesc), "moving_descriptor_count": len(mdesc),
            "descriptor_matches": len(matches), "best_candidate_index": best_index}


def similarity_from_descriptors(ref_xy, mov_xy, ref_desc, ref_idx, mov_desc, mov_idx, tolerance_px: float = 2.0,
                                descriptor_radius: float = 0.1) -> dict:
    """src/glass_cuda.py:2097-2140: every (reference, moving) descriptor pair
    within the radius, float32 descriptor distance, both orientations, no refit."""
    ref = np.asarray(ref_xy, dtype=np.float32).reshape(-1, 2).astype(np.float64)
    mov = np.asarray(mov_xy, dtype=np.float32).reshape(-1, 2).astype(np.float64)
    rd = np.asarray(ref_desc, dtype=np.float32).reshape(-1, 2)
    md = np.asarray(mov_desc, dtype=np.float32).reshape(-1, 2)
    ri = np.asarray(ref_idx, dtype=np.int32).reshape(-1, 3)
    mi = np.asarray(mov_idx, dtype=np.int32).reshape(-1, 3)
    best, best_pairs, best_rms, best_index = np.eye(3), [], float("inf"), -1
    index = 0
    for r in range(len(rd)):
        for m in range(len(md)):
            if float(np.linalg.norm(rd[r] - md[m])) > descriptor_radius:
                index += 2
                continue
            mt = mov[mi[m]]
            rt = ref[ri[r]]
            for rto in (rt, rt[[1, 0, 2]]):
                mat = fit_similarity(mt, rto)
                if mat is not None:
                    pairs, rms = score(ref, mov, mat, tolerance_px)
                    if len(pairs) > len(best_pairs) or (len(pairs) == len(best_pairs) and rms < best_rms):
                        best, best_pairs, best_rms, best_index = mat, pairs, rms, index
                index += 1
    return {"matrix": best, "inliers": len(best_pairs), "rms_px": best_rms if np.isfinite(best_rms) else float("nan"),
            "status": "ok" if best_pairs else "failed", "pairs": best_pairs, "best_candidate_index": best_index}
