"""Registration-quality frame weighting of the resident run, host side.

Three decisions of the reference's resident registration decide whether a
registered frame keeps its weight:

* the pixel-agreement score of its final matrix,
  score = NCC / (1 + max(0, pixel RMS) / rms_scale_adu), checked against an
  optional minimum (``_resident_triangle_agreement_quality``,
  src/glass/engine/resident_cuda.py:4905-4949);
* what a missed minimum does - "fail" (weight 0), "downweight" (weight x
  min(1, max(min_weight, score / min_score)), 0 is a failure) or "flag"
  (recorded only) - (``_resident_triangle_agreement_policy``,
  resident_cuda.py:4952-4998); the multiplier scales the frame's simple_snr
  weight (resident_cuda.py:12800-12809) and a hard failure zeroes it
  (resident_cuda.py:12466-12475);
* the registration quality gate on inliers and fit RMS
  (``evaluate_resident_registration_quality``,
  src/glass/engine/resident_registration_quality.py:41-136): "auto" means
  "exclude" for the CUDA triangle similarity mode, "off" otherwise.

The pixel NCC and RMS come from the alignment-metrics kernel
(gg_stack_alignment_metrics: bilinear resampling of the moving frame under
the matrix, every `sample_stride`-th pixel) - the metric the reference's
candidate-grid refinement reports for its selected matrix.
"""

from __future__ import annotations

import math
from typing import Any

AGREEMENT_ACTIONS = ("fail", "downweight", "flag")
QUALITY_ACTIONS = ("auto", "off", "warn", "exclude")
DEFAULT_QUALITY_MIN_INLIERS = 4


def _finite_or_nan(value: Any) -> float:
    try:
        v = float(value)
    except (TypeError, ValueError):
        return float("nan")
    return v


def agreement_quality(pixel_ncc: float, pixel_rms_adu: float, fit_rms_px: float, rms_scale_adu: float = 200.0,
                      min_score: float | None = None) -> dict[str, Any]:
    """Pixel-agreement score of one registered frame and its status:
    "audit_only" (no minimum), "unavailable" (no minimum, no score), "ok" or
    "failed" (score missing or below the minimum)."""
    scale = float(rms_scale_adu)
    if not scale > 0.0:
        raise ValueError("triangle agreement RMS scale must be positive")
    if min_score is not None and not 0.0 <= float(min_score) <= 1.0:
        raise ValueError("triangle minimum agreement score must be in [0, 1]")
    ncc, rms = _finite_or_nan(pixel_ncc), _finite_or_nan(pixel_rms_adu)
    if not math.isfinite(ncc):
        score, reason = float("nan"), "pixel_ncc_unavailable"
    elif not math.isfinite(rms):
        score, reason = float("nan"), "pixel_rms_unavailable"
    else:
        score, reason = ncc / (1.0 + max(0.0, rms) / scale), "ok"
    if min_score is None:
        status = "audit_only" if math.isfinite(score) else "unavailable"
    elif math.isfinite(score) and score >= float(min_score):
        status = "ok"
    else:
        status = "failed"
        reason = "below_min_score" if reason == "ok" else reason
    return {"score": score, "status": status, "reason": reason, "pixel_ncc": ncc, "pixel_rms_adu": rms,
            "fit_rms_px": _finite_or_nan(fit_rms_px), "rms_scale_adu": scale,
            "min_score": None if min_score is None else float(min_score)}


def agreement_policy(quality: dict[str, Any], action: str = "fail", min_weight: float = 0.0) -> dict[str, Any]:
    """What a frame's agreement status does to it: the weight multiplier,
    whether it fails hard (weight 0) and the resulting status."""
    if action not in AGREEMENT_ACTIONS:
        raise ValueError("triangle agreement action must be fail, downweight, or flag")
    floor = float(min_weight)
    if not 0.0 <= floor <= 1.0:
        raise ValueError("triangle agreement minimum weight must be in [0, 1]")
    status = str(quality.get("status") or "unavailable")
    out = {"action": action, "status": status, "hard_failure": False, "weight_multiplier": 1.0,
           "failure_message": None}
    if status != "failed":
        return out
    score = _finite_or_nan(quality.get("score"))
    min_score = quality.get("min_score")
    threshold = float("nan") if min_score is None else float(min_score)
    message = f"agreement_score {score:.6g} < {threshold:.6g}"
    if action == "fail":
        out.update(hard_failure=True, failure_message=message)
        return out
    if action == "flag":
        out["status"] = "flagged"
        return out
    if math.isfinite(score) and math.isfinite(threshold) and threshold > 0.0:
        multiplier = min(1.0, max(floor, max(0.0, score) / threshold))
    else:
        multiplier = floor if floor > 0.0 else 0.0
    out["weight_multiplier"] = float(multiplier)
    if multiplier > 0.0:
        out["status"] = "downweighted"
    else:
        out.update(status="failed", hard_failure=True,
                   failure_message=message + "; downweight multiplier was zero")
    return out


def resolve_quality_action(requested: str | None, registration_mode: str) -> str:
    action = str(requested or "auto").lower()
    if action not in QUALITY_ACTIONS:
        raise ValueError("resident registration quality gate must be auto, off, warn, or exclude")
    if action == "auto":
        return "exclude" if registration_mode == "similarity_cuda_triangle" else "off"
    return action


def registration_quality(status: str, inliers: int, rms_px: float, registration_mode: str = "similarity_cuda_triangle",
                         requested_action: str = "auto", min_inliers: int = DEFAULT_QUALITY_MIN_INLIERS,
                         max_rms_px: float | None = None, reference_stars: int | None = None,
                         moving_stars: int | None = None) -> dict[str, Any]:
    """The inlier / fit-RMS gate of one frame's registration: the final
    status ("ok", "excluded", ...), the decision and its reasons."""
    if min_inliers < 0:
        raise ValueError("resident registration quality min inliers must be non-negative")
    if max_rms_px is not None and not max_rms_px > 0.0:
        raise ValueError("resident registration quality max RMS must be positive when provided")
    action = resolve_quality_action(requested_action, registration_mode)
    original = str(status or "unknown")
    rms = _finite_or_nan(rms_px)
    capacity = None
    if reference_stars is not None and moving_stars is not None:
        capacity = min(int(reference_stars), int(moving_stars))
    reasons: list[str] = []
    if action in ("warn", "exclude") and original == "ok":
        if int(inliers) < int(min_inliers) and (capacity is None or capacity >= int(min_inliers)):
            reasons.append(f"registration_inliers_below_min:{int(inliers)}<{int(min_inliers)}")
        if max_rms_px is not None:
            if not math.isfinite(rms):
                reasons.append(f"registration_rms_non_finite:max={float(max_rms_px):.6g}")
            elif rms > float(max_rms_px):
                reasons.append(f"registration_rms_above_max:{rms:.6g}>{float(max_rms_px):.6g}")
    final, applied = original, "none"
    decisions = {"reference": "reference", "excluded": "already_excluded", "failed": "already_failed"}
    if action == "off":
        decision = "disabled"
    elif original in decisions:
        decision = decisions[original]
    elif original != "ok":
        decision = "not_applicable"
    elif reasons:
        decision, applied = ("rejected", "exclude") if action == "exclude" else ("warning", "warn")
        if action == "exclude":
            final = "excluded"
    else:
        decision = "accepted"
    return {"effective_action": action, "original_status": original, "final_status": final,
            "decision_status": decision, "action_applied": applied, "accepted": final in ("ok", "reference"),
            "inliers": int(inliers), "rms_px": rms if math.isfinite(rms) else None, "reasons": reasons,
            "catalog_capacity_limited": bool(capacity is not None and capacity < int(min_inliers)
                                             and int(inliers) < int(min_inliers))}
