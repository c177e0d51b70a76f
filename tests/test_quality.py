"""Registration-quality policy (glass_gb300.quality) against the reference's
own functions: tests/golden/quality.npz holds the outputs of
`_resident_triangle_agreement_quality` / `_resident_triangle_agreement_policy`
(src/glass/engine/resident_cuda.py:4905-4998) and
`evaluate_resident_registration_quality`
(src/glass/engine/resident_registration_quality.py:41-136) on a grid of
inputs - NaN and missing metrics, negative RMS, every action, floors,
reference / failed / excluded statuses, catalog-capacity limits - made by
tests/golden/make_golden.py `make_quality`."""

from __future__ import annotations

import json
import math

import numpy as np
import pytest

from glass_gb300 import quality

from .conftest import GOLDEN


@pytest.fixture(scope="module")
def golden_quality():
    z = np.load(GOLDEN / "quality.npz")
    return json.loads(bytes(z["json"]).decode())


def _same(a, b):
    if isinstance(a, float) and isinstance(b, float) and math.isnan(a) and math.isnan(b):
        return True
    return a == b


def test_agreement_quality_and_policy_match_reference(golden_quality):
    records = golden_quality["agreement"]
    assert len(records) > 1000
    for rec in records:
        ncc, rms, fit, scale, min_score, action, floor = rec["args"]
        q = quality.agreement_quality(ncc, rms, fit, scale, min_score)
        for key, exp in rec["quality"].items():
            assert _same(q[key], exp), (rec["args"], key, q[key], exp)
        pol = quality.agreement_policy(q, action, floor)
        for key, exp in rec["policy"].items():
            assert _same(pol[key], exp), (rec["args"], key, pol[key], exp)


def test_registration_gate_matches_reference(golden_quality):
    gates = golden_quality["gate"]
    assert len(gates) > 500
    for rec in gates:
        status, inliers, rms, mode, action, min_inliers, max_rms, ref_stars, mov_stars = rec["args"]
        got = quality.registration_quality(status, inliers, rms, mode, action, min_inliers, max_rms, ref_stars,
                                           mov_stars)
        for key, exp in rec["out"].items():
            assert _same(got[key], exp), (rec["args"], key, got[key], exp)


def test_policy_argument_errors():
    with pytest.raises(ValueError):
        quality.agreement_quality(0.5, 10.0, 0.1, 0.0)
    with pytest.raises(ValueError):
        quality.agreement_quality(0.5, 10.0, 0.1, 200.0, 1.5)
    with pytest.raises(ValueError):
        quality.agreement_policy({"status": "failed"}, "drop")
    with pytest.raises(ValueError):
        quality.registration_quality("ok", 3, 0.1, requested_action="maybe")
