"""Pins the oracle: it must reproduce the reference's outputs bit for bit.

Golden vectors come from the reference's own CPU code (tests/golden/
make_golden.py); the known-answer cases restate the reference's
tests/test_cpu_integration.py:10-97.
"""

from __future__ import annotations

import ast

import numpy as np
import pytest

from oracle import calibration as ocal
from oracle import integration as oint


def _variants(golden):
    out = []
    for spec in golden["_variants"]:
        rej, lo, hi, ms, mf = str(spec).split("|")
        out.append((rej, float(lo), float(hi), int(ms), float(mf)))
    return out


def test_integration_golden_bit_exact(golden_integration):
    g = golden_integration
    variants = _variants(g)
    names = [str(n) for n in g["_names"]]
    assert len(names) > 60
    for name in names:
        stack = g[f"{name}/stack"]
        weights = g[f"{name}/weights"] if f"{name}/weights" in g.files else None
        for vi, (rej, lo, hi, ms, mf) in enumerate(variants):
            out = oint.weighted_integrate_stack(stack, weights, rej, lo, hi, ms, mf)
            for key, value in zip(("master", "weight", "coverage", "low", "high"), out):
                expected = g[f"{name}/v{vi}/{key}"]
                assert value.dtype == expected.dtype, (name, vi, key)
                np.testing.assert_array_equal(value, expected, err_msg=f"{name} v{vi} {key}")


def test_integration_known_answers():
    """tests/test_cpu_integration.py:26-97 of the reference, restated."""
    stack = np.stack([np.ones((3, 3), np.float32), np.ones((3, 3), np.float32) * 3])
    cov = np.ones_like(stack)
    cov[1, 0, 0] = 0
    master, weight, c, low, high = oint.weighted_integrate_stack(stack, np.array([1, 3]), coverage=cov)
    assert np.allclose(master[1:, 1:], 2.5) and master[0, 0] == 1.0 and weight[0, 0] == 1.0 and c[0, 0] == 1.0

    stack = np.stack([np.ones((4, 4), np.float32)] * 4 + [np.ones((4, 4), np.float32) * 9])
    master, weight, c, low, high = oint.weighted_integrate_stack(stack, rejection="winsorized_sigma", high_sigma=1.0)
    assert np.allclose(master, 1) and np.all(weight == 4) and np.all(c == 4)
    assert np.sum(low) == 0 and np.sum(high) > 0

    stack = np.stack([np.ones((2, 2), np.float32)] * 3 + [np.ones((2, 2), np.float32) * 12])
    sm, _, sc, _, sh = oint.weighted_integrate_stack(stack, rejection="sigma_clip", low_sigma=2.4, high_sigma=2.4)
    assert np.allclose(sm, 3.75) and np.all(sc == 4) and np.sum(sh) == 0
    wm, ww, wc, wl, wh = oint.weighted_integrate_stack(stack, rejection="winsorized_sigma", low_sigma=2.4,
                                                       high_sigma=2.4)
    assert np.allclose(wm, 1.0) and np.all(ww == 3) and np.all(wc == 3) and np.sum(wl) == 0 and np.sum(wh) == 4
    gm, gw, gc, gl, gh = oint.weighted_integrate_stack(stack, rejection="winsorized_sigma", low_sigma=2.4,
                                                       high_sigma=2.4, max_reject_fraction=0.05)
    assert np.allclose(gm, 3.75) and np.all(gw == 4) and np.all(gc == 4) and np.sum(gl) == 0 and np.sum(gh) == 0


def test_integration_argument_errors():
    with pytest.raises(ValueError):
        oint.weighted_integrate_stack(np.zeros((2, 2), np.float32))
    with pytest.raises(ValueError):
        oint.weighted_integrate_stack(np.zeros((2, 2, 2), np.float32), min_samples=0)
    with pytest.raises(ValueError):
        oint.weighted_integrate_stack(np.zeros((2, 2, 2), np.float32), max_reject_fraction=1.5)
    with pytest.raises(ValueError):
        oint.weighted_integrate_stack(np.zeros((2, 2, 2), np.float32), rejection="bogus")


def test_calibration_golden_bit_exact(golden_calibration):
    g = golden_calibration
    specs = [ast.literal_eval(str(s)) for s in g["_specs"]]
    assert len(specs) >= 20
    for k, spec in enumerate(specs):
        policy = spec["policy"]
        out = ocal.calibrate_light(
            g["light"], g["bias"] if spec["bias"] else None, g["dark"] if spec["dark"] else None,
            g["flat"] if spec["flat"] else None, spec["t_light"], spec["t_dark"],
            master_dark_includes_bias=policy.get("master_dark_includes_bias", True),
            dark_scaling_enabled=policy.get("dark_scaling_enabled", True),
            flat_floor=policy.get("flat_floor", 1.0e-6), pedestal=policy.get("pedestal", 0.0),
        )
        np.testing.assert_array_equal(out, g[f"case{k}/out"], err_msg=f"case {k}: {spec}")


def test_fits_u16_round_trip():
    values = np.arange(0, 65536, 7, dtype=np.uint16)
    raw = ocal.encode_fits_u16be(values)
    assert raw.dtype == np.uint8 and raw.size == values.size * 2
    np.testing.assert_array_equal(ocal.decode_fits_u16be(raw, values.shape), values)
    # BZERO 32768: stored int16 -32768 is value 0
    assert ocal.decode_fits_u16be(np.array([0x80, 0x00], np.uint8), (1,))[0] == 0


def test_linear_fit_definition_rejects_outliers():
    col = np.concatenate([np.linspace(100.0, 110.0, 20), [500.0, -300.0]])
    lo, hi = oint.linear_fit_clip_reference(col, 3.0, 3.0)
    ordered = np.sort(col)
    assert ordered[lo] > -300.0 and ordered[hi - 1] < 500.0
    assert hi - lo == 20
