"""GPU parity of the rejection/integration kernel against the oracle.

Bar: rejection and coverage maps bit-exact; master and weight maps within one
float32 ulp of the reference CPU output (the CPU sums in float64, the kernel
in float-float; both round once to float32).  Golden vectors come from the
reference's own code (tests/golden/make_golden.py).
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import integration as oint

pytestmark = pytest.mark.gpu

MODES = {"none": 0, "sigma_clip": 1, "winsorized_sigma": 2, "linear_fit": 3}


def _variants(golden):
    out = []
    for spec in golden["_variants"]:
        rej, lo, hi, ms, mf = str(spec).split("|")
        out.append((rej, float(lo), float(hi), int(ms), float(mf)))
    return out


def _stack_from(native, stack):
    n, h, w = stack.shape
    s = native.ResidentCalibratedStack(n, h, w)
    for i in range(n):
        s.upload_calibrated_frame(i, stack[i])
    return s


def assert_within_ulp(actual, expected, ulps=1, what=""):
    actual = np.asarray(actual, np.float32)
    expected = np.asarray(expected, np.float32)
    assert actual.shape == expected.shape
    both_nan = np.isnan(actual) & np.isnan(expected)
    diff = np.abs(actual.astype(np.float64) - expected.astype(np.float64))
    tol = ulps * np.spacing(np.maximum(np.abs(expected), np.abs(actual)).astype(np.float32)).astype(np.float64)
    bad = ~both_nan & (diff > tol)
    assert not bad.any(), f"{what}: {bad.sum()} pixels beyond {ulps} ulp, max diff {diff[bad].max()}"


def test_integration_matches_reference_golden(native, golden_integration):
    g = golden_integration
    variants = _variants(g)
    checked = 0
    for name in [str(n) for n in g["_names"]]:
        stack = g[f"{name}/stack"]
        weights = g[f"{name}/weights"] if f"{name}/weights" in g.files else None
        s = _stack_from(native, stack)
        for vi, (rej, lo, hi, ms, mf) in enumerate(variants):
            s.integrate_async(weights, MODES[rej], lo, hi, ms, mf, count_map_dtype="float32")
            master, weight, cov, low, high, dq = s.download_maps("full")
            tag = f"{name} v{vi} {rej}"
            np.testing.assert_array_equal(cov, g[f"{name}/v{vi}/coverage"], err_msg=tag + " coverage")
            np.testing.assert_array_equal(low, g[f"{name}/v{vi}/low"], err_msg=tag + " low")
            np.testing.assert_array_equal(high, g[f"{name}/v{vi}/high"], err_msg=tag + " high")
            assert_within_ulp(weight, g[f"{name}/v{vi}/weight"], 1, tag + " weight")
            assert_within_ulp(master, g[f"{name}/v{vi}/master"], 1, tag + " master")
            expected_dq = oint.dq_map(master, weight, cov, low, high)
            np.testing.assert_array_equal(dq, expected_dq, err_msg=tag + " dq")
            checked += 1
        s.close()
    assert checked > 300


def test_integration_uint16_count_maps_and_download_modes(native):
    rng = np.random.default_rng(3)
    stack = (500 + 10 * rng.standard_normal((9, 33, 47))).astype(np.float32)
    stack[2, 5, 5] = 9000.0
    s = _stack_from(native, stack)
    m, w, c, lo, hi = s.integrate_hardened_winsorized_sigma(None, 3.0, 3.0, 3, 0.5, "uint16")
    assert c.dtype == np.uint16 and lo.dtype == np.uint16 and hi.dtype == np.uint16
    em, ew, ec, el, eh = oint.weighted_integrate_stack(stack, None, "winsorized_sigma")
    np.testing.assert_array_equal(c.astype(np.float32), ec)
    np.testing.assert_array_equal(hi.astype(np.float32), eh)
    assert hi[5, 5] == 1
    m2, w2, c2, l2, h2 = s.integrate_hardened_winsorized_sigma(download_mode="master_only")
    assert w2 is None and c2 is None
    np.testing.assert_array_equal(m2, m)
    master, weight = s.integrate_mean()
    mm, mw, *_ = oint.weighted_integrate_stack(stack)
    assert_within_ulp(master, mm, 1, "mean")
    np.testing.assert_array_equal(weight, mw)


def test_integration_odd_shapes_and_single_frame(native):
    rng = np.random.default_rng(11)
    for n, h, w in ((1, 1, 1), (2, 3, 3), (3, 1, 129), (5, 127, 1), (70, 5, 7), (129, 3, 11)):
        stack = (100 + rng.standard_normal((n, h, w))).astype(np.float32)
        stack[rng.random(stack.shape) < 0.1] = np.nan
        s = _stack_from(native, stack)
        for rej in ("sigma_clip", "winsorized_sigma", "none"):
            s.integrate_async(None, MODES[rej], 2.5, 2.5, 2, 0.4, count_map_dtype="float32")
            master, weight, cov, low, high, _ = s.download_maps("full")
            em, ew, ec, el, eh = oint.weighted_integrate_stack(stack, None, rej, 2.5, 2.5, 2, 0.4)
            tag = f"{n}x{h}x{w} {rej}"
            np.testing.assert_array_equal(cov, ec, err_msg=tag)
            np.testing.assert_array_equal(low, el, err_msg=tag)
            np.testing.assert_array_equal(high, eh, err_msg=tag)
            assert_within_ulp(master, em, 1, tag)
        s.close()


@pytest.mark.parametrize("n", [33, 64, 100, 200, 257, 512])
def test_integration_large_stacks_warp_per_pixel(native, n):
    """32 < N <= 512 runs one warp per pixel (warp-wide sort, float-float sums
    combined across lanes): same bar as the column kernels, for the all-valid
    and the partly-valid formula families, unit and non-unit weights."""
    rng = np.random.default_rng(100 + n)
    h, w = 7, 37  # 259 pixels: a partial last tile of 32
    base = (800 + 12 * rng.standard_normal((n, h, w))).astype(np.float32)
    base[rng.random(base.shape) < 0.03] += 5000.0  # outliers to reject
    holes = base.copy()
    holes[rng.random(base.shape) < 0.05] = np.nan
    holes[:, 0, 0] = np.nan  # a pixel without samples
    weights = rng.uniform(0.5, 2.0, n).astype(np.float32)
    weights[3] = 0.0  # an excluded frame
    for tag, stack in (("all-valid", base), ("holes", holes)):
        s = _stack_from(native, stack)
        for wv in (None, weights):
            for rej in ("winsorized_sigma", "sigma_clip", "none"):
                s.integrate_async(wv, MODES[rej], 3.0, 3.0, 3, 0.5, count_map_dtype="float32")
                master, weight, cov, low, high, _ = s.download_maps("full")
                em, ew, ec, el, eh = oint.weighted_integrate_stack(stack, wv, rej, 3.0, 3.0, 3, 0.5)
                what = f"n={n} {tag} {'weights' if wv is not None else 'unit'} {rej}"
                np.testing.assert_array_equal(cov, ec, err_msg=what)
                np.testing.assert_array_equal(low, el, err_msg=what)
                np.testing.assert_array_equal(high, eh, err_msg=what)
                assert_within_ulp(weight, ew, 1, what + " weight")
                assert_within_ulp(master, em, 1, what + " master")
        s.close()


def test_linear_fit_clip_against_fp64_definition(native):
    rng = np.random.default_rng(5)
    n, h, w = 25, 6, 9
    stack = (1000 + 15 * rng.standard_normal((n, h, w))).astype(np.float32)
    stack[rng.random(stack.shape) < 0.08] += 4000.0
    s = _stack_from(native, stack)
    master, weight, cov, low, high = s.integrate_linear_fit_clip(None, 3.0, 3.0, 3, 0.5, 5)
    em, ew, ec, el, eh = oint.weighted_integrate_stack(stack, None, "linear_fit", 3.0, 3.0, 3, 0.5)
    # Masks follow the float64 definition except where a sample sits within
    # float32 rounding of a threshold (none expected for this seed).
    np.testing.assert_array_equal(low, el)
    np.testing.assert_array_equal(high, eh)
    np.testing.assert_allclose(master, em, rtol=2e-6)


def test_integration_errors_map_to_reference_exceptions(native):
    s = native.ResidentCalibratedStack(3, 4, 5)
    s.upload_calibrated_frame(0, np.zeros((4, 5), np.float32))
    with pytest.raises(RuntimeError, match="loaded"):
        s.integrate_hardened_winsorized_sigma()
    s.upload_calibrated_frame(1, np.zeros((4, 5), np.float32))
    s.upload_calibrated_frame(2, np.zeros((4, 5), np.float32))
    with pytest.raises(ValueError):
        s.integrate_hardened_winsorized_sigma(min_samples=0)
    with pytest.raises(ValueError):
        s.integrate_hardened_winsorized_sigma(count_map_dtype="int8")
    with pytest.raises(ValueError):
        s.integrate_hardened_winsorized_sigma(weights=np.ones(4))
    with pytest.raises(IndexError):
        s.upload_calibrated_frame(3, np.zeros((4, 5), np.float32))
    with pytest.raises(ValueError):
        s.upload_calibrated_frame(0, np.zeros((5, 4), np.float32))


def test_frame_global_stats_match_float64(native):
    rng = np.random.default_rng(9)
    stack = (800 + 30 * rng.standard_normal((3, 64, 80))).astype(np.float32)
    stack[1, :3, :3] = np.nan
    s = _stack_from(native, stack)
    for i in range(3):
        st = s.frame_global_stats(i)
        v = stack[i][np.isfinite(stack[i])].astype(np.float64)
        assert st["valid_pixels"] == v.size
        assert st["nonfinite_pixels"] == stack[i].size - v.size
        np.testing.assert_allclose(st["mean"], v.mean(), rtol=1e-12)
        np.testing.assert_allclose(st["std"], v.std(), rtol=1e-7)
