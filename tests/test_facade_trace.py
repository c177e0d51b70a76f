"""The drop-in boundary as the reference's own facade drives it.

tests/golden/facade_trace.npz holds the native calls the reference's
`glass_cuda` facade (src/glass_cuda.py, unchanged) makes for a small resident
run - masters, per-frame calibration, frame statistics, the batch grid
catalog, the Lanczos3 warp and the hardened winsorized integration - recorded
by tests/golden/make_facade_trace.py over a stand-in with this module's public
names.  Here every recorded call must bind to the drop-in module's signature
(CPU), and replayed against the real library it must produce the oracle's
results (GPU): calibration bit-exact, statistics to 1e-12, catalog counts,
order and values exact with centroids within 1 ulp, warp within the Lanczos3
bar, integration counts exact and maps within 1 ulp.
"""

from __future__ import annotations

import inspect
import json
import sys
from pathlib import Path

import numpy as np
import pytest

from glass_gb300 import _glass_cuda_native as shim

TRACE = Path(__file__).resolve().parent / "golden" / "facade_trace.npz"
REFERENCE_SRC = Path("/root/reference/src")


def _load():
    z = np.load(TRACE)
    calls = json.loads(bytes(z["calls"]).decode())
    arrays = {k: z[k] for k in z.files if k != "calls"}

    def decode(v):
        if "array" in v:
            return arrays[v["array"]]
        if "list" in v:
            return [decode(x) for x in v["list"]]
        if "dict" in v:
            return {k: decode(x) for k, x in v["dict"].items()}
        if "float" in v:
            return v["float"]
        if "float_str" in v:
            return float(v["float_str"])
        return v["value"]

    return [(c["call"], [decode(a) for a in c["args"]], {k: decode(x) for k, x in c["kwargs"].items()})
            for c in calls]


def test_every_recorded_call_binds_to_the_drop_in():
    calls = _load()
    assert calls[0][0] == "ResidentCalibratedStack"
    for name, args, kwargs in calls[1:]:
        method = getattr(shim.ResidentCalibratedStack, name, None)
        assert method is not None, f"drop-in lacks ResidentCalibratedStack.{name}"
        inspect.signature(method).bind(None, *args, **kwargs)
    inspect.signature(shim.ResidentCalibratedStack).bind(*calls[0][1])


@pytest.mark.skipif(not REFERENCE_SRC.exists(), reason="reference sources not present")
def test_resident_feature_gates_pass_over_the_drop_in():
    """The resident engine's gate for the hardened winsorized path
    (resident_cuda.py:4167-4176) and its batch-catalog gate
    (resident_cuda.py:10527-10610) see the methods they need."""
    import ast

    import glass_gb300

    glass_gb300.install_drop_in()
    sys.path.insert(0, str(REFERENCE_SRC))
    try:
        import glass_cuda

        path = REFERENCE_SRC / "glass" / "engine" / "resident_cuda.py"
        tree = ast.parse(path.read_text())
        keep = [n for n in tree.body if isinstance(n, ast.FunctionDef)
                and n.name == "_resident_stack_hardened_winsorized_available"]
        ns: dict = {"Any": object}
        exec(compile(ast.Module(body=keep, type_ignores=[]), str(path), "exec"), ns)
        assert ns["_resident_stack_hardened_winsorized_available"](glass_cuda) == (True, None)
        for name in ("star_grid_top_nms_candidates_batch_deterministic_centroid",
                     "star_grid_top_nms_candidates_batch_centroid", "star_grid_top_nms_candidates_batch",
                     "star_grid_top_nms_candidates_deterministic_centroid", "frame_global_stats",
                     "integrate_hardened_winsorized_sigma", "apply_matrix_lanczos3_frames"):
            assert hasattr(glass_cuda._native().ResidentCalibratedStack, name), name
    finally:
        sys.path.remove(str(REFERENCE_SRC))


@pytest.mark.gpu
def test_replayed_facade_calls_match_the_oracle(native):
    from oracle.calibration import calibrate_light
    from oracle.catalog import grid_catalog
    from oracle.integration import weighted_integrate_stack
    from oracle.warp import warp_matrix

    calls = _load()
    stack = native.ResidentCalibratedStack(*calls[0][1])
    masters = None
    lights = {}
    checked = set()
    try:
        for name, args, kwargs in calls[1:]:
            if name == "set_calibration_masters":
                masters = args
            before = None
            if name == "apply_matrix_lanczos3_frames":
                before = {int(k): stack.download_frame(int(k)) for k in args[0]}
            if name == "integrate_hardened_winsorized_sigma":
                frames = np.stack([stack.download_frame(k) for k in range(stack.frame_count)])
            result = getattr(stack, name)(*args, **kwargs)
            if name == "calibrate_frame":
                index, light, t_l, t_d, policy = args
                lights[index] = light
                exp = calibrate_light(light, *masters, t_l, t_d,
                                      master_dark_includes_bias=policy["master_dark_includes_bias"],
                                      dark_scaling_enabled=policy["dark_scaling_enabled"],
                                      flat_floor=policy["flat_floor"], pedestal=policy["pedestal"])
                np.testing.assert_array_equal(stack.download_frame(index), exp)
                checked.add(name)
            elif name == "frame_global_stats":
                frame = stack.download_frame(args[0]).astype(np.float64)
                vals = frame[np.isfinite(frame)]
                assert result["valid_pixels"] == vals.size
                np.testing.assert_allclose(result["mean"], vals.mean(), rtol=1e-12)
                np.testing.assert_allclose(result["std"], vals.std(), rtol=1e-7)
                checked.add(name)
            elif name == "star_grid_top_nms_candidates_batch_deterministic_centroid":
                indices, thr, cols, rows, k, mo, sep, radius, gmean = args
                for got in result:
                    exp = grid_catalog(stack.download_frame(got["frame_index"]), thr, cols, rows, k, mo, sep, radius,
                                       gmean)
                    assert got["count"] == exp["count"] and got["stored_count"] == exp["stored_count"]
                    assert got["stored_count"] > 5
                    np.testing.assert_array_equal(got["flux"], exp["flux"])
                    for key in ("x", "y"):
                        assert np.all(np.abs(got[key] - exp[key]) <= np.spacing(np.maximum(np.abs(exp[key]), 1.0)))
                checked.add(name)
            elif name == "apply_matrix_lanczos3_frames":
                for k, m in zip(args[0], args[1]):
                    exp, cov = warp_matrix(before[int(k)], m, "lanczos3", args[2])
                    got = stack.download_frame(int(k))
                    ok = cov > 0
                    assert np.array_equal(np.isnan(got), np.isnan(exp))
                    scale = float(np.nanmax(np.abs(before[int(k)])))
                    assert np.all(np.abs(got[ok] - exp[ok]) <= 3e-6 * scale + 1e-5 * np.abs(exp[ok]))
                checked.add(name)
            elif name == "integrate_hardened_winsorized_sigma":
                weights, lo, hi, min_samples, max_frac = args[:5]
                master, weight, cov, low, high = result[:5]
                em, ew, ec, el, eh = weighted_integrate_stack(frames, weights, "winsorized_sigma", lo, hi,
                                                              min_samples, max_frac)
                for got, exp in ((cov, ec), (low, el), (high, eh)):
                    np.testing.assert_array_equal(got.astype(np.float32), exp)
                for got, exp in ((master, em), (weight, ew)):
                    fin = np.isfinite(exp)
                    assert np.array_equal(fin, np.isfinite(got))
                    assert np.all(np.abs(got[fin] - exp[fin]) <= np.spacing(np.abs(exp[fin])))
                assert isinstance(result[5], dict)
                checked.add(name)
    finally:
        stack.close()
    assert checked == {"calibrate_frame", "frame_global_stats",
                       "star_grid_top_nms_candidates_batch_deterministic_centroid",
                       "apply_matrix_lanczos3_frames", "integrate_hardened_winsorized_sigma"}
