"""Records the native calls the reference's `glass_cuda` facade makes for a
resident run, as a replayable fixture (tests/golden/facade_trace.npz).

Run where the GLASS reference sources are available:

    python tests/golden/make_facade_trace.py --reference /path/to/GLASS

The reference facade (src/glass_cuda.py) is imported unchanged with a
recording stand-in registered as `_glass_cuda_native`.  The stand-in exposes
exactly the public names of this project's drop-in module
(glass_gb300._glass_cuda_native), so the facade's hasattr() feature gates see
what they would see over the real library; every call is logged with its
arguments (arrays stored in the fixture) and answered with a placeholder of the
right type.  The scenario follows the resident run's order
(src/glass/engine/resident_cuda.py: masters :8542, calibration :8974-9280, frame
statistics :12766-12785, grid catalogs :10914, Lanczos3 warp :12505,
hardened winsorized integration :13435-13443).  tests/test_facade_trace.py
replays the log against the real library on a GPU and checks every result
against the oracle; nothing at test time reads the reference.
"""

from __future__ import annotations

import argparse
import json
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def _placeholder(name: str, stack, args):
    n, h, w = stack._n, stack._h, stack._w
    if name == "frame_global_stats":
        return {"mean": 1.0, "std": 1.0, "valid_pixels": h * w, "total_pixels": h * w, "nonfinite_pixels": 0,
                "model": "recorded"}
    if name.startswith("star_grid_top_nms_candidates_batch"):
        return [{"frame_index": int(i), "count": 0, "stored_count": 0, "grid_cols": 1, "grid_rows": 1,
                 "candidates_per_cell": 1, "max_output_candidates": 1, "min_separation_px": 0.0,
                 "x": np.zeros(0, np.float32), "y": np.zeros(0, np.float32), "flux": np.zeros(0, np.float32)}
                for i in args[0]]
    if name.startswith("apply_matrix"):
        return {"frames": len(args[0])}
    if name.startswith("integrate_hardened_winsorized_sigma"):
        maps = (np.zeros((h, w), np.float32), np.zeros((h, w), np.float32), np.zeros((h, w), np.uint16),
                np.zeros((h, w), np.uint16), np.zeros((h, w), np.uint16))
        profile = args[6] if len(args) > 6 else False
        return maps + ({"enqueue_s": 0.0},) if profile else maps
    return None


def recording_module(shim_module, log: list, arrays: dict):
    """A stand-in for `_glass_cuda_native` with the shim's public names."""

    def encode(value):
        if isinstance(value, np.ndarray):
            key = f"a{len(arrays)}"
            arrays[key] = np.ascontiguousarray(value)
            return {"array": key}
        if isinstance(value, (list, tuple)):
            return {"list": [encode(v) for v in value]}
        if isinstance(value, dict):
            return {"dict": {k: encode(v) for k, v in value.items()}}
        if isinstance(value, (np.floating, float)):
            return {"float": float(value)} if np.isfinite(value) else {"float_str": repr(float(value))}
        if isinstance(value, (np.integer, int, bool, str)) or value is None:
            return {"value": value.item() if isinstance(value, np.generic) else value}
        raise TypeError(f"cannot record {type(value)}")

    shim_cls = shim_module.ResidentCalibratedStack

    class RecordingStack:
        def __init__(self, frame_count, height, width):
            self._n, self._h, self._w = int(frame_count), int(height), int(width)
            log.append({"call": "ResidentCalibratedStack", "args": [encode(frame_count), encode(height),
                                                                    encode(width)], "kwargs": {}})

        frame_count = property(lambda self: self._n)
        height = property(lambda self: self._h)
        width = property(lambda self: self._w)
        pixels_per_frame = property(lambda self: self._h * self._w)

    def method(name):
        def record(self, *args, **kwargs):
            log.append({"call": name, "args": [encode(a) for a in args],
                        "kwargs": {k: encode(v) for k, v in kwargs.items()}})
            return _placeholder(name, self, args)
        return record

    for name in dir(shim_cls):
        if name.startswith("_") or hasattr(RecordingStack, name):
            continue
        attr = getattr(shim_cls, name)
        if isinstance(attr, property):
            setattr(RecordingStack, name, property(lambda self: 0))
        elif callable(attr):
            setattr(RecordingStack, name, method(name))
    module = types.ModuleType("_glass_cuda_native")
    for name in dir(shim_module):
        if not name.startswith("_") and callable(getattr(shim_module, name)):
            setattr(module, name, lambda *a, **k: None)
    module.ResidentCalibratedStack = RecordingStack
    module.cuda_available = lambda: True
    return module


def scenario(glass_cuda, rng):
    """A small resident run through the facade (frames with stars, cosmic
    rays and one NaN patch; masters; a similarity per frame)."""
    n, h, w = 6, 96, 128
    bias = (500.0 + rng.normal(0, 2, (h, w))).astype(np.float32)
    dark = rng.uniform(5.0, 7.0, (h, w)).astype(np.float32)
    flat = rng.uniform(0.9, 1.05, (h, w)).astype(np.float32)
    yy, xx = np.mgrid[0:h, 0:w]
    stars = [(rng.uniform(5, w - 6), rng.uniform(5, h - 6), rng.uniform(800, 6000)) for _ in range(25)]
    lights = []
    mats = []
    for k in range(n):
        t = np.deg2rad(rng.uniform(-0.4, 0.4)) if k else 0.0
        dx, dy = (rng.uniform(-3, 3), rng.uniform(-3, 3)) if k else (0.0, 0.0)
        m = np.array([[np.cos(t), -np.sin(t), dx], [np.sin(t), np.cos(t), dy], [0, 0, 1.0]])
        inv = np.linalg.inv(m)
        img = np.full((h, w), 1000.0, np.float64)
        for sx, sy, f in stars:
            px, py = inv[0, 0] * sx + inv[0, 1] * sy + inv[0, 2], inv[1, 0] * sx + inv[1, 1] * sy + inv[1, 2]
            img += f * np.exp(-((xx - px) ** 2 + (yy - py) ** 2) / (2 * 1.4 ** 2))
        img = rng.poisson(img * flat) + bias + dark
        img[rng.random((h, w)) < 0.002] += 20000.0
        if k == 3:
            img[40:44, 60:66] = np.nan
        lights.append(img.astype(np.float32))
        mats.append(m)
    stack = glass_cuda.ResidentCalibratedStack(n, h, w)
    stack.set_calibration_masters(bias, dark, flat)
    policy = {"master_dark_includes_bias": False, "dark_scaling_enabled": True, "flat_floor": 1.0e-6,
              "pedestal": 0.0}
    for k in range(n):
        stack.calibrate_frame(k, lights[k], 300.0, 300.0, policy)
    weights = [stack.frame_global_stats(k) for k in range(n)]
    stack.star_grid_top_nms_candidates_batch_deterministic_centroid(list(range(1, n)), 1500.0, 4, 3, 8, 40, 4.0, 3,
                                                                    "local_median")
    stack.apply_matrix_lanczos3_frames(np.arange(1, n, dtype=np.int64), np.asarray(mats[1:], np.float32), np.nan,
                                       -1.0)
    stack.integrate_hardened_winsorized_sigma_timed(np.linspace(0.5, 1.5, n).astype(np.float32), 3.0, 3.0,
                                                    min_samples=3, max_reject_fraction=0.5,
                                                    count_map_dtype="uint16", download_mode="full")
    return weights


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--reference", required=True, type=Path)
    args = ap.parse_args()
    sys.path.insert(0, str(REPO))
    sys.path.insert(0, str(args.reference / "src"))
    from glass_gb300 import _glass_cuda_native as shim

    log: list = []
    arrays: dict = {}
    sys.modules["_glass_cuda_native"] = recording_module(shim, log, arrays)
    import glass_cuda

    scenario(glass_cuda, np.random.default_rng(4242))
    arrays["calls"] = np.frombuffer(json.dumps(log).encode(), dtype=np.uint8)
    np.savez_compressed(HERE / "facade_trace.npz", **arrays)
    print(f"recorded {len(log)} native calls: {[c['call'] for c in log]}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
