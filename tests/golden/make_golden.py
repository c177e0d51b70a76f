"""Generates the golden vectors in tests/golden/ by running the reference.

Run in a checkout where the GLASS reference sources are available:

    python tests/golden/make_golden.py --reference /path/to/GLASS

It imports the reference's own CPU implementation (src/glass/cpu/*,
src/glass/engine/rejection.py, src/glass_cuda.py NumPy fallbacks) and, for the
warp test oracles that live in tests/test_gpu_warp_vs_cpu.py and
src/glass/engine/warp.py (modules that import astropy at top level), it
compiles just the needed function definitions out of those files.  Inputs are
seeded synthetic arrays; the outputs are stored next to them in .npz files.
Nothing at test time reads the reference: the fixtures are committed.
"""

from __future__ import annotations

import argparse
import ast
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _load_functions(path: Path, names: list[str], namespace: dict) -> dict:
    """Executes only the named top-level function definitions of a file."""
    tree = ast.parse(path.read_text(), filename=str(path))
    keep = [node for node in tree.body if isinstance(node, ast.FunctionDef) and node.name in names]
    missing = set(names) - {node.name for node in keep}
    if missing:
        raise RuntimeError(f"{path}: missing {sorted(missing)}")
    module = ast.Module(body=keep, type_ignores=[])
    exec(compile(module, str(path), "exec"), namespace)
    return namespace


# ---------------------------------------------------------------------------
# integration
# ---------------------------------------------------------------------------
def _integration_cases(rng: np.random.Generator):
    """(name, stack, weights) inputs covering the reference's edge cases."""
    cases = []
    h, w = 12, 10

    def sky(n, hh=h, ww=w, level=1000.0, noise=20.0):
        return (level + noise * rng.standard_normal((n, hh, ww))).astype(np.float32)

    for n in (1, 2, 3, 4, 5, 7, 8, 13, 16, 31, 32, 33, 64, 65, 100, 200, 260):
        stack = sky(n)
        # cosmic rays / satellite hits and cold outliers
        hits = rng.random(stack.shape) < 0.04
        stack[hits] += rng.uniform(500.0, 30000.0, size=int(hits.sum())).astype(np.float32)
        cold = rng.random(stack.shape) < 0.01
        stack[cold] -= rng.uniform(200.0, 900.0, size=int(cold.sum())).astype(np.float32)
        cases.append((f"allvalid_n{n}", stack, None))
        weights = rng.uniform(0.2, 3.0, size=n).astype(np.float32)
        cases.append((f"weighted_n{n}", stack.copy(), weights))
        masked = stack.copy()
        nan = rng.random(masked.shape) < 0.15
        masked[nan] = np.nan
        cases.append((f"nan_n{n}", masked, None))
        if n >= 3:
            w2 = weights.copy()
            w2[0] = 0.0
            w2[-1] = np.nan
            if n >= 4:
                w2[1] = -1.0
            cases.append((f"badweights_n{n}", masked.copy(), w2))
    # integer-valued data with many ties: IQR collapses -> std fallback
    for n in (4, 9, 20, 40):
        ties = rng.integers(0, 3, size=(n, h, w)).astype(np.float32) + 100.0
        ties[:, 0, 0] = 7.0  # constant column: scale 0 everywhere
        cases.append((f"ties_n{n}", ties, None))
        t2 = ties.copy()
        t2[rng.random(t2.shape) < 0.1] = np.nan
        cases.append((f"ties_nan_n{n}", t2, None))
    # columns with 0, 1, 2 valid samples
    sparse = sky(6)
    sparse[:, 0, :] = np.nan
    sparse[1:, 1, :] = np.nan
    sparse[2:, 2, :] = np.nan
    cases.append(("sparse_n6", sparse, None))
    # bias-level data around zero (mixed signs, large exponent span)
    zero = (3.0 * rng.standard_normal((24, h, w))).astype(np.float32)
    zero[rng.random(zero.shape) < 0.05] *= 1000.0
    cases.append(("nearzero_n24", zero, None))
    # star cores: large values, large spread
    star = (20000.0 + 3000.0 * rng.standard_normal((17, h, w))).astype(np.float32)
    cases.append(("bright_n17", star, rng.uniform(0.5, 2.0, 17).astype(np.float32)))
    return cases


def make_integration(ref_src: Path) -> None:
    sys.path.insert(0, str(ref_src))
    from glass.cpu.integration import weighted_integrate_stack  # noqa: E402

    rng = np.random.default_rng(20240531)
    arrays: dict[str, np.ndarray] = {}
    names = []
    variants = [
        ("none", 3.0, 3.0, 3, 0.5),
        ("sigma_clip", 3.0, 3.0, 3, 0.5),
        ("winsorized_sigma", 3.0, 3.0, 3, 0.5),
        ("winsorized_sigma", 2.0, 1.5, 2, 0.3),
        ("sigma_clip", 1.5, 2.5, 1, 1.0),
    ]
    for name, stack, weights in _integration_cases(rng):
        names.append(name)
        arrays[f"{name}/stack"] = stack
        if weights is not None:
            arrays[f"{name}/weights"] = weights
        for vi, (rej, lo, hi, ms, mf) in enumerate(variants):
            out = weighted_integrate_stack(stack, weights=weights, rejection=rej, low_sigma=lo, high_sigma=hi,
                                           min_samples=ms, max_reject_fraction=mf)
            for key, value in zip(("master", "weight", "coverage", "low", "high"), out):
                arrays[f"{name}/v{vi}/{key}"] = np.asarray(value)
    arrays["_names"] = np.asarray(names)
    arrays["_variants"] = np.asarray([f"{r}|{lo}|{hi}|{ms}|{mf}" for r, lo, hi, ms, mf in variants])
    np.savez_compressed(HERE / "integration.npz", **arrays)


# ---------------------------------------------------------------------------
# calibration
# ---------------------------------------------------------------------------
def make_calibration(ref_src: Path) -> None:
    sys.path.insert(0, str(ref_src))
    from glass.cpu.calibration import calibrate_light  # noqa: E402
    from glass.models import CalibrationPolicy  # noqa: E402

    rng = np.random.default_rng(7)
    h, w = 24, 36
    light = rng.integers(0, 65536, size=(h, w)).astype(np.uint16)
    bias = (300.0 + 5.0 * rng.standard_normal((h, w))).astype(np.float32)
    dark = (320.0 + 9.0 * rng.standard_normal((h, w))).astype(np.float32)
    flat = rng.uniform(0.85, 1.1, size=(h, w)).astype(np.float32)
    flat[0, :4] = [0.0, -1.0, 1e-9, np.nan]
    arrays = {"light": light, "bias": bias, "dark": dark, "flat": flat}
    policies = [
        dict(),
        dict(master_dark_includes_bias=False),
        dict(dark_scaling_enabled=False),
        dict(pedestal=500.0),
        dict(flat_floor=0.9),
        dict(master_dark_includes_bias=False, pedestal=123.25, flat_floor=0.5),
    ]
    combos = [(True, True, True), (True, False, True), (False, True, True), (True, True, False),
              (False, False, True), (True, False, False), (False, False, False)]
    exposures = [(300.0, 600.0), (120.0, 120.0), (60.0, None), (45.0, 0.0), (100.0, 30.0)]
    specs = []
    k = 0
    for pi, policy in enumerate(policies):
        for ci, (ub, ud, uf) in enumerate(combos):
            for ei, (tl, td) in enumerate(exposures):
                if (pi + ci + ei) % 3:
                    continue
                out = calibrate_light(light.astype(np.float32), bias if ub else None, dark if ud else None,
                                      flat if uf else None, tl, td, CalibrationPolicy(**policy))
                arrays[f"case{k}/out"] = out
                specs.append({"policy": policy, "bias": ub, "dark": ud, "flat": uf, "t_light": tl, "t_dark": td})
                k += 1
    arrays["_specs"] = np.asarray([repr(s) for s in specs])
    np.savez_compressed(HERE / "calibration.npz", **arrays)


def main() -> int:
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("--reference", default="/root/reference", help="GLASS reference checkout")
    parser.add_argument("--only", default="", help="comma-separated subset")
    args = parser.parse_args()
    ref = Path(args.reference)
    src = ref / "src"
    jobs = {"integration": make_integration, "calibration": make_calibration}
    only = [j for j in args.only.split(",") if j] or list(jobs)
    for job in only:
        jobs[job](src)
        print(f"wrote {job}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
