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


# ---------------------------------------------------------------------------
# warps
# ---------------------------------------------------------------------------
def _similarity(theta_deg: float, dx: float, dy: float, scale: float = 1.0) -> np.ndarray:
    t = np.deg2rad(theta_deg)
    c, s = scale * np.cos(t), scale * np.sin(t)
    return np.array([[c, -s, dx], [s, c, dy], [0.0, 0.0, 1.0]], dtype=np.float32)


def make_warp(ref_src: Path) -> None:
    """Reference warp oracles: the per-pixel CPU functions of
    tests/test_gpu_warp_vs_cpu.py:9-128, the NumPy fallbacks of src/glass_cuda.py
    (warp_translation_f32 :539, warp_matrix_lanczos3_f32 :644) and the tile
    warp of src/glass/engine/warp.py:155-227."""
    sys.path.insert(0, str(ref_src))
    import glass_cuda  # noqa: E402  (NumPy fallbacks when no native module)

    ns: dict = {"np": np}
    _load_functions(ref_src.parent / "tests" / "test_gpu_warp_vs_cpu.py",
                    ["_warp_translation_bilinear_cpu", "_warp_matrix_bilinear_cpu", "_sinc", "_lanczos3_weight",
                     "_warp_matrix_lanczos3_cpu"], ns)
    eng: dict = {"np": np}
    _load_functions(ref_src / "glass" / "engine" / "warp.py",
                    ["_cubic_weight", "_sinc", "_lanczos3_weight", "_sample_nearest", "_sample_bilinear",
                     "_sample_windowed", "_warp_tile_matrix"], eng)
    eng["INTERPOLATOR_KERNEL_RADIUS"] = {"nearest": 0, "bilinear": 1, "bicubic": 2, "lanczos3": 3}

    class Reader:
        def __init__(self, image):
            self.image = image
            self.shape = image.shape

        def read_tile(self, y0, y1, x0, x1):
            return self.image[y0:y1, x0:x1]

    class Tile:
        def __init__(self, h, w):
            self.y0, self.y1, self.x0, self.x1 = 0, h, 0, w

    rng = np.random.default_rng(99)
    arrays: dict[str, np.ndarray] = {}
    cases = []
    # the reference tests' own inputs
    yy, xx = np.indices((12, 13), dtype=np.float32)
    ramp = 0.2 * xx + 0.4 * yy
    ramp[:, 7:] += 5.0
    cases.append(("reftest_bilinear7", np.arange(49, dtype=np.float32).reshape(7, 7), _similarity(3.0, 1.2, -0.4),
                  "bilinear", -1.0, -1.0))
    cases.append(("reftest_lanczos12", ramp, _similarity(1.0, 0.35, -0.25), "lanczos3", -1.0, 0.30))
    cases.append(("reftest_lanczos_sin", (np.sin(xx * 0.3) + np.cos(yy * 0.2)).astype(np.float32),
                  _similarity(0.0, 0.4, -0.35), "lanczos3", np.nan, 0.30))
    for k in range(10):
        h, w = int(rng.integers(9, 40)), int(rng.integers(9, 44))
        img = (1000.0 + 50.0 * rng.standard_normal((h, w))).astype(np.float32)
        img[rng.random((h, w)) < 0.02] += 20000.0
        m = _similarity(float(rng.uniform(-4, 4)), float(rng.uniform(-6, 6)), float(rng.uniform(-6, 6)),
                        float(rng.uniform(0.97, 1.03)))
        for interp in ("bilinear", "lanczos3"):
            clamp = float(rng.choice([-1.0, 0.0, 0.3])) if interp == "lanczos3" else -1.0
            cases.append((f"rand{k}_{interp}", img, m, interp, np.nan, clamp))
        nanimg = img.copy()
        nanimg[rng.random((h, w)) < 0.05] = np.nan
        cases.append((f"rand{k}_lanczos3_nan", nanimg, m, "lanczos3", np.nan, 0.3 if k % 2 else -1.0))
    # projective
    proj = _similarity(2.0, 1.5, -2.0)
    proj[2, 0], proj[2, 1] = 1.0e-4, -2.0e-4
    img = (500.0 + 20.0 * rng.standard_normal((30, 34))).astype(np.float32)
    cases.append(("projective_bilinear", img, proj, "bilinear", np.nan, -1.0))
    cases.append(("projective_lanczos3", img, proj, "lanczos3", np.nan, -1.0))
    names = []
    for name, image, matrix, interp, fill, clamp in cases:
        if interp == "bilinear":
            out, cov = ns["_warp_matrix_bilinear_cpu"](image, matrix, fill)
        else:
            out, cov = ns["_warp_matrix_lanczos3_cpu"](image, matrix, fill, clamp)
        arrays[f"{name}/image"] = image
        arrays[f"{name}/matrix"] = matrix
        arrays[f"{name}/out"] = out
        arrays[f"{name}/coverage"] = cov
        arrays[f"{name}/params"] = np.array([1.0 if interp == "bilinear" else 3.0, fill, clamp])
        if np.all(np.isfinite(image)):
            # engine/warp.py tile warp (no NaN skipping there, so finite inputs only)
            eout, ecov = eng["_warp_tile_matrix"](Reader(image), Tile(*image.shape), matrix.tolist(), fill,
                                                  interp)
            arrays[f"{name}/engine_out"] = eout
            arrays[f"{name}/engine_coverage"] = ecov
        if interp == "lanczos3":
            gout, gcov = glass_cuda.warp_matrix_lanczos3_f32(image, matrix, fill, clamp)
            arrays[f"{name}/fallback_out"] = gout
            arrays[f"{name}/fallback_coverage"] = gcov
        names.append(name)
    # translations (cpu/warp.py via the glass_cuda fallbacks)
    img = np.arange(36, dtype=np.float32).reshape(6, 6)
    for k, (dx, dy) in enumerate([(1, -2), (0.6, 2.5), (-3.4, 0.5), (2.5, -1.5)]):
        out, cov = glass_cuda.warp_translation_f32(img, dx, dy, -1.0)
        arrays[f"translation{k}/out"] = out
        arrays[f"translation{k}/coverage"] = cov
        arrays[f"translation{k}/shift"] = np.array([dx, dy])
        bout, bcov = ns["_warp_translation_bilinear_cpu"](img, dx, dy, -1.0)
        arrays[f"translation{k}/bilinear_out"] = bout
        arrays[f"translation{k}/bilinear_coverage"] = bcov
    arrays["translation_image"] = img
    arrays["_names"] = np.asarray(names)
    np.savez_compressed(HERE / "warp.npz", **arrays)


# ---------------------------------------------------------------------------
# star detection
# ---------------------------------------------------------------------------
STAR_FIELDS = ("x", "y", "flux", "peak", "fwhm_px", "eccentricity", "snr", "sharpness", "npix")


def _star_field(rng, h, w, n, background, noise, fwhm=(2.0, 3.5)):
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.full((h, w), background, dtype=np.float64)
    for _ in range(n):
        x0, y0 = rng.uniform(2, w - 3), rng.uniform(2, h - 3)
        s = rng.uniform(*fwhm) / 2.3548
        img += rng.uniform(200, 20000) * np.exp(-((xx - x0) ** 2 + (yy - y0) ** 2) / (2 * s * s))
    img += noise * rng.standard_normal((h, w))
    return img.astype(np.float32)


def make_stars(ref_src: Path) -> None:
    """detect_stars (src/glass/cpu/star_detect.py:121-168) on seeded fields and
    on the reference tests' own images (tests/test_cpu_star_detect.py:15-38,
    rendered by src/glass/synthetic/generator.py:render_star_field)."""
    sys.path.insert(0, str(ref_src))
    from glass.cpu.star_detect import detect_stars  # noqa: E402

    gen: dict = {"np": np}
    _load_functions(ref_src / "glass" / "synthetic" / "generator.py", ["render_star_field"], gen)
    rng = np.random.default_rng(314)
    cases = []
    stars = np.array([[16.0, 16.0, 1000.0], [8.0, 20.0, 800.0]], dtype=np.float32)
    cases.append(("reftest_two_stars", gen["render_star_field"](32, 32, stars), dict(threshold_sigma=3.0)))
    yy, xx = np.mgrid[0:64, 0:64]
    ell = (1000.0 * np.exp(-(((xx - 32.0) / 2.3) ** 2 + ((yy - 32.0) / 1.0) ** 2) / 2.0)).astype(np.float32)
    cases.append(("reftest_elliptical", ell, dict(threshold_sigma=3.0)))
    for k in range(6):
        h, w = int(rng.integers(40, 120)), int(rng.integers(40, 140))
        img = _star_field(rng, h, w, int(rng.integers(5, 60)), 1000.0, 15.0)
        if k % 2:
            img[rng.random((h, w)) < 0.01] = np.nan
        if k == 2:  # plateau: two equal neighbouring maxima
            img[20, 20] = img[20, 21] = 30000.0
        if k == 3:  # close pair (de-duplication)
            img[30, 30] = 25000.0
            img[31, 32] = 24000.0
        params = dict(threshold_sigma=float(rng.choice([3.0, 5.0])), max_stars=int(rng.choice([5, 20, 500])))
        cases.append((f"field{k}", img, params))
    cases.append(("field_big", _star_field(rng, 256, 256, 300, 800.0, 10.0), dict(threshold_sigma=5.0)))
    cases.append(("field_given_bg", _star_field(rng, 64, 64, 10, 500.0, 8.0),
                  dict(threshold_sigma=4.0, background=480.25, noise=9.5)))
    cases.append(("field_window2_sep5", _star_field(rng, 80, 90, 40, 1200.0, 20.0),
                  dict(threshold_sigma=3.0, window_radius=2, min_separation_px=5.0)))
    flat = np.full((20, 24), 7.0, dtype=np.float32)
    flat[10, 12] = 50.0
    cases.append(("constant_background", flat, dict(threshold_sigma=3.0)))
    arrays: dict[str, np.ndarray] = {}
    names = []
    for name, img, params in cases:
        found = detect_stars(img, **params)
        arrays[f"{name}/image"] = img
        arrays[f"{name}/params"] = np.asarray(repr(params))
        for field in STAR_FIELDS:
            vals = [getattr(s, field) for s in found]
            arrays[f"{name}/{field}"] = np.asarray([np.nan if v is None else v for v in vals], dtype=np.float64)
        names.append(name)
    arrays["_names"] = np.asarray(names)
    np.savez_compressed(HERE / "stars.npz", **arrays)


# ---------------------------------------------------------------------------
# registration
# ---------------------------------------------------------------------------
def _similar_catalog(rng, n, theta_deg, scale, dx, dy, noise, extent=2000.0, drop=0, add=0, swap=0):
    """Reference catalog (n, 2) and a moving catalog that the similarity
    (theta, scale, dx, dy) maps back onto it, with centroid noise, dropped and
    spurious stars and a perturbed brightness order."""
    ref = rng.uniform(20.0, extent - 20.0, size=(n, 2))
    t = np.deg2rad(theta_deg)
    lin = scale * np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
    mov = (ref - np.array([dx, dy])) @ np.linalg.inv(lin).T + noise * rng.standard_normal((n, 2))
    keep = np.sort(rng.permutation(n)[: n - drop])
    mov = mov[keep]
    if add:
        mov = np.vstack([mov, rng.uniform(0.0, extent, size=(add, 2))])
    order = np.arange(len(mov))
    for _ in range(swap):  # neighbouring brightness swaps
        i = int(rng.integers(0, len(mov) - 1))
        order[i], order[i + 1] = order[i + 1], order[i]
    return ref, mov[order]


def make_registration(ref_src: Path) -> None:
    """estimate_triangle_asterism_transform and _local_triangle_descriptors
    (src/glass/cpu/registration.py:273-475) on seeded catalogs and on the
    reference tests' own cases (tests/test_cpu_registration.py:114-149,
    206-235), plus the descriptor-list similarity fallback of
    src/glass_cuda.py:2054-2140."""
    sys.path.insert(0, str(ref_src))
    from glass.cpu.registration import _local_triangle_descriptors, estimate_triangle_asterism_transform
    from glass.cpu.star_detect import Star, detect_stars
    import glass_cuda

    rng = np.random.default_rng(2718)
    cases = []
    # reftest: 8 points, similarity (-7 deg, 0.98, (-4, 3)) plus one outlier
    pts = np.array([(10, 10), (20, 10), (10, 25), (30, 30), (5, 35), (35, 5), (25, 18), (14, 32)], dtype=np.float64)
    ang = np.deg2rad(-7.0)
    lin = 0.98 * np.array([[np.cos(ang), -np.sin(ang)], [np.sin(ang), np.cos(ang)]])
    mov = np.vstack([(pts - np.array([-4.0, 3.0])) @ np.linalg.inv(lin).T, [[100.0, 100.0]]])
    cases.append(("reftest_outlier", pts, mov, dict(min_inliers=8, tolerance_px=0.5, neighbors=5,
                                                     descriptor_radius=0.1)))
    # reftest: detected star field shifted by (4, -3)
    shape = (96, 112)
    field = np.full(shape, 10.0, dtype=np.float32)
    yy, xx = np.indices(shape, dtype=np.float32)
    for x, y, flux in [(12, 17, 100.0), (30, 42, 220.0), (71, 15, 160.0), (88, 63, 180.0), (45, 79, 250.0),
                       (19, 86, 130.0), (101, 33, 145.0), (53, 55, 190.0)]:
        field += flux * np.exp(-(((xx - x) ** 2 + (yy - y) ** 2) / (2.0 * 1.4 ** 2)))
    field = field.astype(np.float32)
    shifted = np.zeros_like(field)
    shifted[0:93, 4:112] = field[3:96, 0:108]
    rs = detect_stars(field, threshold_sigma=3, max_stars=50)
    ms = detect_stars(shifted, threshold_sigma=3, max_stars=50)
    cases.append(("reftest_star_field", np.array([(s.x, s.y) for s in rs]), np.array([(s.x, s.y) for s in ms]),
                  dict(min_inliers=6, tolerance_px=0.5, neighbors=5, descriptor_radius=0.1)))
    # seeded catalogs
    specs = [
        (80, 0.3, 1.0, 12.5, -7.25, 0.05, 0, 0, 0, {}),
        (80, -2.0, 1.01, -40.0, 33.0, 0.1, 5, 5, 6, {}),
        (60, 4.5, 0.99, 3.0, 150.0, 0.2, 8, 10, 10, dict(tolerance_px=2.0)),
        (40, 0.0, 1.0, 0.5, 0.25, 0.0, 0, 0, 0, dict(neighbors=4)),
        (80, 1.0, 1.0, -5.0, 5.0, 0.05, 0, 0, 0, dict(neighbors=6, max_candidates=200)),
        (80, -0.7, 1.0, 8.0, -2.0, 0.05, 2, 3, 4, dict(max_descriptors=100, max_candidates=50)),
        (50, 10.0, 1.05, 100.0, -80.0, 0.1, 0, 0, 0, dict(max_stars=30)),
        (25, 0.2, 1.0, 1.0, 1.0, 0.05, 10, 12, 0, dict(min_inliers=10)),
        (12, 0.0, 1.0, 2.0, 3.0, 0.0, 0, 0, 0, dict(tolerance_px=1.0)),
        (80, 180.0, 1.0, 2000.0, 2000.0, 0.05, 0, 0, 0, {}),
        (80, 0.5, 1.0, 3.0, 4.0, 0.05, 0, 0, 0, dict(descriptor_radius=0.02)),
        (80, 0.5, 1.0, 3.0, 4.0, 0.05, 0, 0, 0, dict(descriptor_radius=0.0)),
    ]
    for k, (n, th, sc, dx, dy, noise, drop, add, swap, params) in enumerate(specs):
        ref, mov = _similar_catalog(rng, n, th, sc, dx, dy, noise, drop=drop, add=add, swap=swap)
        cases.append((f"seeded{k}", ref, mov, params))
    # dense field: many point pairs inside the tolerance
    ref, mov = _similar_catalog(rng, 80, 0.1, 1.0, 1.0, 1.0, 0.3, extent=120.0)
    cases.append(("dense", ref, mov, dict(tolerance_px=3.0)))
    # mirrored moving catalog: the SVD reflection branch
    ref = rng.uniform(0.0, 500.0, size=(30, 2))
    cases.append(("mirrored", ref, ref * np.array([-1.0, 1.0]) + 600.0, {}))
    # regular grid: identical descriptors, ties everywhere
    g = np.stack(np.meshgrid(np.arange(8) * 25.0 + 10.0, np.arange(8) * 25.0 + 10.0), -1).reshape(-1, 2)
    cases.append(("grid", g, g + np.array([3.0, -2.0]), dict(max_candidates=300)))
    # degenerate inputs
    line = np.column_stack([np.arange(10) * 7.0, np.arange(10) * 3.0])
    cases.append(("collinear", line, line + 1.0, {}))
    cases.append(("two_stars", np.array([[1.0, 2.0], [30.0, 40.0]]), np.array([[2.0, 2.0], [31.0, 40.0]]), {}))
    cases.append(("empty_moving", rng.uniform(0, 100, (10, 2)), np.zeros((0, 2)), {}))
    cases.append(("duplicates", np.repeat(rng.uniform(0, 300, (6, 2)), 2, axis=0),
                  np.repeat(rng.uniform(0, 300, (6, 2)), 2, axis=0), {}))

    arrays: dict[str, np.ndarray] = {}
    names = []
    for name, ref, mov, params in cases:
        rstars = [Star(float(x), float(y), 1000.0 - i) for i, (x, y) in enumerate(ref)]
        mstars = [Star(float(x), float(y), 1000.0 - i) for i, (x, y) in enumerate(mov)]
        res = estimate_triangle_asterism_transform(rstars, mstars, "similarity", **params)
        arrays[f"{name}/ref"] = np.asarray(ref, dtype=np.float64).reshape(-1, 2)
        arrays[f"{name}/mov"] = np.asarray(mov, dtype=np.float64).reshape(-1, 2)
        arrays[f"{name}/params"] = np.asarray(repr(params))
        arrays[f"{name}/matrix"] = np.asarray(res.matrix, dtype=np.float64)
        arrays[f"{name}/inliers"] = np.asarray(res.inliers)
        arrays[f"{name}/rms_px"] = np.asarray(res.rms_px)
        arrays[f"{name}/status"] = np.asarray(res.status)
        arrays[f"{name}/pairs"] = np.asarray(res.pairs, dtype=np.int32).reshape(-1, 2)
        arrays[f"{name}/warnings"] = np.asarray(res.warnings)
        names.append(name)
    arrays["_names"] = np.asarray(names)

    # descriptors of single catalogs
    dnames = []
    for k, (n, mp, nb, md) in enumerate([(80, 80, 5, 1200), (80, 80, 6, 1200), (50, 40, 4, 1200), (80, 80, 5, 300),
                                         (10, 80, 2, 1200), (3, 80, 5, 1200), (64, 80, 5, 1200)]):
        pts = rng.uniform(0.0, 1500.0, size=(n, 2)) if k != 6 else g + 0.0
        desc = _local_triangle_descriptors(pts, max_points=mp, neighbors=nb, max_descriptors=md)
        key = f"desc{k}"
        arrays[f"{key}/points"] = pts
        arrays[f"{key}/params"] = np.asarray(repr(dict(max_points=mp, neighbors=nb, max_descriptors=md)))
        arrays[f"{key}/descriptors"] = np.asarray([d[0] for d in desc], dtype=np.float64).reshape(-1, 2)
        arrays[f"{key}/indices"] = np.asarray([d[1] for d in desc], dtype=np.int32).reshape(-1, 3)
        arrays[f"{key}/areas"] = np.asarray([d[2] for d in desc], dtype=np.float64)
        dnames.append(key)
    arrays["_desc_names"] = np.asarray(dnames)

    # descriptor-list similarity (module fallback; glass_cuda._native() is None here)
    assert glass_cuda._native() is None
    lnames = []
    for k, (n, th, dx, dy, tol) in enumerate([(30, 1.0, 5.0, -3.0, 2.0), (60, -3.0, 20.0, 10.0, 1.0),
                                              (20, 0.0, 0.5, 0.5, 2.0)]):
        ref, mov = _similar_catalog(rng, n, th, 1.0, dx, dy, 0.05, extent=1000.0, drop=2, add=2)
        ref32, mov32 = ref.astype(np.float32), mov.astype(np.float32)
        rdesc = glass_cuda.triangle_asterism_descriptors_f32(ref32[:, 0], ref32[:, 1], 80, 5, 400)
        mdesc = glass_cuda.triangle_asterism_descriptors_f32(mov32[:, 0], mov32[:, 1], 80, 5, 400)
        res = glass_cuda.estimate_similarity_from_triangle_descriptors_f32(
            ref32[:, 0], ref32[:, 1], mov32[:, 0], mov32[:, 1], rdesc["descriptors"], rdesc["indices"],
            mdesc["descriptors"], mdesc["indices"], tolerance_px=tol, descriptor_radius=0.1)
        key = f"list{k}"
        arrays[f"{key}/ref"] = ref32
        arrays[f"{key}/mov"] = mov32
        arrays[f"{key}/ref_desc"] = rdesc["descriptors"]
        arrays[f"{key}/ref_idx"] = rdesc["indices"]
        arrays[f"{key}/mov_desc"] = mdesc["descriptors"]
        arrays[f"{key}/mov_idx"] = mdesc["indices"]
        arrays[f"{key}/tolerance_px"] = np.asarray(tol)
        arrays[f"{key}/matrix32"] = np.asarray(res["matrix"], dtype=np.float32)
        arrays[f"{key}/inliers"] = np.asarray(res["inliers"])
        arrays[f"{key}/rms_px"] = np.asarray(res["rms_px"])
        arrays[f"{key}/best_candidate_index"] = np.asarray(res["best_candidate_index"])
        arrays[f"{key}/status"] = np.asarray(res["status"])
        lnames.append(key)
    arrays["_list_names"] = np.asarray(lnames)
    np.savez_compressed(HERE / "registration.npz", **arrays)


# ---------------------------------------------------------------------------
# alignment metrics / sub-pixel refinement
# ---------------------------------------------------------------------------
def _shifted_field(rng, h, w, n, dx, dy, theta_deg=0.0, noise=3.0):
    """Gaussian stars rendered in the reference frame and in a frame related by
    moving -> reference = rotation(theta) then translation (dx, dy)."""
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    pts = np.column_stack([rng.uniform(3, w - 4, n), rng.uniform(3, h - 4, n)])
    flux = rng.uniform(200.0, 3000.0, n)
    t = np.deg2rad(theta_deg)
    fwd = np.array([[np.cos(t), -np.sin(t), dx], [np.sin(t), np.cos(t), dy], [0.0, 0.0, 1.0]])
    inv = np.linalg.inv(fwd)
    mov_pts = np.column_stack([pts, np.ones(n)]) @ inv.T

    def render(p):
        img = np.full((h, w), 100.0)
        for (x0, y0, _), f in zip(np.column_stack([p[:, :2], np.ones(n)]), flux):
            img += f * np.exp(-((xx - x0) ** 2 + (yy - y0) ** 2) / (2 * 1.3 ** 2))
        return (img + noise * rng.standard_normal((h, w))).astype(np.float32)

    return render(pts), render(mov_pts), fwd


def make_alignment(ref_src: Path) -> None:
    """matrix_alignment_metrics_f32, refine_matrix_translation_with_metrics_f32
    and estimate_translation_subpixel_ncc_f32 (src/glass_cuda.py:706-1245) on
    their NumPy paths (no native module importable here)."""
    sys.path.insert(0, str(ref_src))
    import glass_cuda

    assert glass_cuda._native() is None
    rng = np.random.default_rng(1618)
    arrays: dict[str, np.ndarray] = {}
    # metrics
    ref, mov, _fwd = _shifted_field(rng, 30, 38, 12, 0.37, -0.61)
    mov_nan = mov.copy()
    mov_nan[rng.random(mov.shape) < 0.03] = np.nan
    ref_nan = ref.copy()
    ref_nan[5, 7] = np.nan
    mcases = []
    mats = {"identity": np.eye(3), "shift": np.array([[1.0, 0.0, 0.37], [0.0, 1.0, -0.61], [0.0, 0.0, 1.0]]),
            "rotate": np.array([[0.9998, -0.0175, 1.2], [0.0175, 0.9998, -0.8], [0.0, 0.0, 1.0]]),
            "projective": np.array([[1.0, 0.01, 0.5], [-0.01, 1.0, 0.25], [1e-4, -2e-4, 1.0]]),
            "outside": np.array([[1.0, 0.0, 500.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])}
    for (rname, r), (mname, m) in [(("ref", ref), ("mov", mov)), (("refnan", ref_nan), ("movnan", mov_nan))]:
        for key, mat in mats.items():
            for stride in (1, 2, 3):
                name = f"metrics_{rname}_{mname}_{key}_s{stride}"
                res = glass_cuda.matrix_alignment_metrics_f32(r, m, mat, sample_stride=stride)
                arrays[f"{name}/ref"] = r
                arrays[f"{name}/mov"] = m
                arrays[f"{name}/matrix"] = mat
                arrays[f"{name}/stride"] = np.asarray(stride)
                for k in ("valid_pixels", "sampled_pixels", "rms", "mean_abs_diff", "ncc"):
                    arrays[f"{name}/{k}"] = np.asarray(res[k])
                mcases.append(name)
    arrays["_metric_names"] = np.asarray(mcases)
    # refinement
    rcases = []
    specs = [
        ("refine_default", (0.37, -0.61, 0.0), np.array([[1.0, 0.0, 0.25], [0.0, 1.0, -0.5], [0.0, 0.0, 1.0]]), {}),
        ("refine_rotated", (1.1, 0.4, 0.6),
         np.array([[0.99995, -0.0105, 1.0], [0.0105, 0.99995, 0.5], [0.0, 0.0, 1.0]]),
         dict(search_radius_px=0.5, coarse_step_px=0.25, fine_radius_px=0.125, fine_step_px=0.0625,
              coarse_sample_stride=2, final_sample_stride=1)),
        ("refine_rescore", (-0.3, 0.2, 0.0), np.eye(3),
         dict(search_radius_px=0.5, coarse_step_px=0.25, fine_radius_px=0.0, coarse_sample_stride=3,
              final_sample_stride=1)),
        ("refine_coarse_only", (0.1, 0.1, 0.0), np.eye(3),
         dict(search_radius_px=0.25, coarse_step_px=0.125, fine_radius_px=0.0, coarse_sample_stride=2,
              final_sample_stride=2)),
    ]
    for name, (dx, dy, th), seed, params in specs:
        r, m, _ = _shifted_field(rng, 28, 34, 10, dx, dy, th)
        if name == "refine_rotated":
            m[rng.random(m.shape) < 0.02] = np.nan
        res = glass_cuda.refine_matrix_translation_with_metrics_f32(r, m, seed, **params)
        arrays[f"{name}/ref"] = r
        arrays[f"{name}/mov"] = m
        arrays[f"{name}/seed"] = seed
        arrays[f"{name}/params"] = np.asarray(repr(params))
        arrays[f"{name}/matrix"] = np.asarray(res["matrix"], dtype=np.float32)
        arrays[f"{name}/dx_correction"] = np.asarray(res["dx_correction"])
        arrays[f"{name}/dy_correction"] = np.asarray(res["dy_correction"])
        arrays[f"{name}/coarse_candidates"] = np.asarray(res["coarse_candidates"])
        arrays[f"{name}/fine_candidates"] = np.asarray(res["fine_candidates"])
        for k in ("valid_pixels", "sampled_pixels", "sample_stride", "rms", "mean_abs_diff", "ncc"):
            arrays[f"{name}/metrics_{k}"] = np.asarray(res["metrics"][k])
        rcases.append(name)
    arrays["_refine_names"] = np.asarray(rcases)
    # translation NCC
    ncases = []
    r, m, _ = _shifted_field(rng, 26, 30, 9, 0.8, -0.45)
    flat = np.full((12, 14), 5.0, dtype=np.float32)
    for name, (rr, mm, cdx, cdy, rad, step, stride) in {
            "ncc_s1": (r, m, 0.75, -0.5, 2, 0.125, 1), "ncc_s2": (r, m, 1.0, 0.0, 3, 0.25, 2),
            "ncc_flat": (flat, flat, 0.0, 0.0, 1, 0.5, 1)}.items():
        res = glass_cuda.estimate_translation_subpixel_ncc_f32(rr, mm, cdx, cdy, rad, step, stride)
        arrays[f"{name}/ref"] = rr
        arrays[f"{name}/mov"] = mm
        arrays[f"{name}/args"] = np.asarray([cdx, cdy, rad, step, stride], dtype=np.float64)
        for k in ("dx", "dy", "score", "candidate_count"):
            arrays[f"{name}/{k}"] = np.asarray(res[k])
        ncases.append(name)
    arrays["_ncc_names"] = np.asarray(ncases)
    np.savez_compressed(HERE / "alignment.npz", **arrays)


# ---------------------------------------------------------------------------
# local normalisation
# ---------------------------------------------------------------------------
def make_local_norm(ref_src: Path) -> None:
    """_grid_local_norm_coefficients (src/glass/engine/resident_cuda.py:1897)
    on seeded tile statistics with empty and offset-only tiles, and
    apply_grid_normalization (src/glass/cpu/local_norm.py:197) on seeded
    frames whose size is not a multiple of the tile."""
    ns: dict = {"np": np, "Any": object}
    _load_functions(ref_src / "glass" / "engine" / "resident_cuda.py", ["_grid_local_norm_coefficients"], ns)
    _load_functions(ref_src / "glass" / "cpu" / "local_norm.py", ["apply_grid_normalization"], ns)
    rng = np.random.default_rng(31)
    arrays: dict = {}
    rows, cols = 5, 7
    stats = {
        "source_mean": rng.uniform(500, 1500, (rows, cols)).astype(np.float32),
        "source_std": rng.uniform(5, 60, (rows, cols)).astype(np.float32),
        "reference_mean": rng.uniform(500, 1500, (rows, cols)).astype(np.float32),
        "reference_std": rng.uniform(5, 60, (rows, cols)).astype(np.float32),
        "valid_pixels": rng.integers(1, 65536, (rows, cols)).astype(np.uint64),
    }
    stats["valid_pixels"][0, 0] = 0
    stats["valid_pixels"][3, 6] = 0
    stats["source_std"][1, 2] = np.float32(5e-7)
    stats["reference_std"][2, 4] = np.float32(1e-6)
    stats["source_std"][4, 1] = np.float32(0.0)
    coeffs = ns["_grid_local_norm_coefficients"](stats, eps=1.0e-6)
    for k, v in stats.items():
        arrays[f"coeff/{k}"] = v
    arrays["coeff/scales"] = coeffs["scales"]
    arrays["coeff/offsets"] = coeffs["offsets"]
    for name, (h, w, th, tw) in {"odd": (150, 210, 64, 96), "exact": (128, 192, 64, 64)}.items():
        data = rng.normal(1000.0, 40.0, (h, w)).astype(np.float32)
        data[rng.integers(0, h, 20), rng.integers(0, w, 20)] = np.nan
        gr, gc = -(-h // th), -(-w // tw)
        scales = rng.uniform(0.8, 1.25, (gr, gc)).astype(np.float32)
        offsets = rng.uniform(-200, 200, (gr, gc)).astype(np.float32)
        arrays[f"apply/{name}/data"] = data
        arrays[f"apply/{name}/scales"] = scales
        arrays[f"apply/{name}/offsets"] = offsets
        arrays[f"apply/{name}/tile"] = np.array([th, tw], dtype=np.int64)
        arrays[f"apply/{name}/out"] = ns["apply_grid_normalization"](data, scales, offsets, th, tw)
    arrays["_apply_names"] = np.array(["odd", "exact"])
    np.savez_compressed(HERE / "local_norm.npz", **arrays)


# ---------------------------------------------------------------------------
# cosmetic (source DQ)
# ---------------------------------------------------------------------------
def make_cosmetic(ref_src: Path) -> None:
    """detect_isolated_cosmetic_defects and detect_star_protected_cosmetic_defects
    (src/glass/cpu/cosmetic.py:97-307) on seeded star fields with hot, cold
    and clustered defects and a NaN patch; stores the HOT / COLD bits."""
    sys.path.insert(0, str(ref_src))
    from glass.cpu import cosmetic
    from glass.engine.contracts import DQFlag

    rng = np.random.default_rng(41)
    arrays: dict = {}
    names = []
    for name, (h, w, nstars) in {"small": (96, 128, 25), "wide": (120, 200, 60)}.items():
        img = _star_field(rng, h, w, nstars, 800.0, 10.0)
        ys, xs = rng.integers(2, h - 2, 30), rng.integers(2, w - 2, 30)
        img[ys[:15], xs[:15]] += np.float32(3000.0)  # isolated hot
        img[ys[15:25], xs[15:25]] -= np.float32(700.0)  # isolated cold
        y, x = int(ys[25]), int(xs[25])
        img[y:y + 2, x:x + 2] += np.float32(4000.0)  # supported cluster (kept)
        img[int(ys[26]), :4] = np.nan
        img[0, 0] += np.float32(5000.0)  # corner: edge-padded neighbours
        for kind, fn in (("isolated", cosmetic.detect_isolated_cosmetic_defects),
                         ("protected", cosmetic.detect_star_protected_cosmetic_defects)):
            res = fn(img)
            bits = res.dq_mask.data
            arrays[f"{name}/{kind}/hot"] = (bits & int(DQFlag.HOT_PIXEL)) != 0
            arrays[f"{name}/{kind}/cold"] = (bits & int(DQFlag.COLD_PIXEL)) != 0
        arrays[f"{name}/image"] = img
        names.append(name)
    arrays["_names"] = np.array(names)
    np.savez_compressed(HERE / "cosmetic.npz", **arrays)


# ---------------------------------------------------------------------------
# DQ map (resident_cuda.py:3110-3297, helpers :2961-3100, flags contracts.py:77)
# ---------------------------------------------------------------------------
def make_dq(ref_src: Path) -> None:
    sys.path.insert(0, str(ref_src))
    from glass.engine.contracts import DQFlag

    ns: dict = {"np": np, "Any": object, "DQFlag": DQFlag}
    _load_functions(ref_src / "glass" / "engine" / "resident_cuda.py",
                    ["_resident_dq_flag_dtype", "_resident_dq_map_python", "_resident_coverage_array_stats_from_values",
                     "_resident_finite_count_coverage_stats", "_resident_count_map_array_stats_from_values",
                     "_resident_finite_count_map_array_stats_from_values"], ns)
    dq_fn = ns["_resident_dq_map_python"]
    rng = np.random.default_rng(3110)
    out = {}
    names = []
    h, w = 23, 31
    for case in range(12):
        master = rng.normal(1000.0, 30.0, (h, w)).astype(np.float32)
        weight = rng.uniform(0.0, 9.0, (h, w)).astype(np.float32)
        frames = int(rng.integers(3, 40))
        coverage = rng.integers(0, frames + 1, (h, w)).astype(np.float32)
        low = rng.integers(0, 3, (h, w)).astype(np.float32) * (rng.random((h, w)) < 0.2)
        high = rng.integers(0, 4, (h, w)).astype(np.float32) * (rng.random((h, w)) < 0.3)
        geometric = rng.integers(0, frames + 1, (h, w)).astype(np.float32)
        geometric[rng.random((h, w)) < 0.4] = frames
        if case % 3 == 1:  # non-finite maps, zero and negative weights
            master[rng.random((h, w)) < 0.05] = np.nan
            master[rng.random((h, w)) < 0.02] = np.inf
            weight[rng.random((h, w)) < 0.05] = 0.0
            weight[rng.random((h, w)) < 0.03] = -1.0
            weight[rng.random((h, w)) < 0.02] = np.nan
            coverage[rng.random((h, w)) < 0.03] = np.nan
            low[rng.random((h, w)) < 0.02] = np.nan
            high[rng.random((h, w)) < 0.02] = np.inf
            geometric[rng.random((h, w)) < 0.03] = np.nan
        coverage[rng.random((h, w)) < 0.05] = 0.5  # the <= 0.5 edge
        geometric[rng.random((h, w)) < 0.05] = frames - 0.5  # the partial-coverage edge
        use = [case % 2 == 0, case % 4 != 3, case % 4 != 3, case % 3 != 2]  # coverage, low, high, geometric
        active = frames if case % 5 != 4 else 0
        args = [master, weight, coverage if use[0] else None, low if use[1] else None, high if use[2] else None,
                geometric if use[3] else None, active]
        dq, _summary = dq_fn(*args, dq_dtype=np.int16)
        name = f"case{case}"
        names.append(name)
        out[f"{name}/master"], out[f"{name}/weight"] = master, weight
        for key, arr, flag in (("coverage", coverage, use[0]), ("low", low, use[1]), ("high", high, use[2]),
                               ("geometric", geometric, use[3])):
            if flag:
                out[f"{name}/{key}"] = arr
        out[f"{name}/active"] = np.int64(active)
        out[f"{name}/dq"] = dq
    out["_names"] = np.array(names)
    np.savez_compressed(HERE / "dq.npz", **out)


# ---------------------------------------------------------------------------
# tile-local weighting: the reference test's own CPU expectation
# (tests/test_cuda_resident_stack.py:523-583, `_expected_tile_local_sigma`)
# ---------------------------------------------------------------------------
def make_tile_local(ref_src: Path) -> None:
    ns: dict = {"np": np}
    _load_functions(ref_src.parent / "tests" / "test_cuda_resident_stack.py", ["_expected_tile_local_sigma"], ns)
    expected = ns["_expected_tile_local_sigma"]
    rng = np.random.default_rng(1658)
    out = {}
    names = []
    for case in range(8):
        n = int(rng.integers(3, 9))
        h, w = int(rng.integers(5, 14)), int(rng.integers(6, 15))
        frames = rng.normal(100.0, 5.0, (n, h, w)).astype(np.float32)
        frames[rng.random(frames.shape) < 0.05] += 80.0
        frames[rng.random(frames.shape) < 0.03] = np.nan
        weights = rng.uniform(0.3, 2.0, n).astype(np.float32)
        if case % 3 == 2:
            weights[0] = 0.0
        target = (rng.random(n) < 0.5).astype(np.uint8)
        target[int(rng.integers(0, n))] = 1
        # non-overlapping tiles (the resident path rejects overlaps,
        # resident_cuda.py:5355-5357): cells of a 2 x 2 split, each shrunk
        # at random, some of them dropped
        xs, ys = int(rng.integers(2, w - 1)), int(rng.integers(2, h - 1))
        tiles = []
        for cx0, cx1 in ((0, xs), (xs, w)):
            for cy0, cy1 in ((0, ys), (ys, h)):
                if rng.random() < 0.3 and tiles:
                    continue
                x0 = int(rng.integers(cx0, cx1))
                y0 = int(rng.integers(cy0, cy1))
                tiles.append([x0, y0, int(rng.integers(x0 + 1, cx1 + 1)), int(rng.integers(y0 + 1, cy1 + 1))])
        extents = np.asarray(tiles, dtype=np.int32)
        multipliers = rng.uniform(0.0, 3.0, len(tiles)).astype(np.float32)
        name = f"case{case}"
        names.append(name)
        out[f"{name}/frames"], out[f"{name}/weights"], out[f"{name}/target"] = frames, weights, target
        out[f"{name}/extents"], out[f"{name}/multipliers"] = extents, multipliers
        # no rejection (huge thresholds): the weighted mean
        m = expected(list(frames), weights, target, extents, multipliers, 1e30, 1e30, False)
        out[f"{name}/mean/master"], out[f"{name}/mean/weight"] = m[0], m[1]
        for mode, wins in (("sigma", False), ("winsorized", True)):
            r = expected(list(frames), weights, target, extents, multipliers, 3.0, 1.0, wins)
            for key, arr in zip(("master", "weight", "coverage", "low", "high"), r):
                out[f"{name}/{mode}/{key}"] = arr
    out["_names"] = np.array(names)
    np.savez_compressed(HERE / "tile_local.npz", **out)


def _affine_catalog(rng, n, linear, dx, dy, noise, extent=2000.0, drop=0, add=0, swap=0):
    """Reference catalog (n, 2) and a moving catalog that the affine map
    (linear, (dx, dy)) sends back onto it, with centroid noise, dropped and
    spurious stars and a perturbed brightness order."""
    ref = rng.uniform(20.0, extent - 20.0, size=(n, 2))
    lin = np.asarray(linear, dtype=np.float64)
    mov = (ref - np.array([dx, dy])) @ np.linalg.inv(lin).T + noise * rng.standard_normal((n, 2))
    keep = np.sort(rng.permutation(n)[: n - drop])
    mov = mov[keep]
    if add:
        mov = np.vstack([mov, rng.uniform(0.0, extent, size=(add, 2))])
    order = np.arange(len(mov))
    for _ in range(swap):
        i = int(rng.integers(0, len(mov) - 1))
        order[i], order[i + 1] = order[i + 1], order[i]
    return ref, mov[order]


def make_registration_affine(ref_src: Path) -> None:
    """estimate_triangle_asterism_transform with transform_model="affine"
    (src/glass/cpu/registration.py:106-119, 361-475) on seeded catalogs under
    affine maps (shear and anisotropic scale that a similarity cannot
    represent), the reference test's similarity case and degenerate inputs."""
    sys.path.insert(0, str(ref_src))
    from glass.cpu.registration import estimate_triangle_asterism_transform
    from glass.cpu.star_detect import Star

    rng = np.random.default_rng(31415)
    cases = []
    pts = np.array([(10, 10), (20, 10), (10, 25), (30, 30), (5, 35), (35, 5), (25, 18), (14, 32)], dtype=np.float64)
    ang = np.deg2rad(-7.0)
    lin = 0.98 * np.array([[np.cos(ang), -np.sin(ang)], [np.sin(ang), np.cos(ang)]])
    mov = np.vstack([(pts - np.array([-4.0, 3.0])) @ np.linalg.inv(lin).T, [[100.0, 100.0]]])
    cases.append(("reftest_outlier", pts, mov, dict(min_inliers=8, tolerance_px=0.5)))
    specs = [  # (n, linear perturbation sigma, rotation deg, dx, dy, noise, drop, add, swap, params)
        (80, 1e-3, 0.0, 0.4, -0.3, 0.05, 0, 0, 0, {}),
        (80, 3e-3, 0.3, 12.5, -7.25, 0.05, 0, 0, 0, {}),
        (80, 1e-2, -2.0, -40.0, 33.0, 0.1, 5, 5, 6, {}),
        (60, 2e-2, 4.5, 3.0, 150.0, 0.2, 8, 10, 10, dict(tolerance_px=2.0)),
        (40, 5e-3, 0.0, 0.5, 0.25, 0.0, 0, 0, 0, dict(neighbors=4)),
        (80, 2e-3, 1.0, -5.0, 5.0, 0.05, 0, 0, 0, dict(neighbors=6, max_candidates=200)),
        (80, 4e-3, -0.7, 8.0, -2.0, 0.05, 2, 3, 4, dict(max_descriptors=100, max_candidates=50)),
        (50, 1e-2, 10.0, 100.0, -80.0, 0.1, 0, 0, 0, dict(max_stars=30)),
        (25, 1e-3, 0.2, 1.0, 1.0, 0.05, 10, 12, 0, dict(min_inliers=10)),
        (12, 0.0, 0.0, 2.0, 3.0, 0.0, 0, 0, 0, dict(tolerance_px=1.0)),
        (80, 1e-3, 180.0, 2000.0, 2000.0, 0.05, 0, 0, 0, {}),
        (80, 2e-3, 0.5, 3.0, 4.0, 0.05, 0, 0, 0, dict(descriptor_radius=0.02)),
    ]
    for k, (n, sig, th, dx, dy, noise, drop, add, swap, params) in enumerate(specs):
        t = np.deg2rad(th)
        rot = np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
        linear = rot @ (np.eye(2) + rng.normal(0.0, sig, (2, 2)))
        ref, mov = _affine_catalog(rng, n, linear, dx, dy, noise, drop=drop, add=add, swap=swap)
        cases.append((f"affine{k}", ref, mov, params))
    line = np.column_stack([np.arange(10) * 7.0, np.arange(10) * 3.0])
    cases.append(("collinear", line, line + 1.0, {}))
    cases.append(("two_stars", np.array([[1.0, 2.0], [30.0, 40.0]]), np.array([[2.0, 2.0], [31.0, 40.0]]), {}))
    cases.append(("empty_moving", rng.uniform(0, 100, (10, 2)), np.zeros((0, 2)), {}))

    arrays: dict[str, np.ndarray] = {}
    names = []
    for name, ref, mov, params in cases:
        rstars = [Star(float(x), float(y), 1000.0 - i) for i, (x, y) in enumerate(ref)]
        mstars = [Star(float(x), float(y), 1000.0 - i) for i, (x, y) in enumerate(mov)]
        res = estimate_triangle_asterism_transform(rstars, mstars, "affine", **params)
        arrays[f"{name}/ref"] = np.asarray(ref, dtype=np.float64).reshape(-1, 2)
        arrays[f"{name}/mov"] = np.asarray(mov, dtype=np.float64).reshape(-1, 2)
        arrays[f"{name}/params"] = np.asarray(repr(params))
        arrays[f"{name}/matrix"] = np.asarray(res.matrix, dtype=np.float64)
        arrays[f"{name}/inliers"] = np.asarray(res.inliers)
        arrays[f"{name}/rms_px"] = np.asarray(res.rms_px)
        arrays[f"{name}/status"] = np.asarray(res.status)
        arrays[f"{name}/pairs"] = np.asarray(res.pairs, dtype=np.int32).reshape(-1, 2)
        names.append(name)
    arrays["_names"] = np.asarray(names)
    np.savez_compressed(HERE / "registration_affine.npz", **arrays)


# ---------------------------------------------------------------------------
# registration-quality policy (resident_cuda.py:4905-4998,
# engine/resident_registration_quality.py:41-136)
# ---------------------------------------------------------------------------
def make_quality(ref_src: Path) -> None:
    import json

    sys.path.insert(0, str(ref_src))
    from glass.engine.resident_registration_quality import evaluate_resident_registration_quality

    ns: dict = {"np": np, "Any": object}
    _load_functions(ref_src / "glass" / "engine" / "resident_cuda.py",
                    ["_float_or_nan", "_resident_triangle_agreement_quality", "_resident_triangle_agreement_policy"], ns)
    quality, policy = ns["_resident_triangle_agreement_quality"], ns["_resident_triangle_agreement_policy"]
    records = []
    for ncc in (0.95, 0.4, 0.02, -0.1, float("nan"), None):
        for rms in (0.0, 35.0, 480.0, 5000.0, -3.0, float("nan")):
            for scale in (200.0, 25.0):
                for min_score in (None, 0.0, 0.02, 0.3, 1.0):
                    q = quality(ncc, rms, 0.4, scale, min_score)
                    for action in ("fail", "downweight", "flag"):
                        for floor in (0.0, 0.25):
                            pol = policy(q, action, floor)
                            records.append({"args": [ncc, rms, 0.4, scale, min_score, action, floor],
                                            "quality": {k: q[k] for k in ("score", "status", "reason")},
                                            "policy": {k: pol[k] for k in ("status", "hard_failure",
                                                                           "weight_multiplier")}})
    gates = []
    for status in ("ok", "failed", "reference", "excluded", "weird"):
        for inliers in (0, 3, 4, 12):
            for rms in (0.2, 2.5, float("nan")):
                for action in ("auto", "off", "warn", "exclude"):
                    for mode in ("similarity_cuda_triangle", "translation"):
                        for max_rms in (None, 1.0):
                            for stars in (None, (2, 50)):
                                d = evaluate_resident_registration_quality(
                                    frame_id="f", registration_mode=mode, requested_action=action, status=status,
                                    matched_stars=inliers, inliers=inliers, rms_px=rms, min_inliers=4,
                                    max_rms_px=max_rms,
                                    diagnostics=None if stars is None else {"reference_stars": stars[0],
                                                                             "moving_stars": stars[1]})
                                gates.append({"args": [status, inliers, rms, mode, action, 4, max_rms,
                                                       None if stars is None else stars[0],
                                                       None if stars is None else stars[1]],
                                              "out": {k: d[k] for k in ("effective_action", "final_status",
                                                                        "decision_status", "action_applied",
                                                                        "accepted", "reasons")}})
    text = json.dumps({"agreement": records, "gate": gates}, allow_nan=True)
    np.savez_compressed(HERE / "quality.npz", json=np.frombuffer(text.encode(), dtype=np.uint8))


def main() -> int:
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("--reference", default="/root/reference", help="GLASS reference checkout")
    parser.add_argument("--only", default="", help="comma-separated subset")
    args = parser.parse_args()
    ref = Path(args.reference)
    src = ref / "src"
    jobs = {"integration": make_integration, "calibration": make_calibration, "warp": make_warp,
            "stars": make_stars, "registration": make_registration,
            "registration_affine": make_registration_affine, "alignment": make_alignment,
            "local_norm": make_local_norm, "cosmetic": make_cosmetic, "dq": make_dq,
            "tile_local": make_tile_local, "quality": make_quality}
    only = [j for j in args.only.split(",") if j] or list(jobs)
    for job in only:
        jobs[job](src)
        print(f"wrote {job}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
