"""Benchmark of the resident light-stack hot path on GB300.

Workload (default): the 32 x 2048 x 2048 uint16 stack (synthetic, seeded;
~2000 stars, hot pixels, cosmic rays, satellite trails) -> fused decode +
calibration -> simple_snr frame weights -> winsorized sigma-clip weighted
integration into the six maps.  Metric: stacked Mpix-frames/s (N*H*W/1e6 per
step / step time), plus the HBM roofline of the dominant kernel.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun each rank processes its own stack (replicas: the path has no
exchange step), value = all ranks' Mpix-frames / max-over-ranks time.
`--impl reference` times the CPU oracle port of the reference algorithm on the
host cores instead (rank 0 only).
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

from glass_gb300 import replicas  # noqa: E402  (no CUDA needed to import)
from glass_gb300.replicas import dist_env  # noqa: E402

L2_BYTES = 129 * 1024 * 1024
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser(description=__doc__)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--config", default="c2", choices=["c1", "c2", "c5"],
                   help="c5: the full 200 x 9600 x 6422 stack resident (device step only, one GPU)")
    p.add_argument("--frames", type=int, default=0, help="override frame count (smaller smoke runs)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-adjoint", action="store_true", help="skip the gradient-refinement registration report")
    return p.parse_args()



def measured_peak():
    path = REPO / "MEASURED_PEAKS.json"
    if path.exists():
        try:
            data = json.loads(path.read_text())
            return float(data["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(name: str):
    """Per-launch DRAM bytes recorded from an ncu capture in profiles/."""
    path = REPO / "profiles" / name
    if not path.exists():
        return None
    for line in path.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch_full_size:"):
            try:
                return int(float(line.split(":", 1)[1].strip()))
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling (every 20 ms) during the timed
    region: samples are time-stamped and only those between mark_start() and
    mark_stop() are summarised."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None
        self.t0 = None
        self.t1 = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=self.file, stderr=subprocess.DEVNULL)
            time.sleep(0.5)  # let the sampler start before the timed region
        except Exception:
            self.proc = None
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_stop(self):
        self.t1 = time.time()
        time.sleep(0.05)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        import datetime as _dt

        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                ts = _dt.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                continue
            if self.t0 is not None and self.t1 is not None and not (self.t0 - 0.02 <= ts <= self.t1 + 0.02):
                continue
            rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples in the timed region"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, val in zip(names, r[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ---------------------------------------------------------------------------
# CPU baseline (the oracle port of the reference algorithm, host cores)
# ---------------------------------------------------------------------------
CPU_CROP = 384  # side of the crops the warp, refinement and integration samples use


_CPU_DATA = None  # (lights, bias, dark, flat, truth) shared with the forked sample processes


def _cpu_step_sample(spec):
    """One bounded sample of every stage of the step, timed with the oracle
    port of the reference's CPU code; returns seconds per stage.  Full frames
    for calibration, detection and registration; crops for the warp, the
    refinement and the integration."""
    from oracle import alignment, registration, stars, warp
    from oracle.calibration import calibrate_light
    from oracle.integration import weighted_integrate_stack

    lights, bias, dark, flat, truth = _CPU_DATA
    mov, y0, x0 = spec
    n = lights.shape[0]
    raw = lights[[0, mov]]
    matrix = truth[mov]
    c = CPU_CROP
    times = {}
    t = time.perf_counter()
    cal = [calibrate_light(raw[k], bias, dark, flat, 1.0, 1.0, master_dark_includes_bias=False) for k in (0, 1)]
    times["calibrate"] = (time.perf_counter() - t) / 2
    t = time.perf_counter()
    cats = []
    for k in (0, 1):
        found = stars.detect_stars(cal[k], threshold_sigma=5.0, max_stars=400)
        cats.append([(s[0], s[1]) for s in found if s[5] is not None and s[5] <= 0.8][:80])
    times["detect_stars"] = (time.perf_counter() - t) / 2
    t = time.perf_counter()
    registration.estimate_triangle_asterism_transform(cats[0], cats[1])
    times["register"] = time.perf_counter() - t
    ref_crop = np.ascontiguousarray(cal[0][y0:y0 + c, x0:x0 + c])
    mov_crop = np.ascontiguousarray(cal[1][y0:y0 + c, x0:x0 + c])
    t = time.perf_counter()
    alignment.refine_translation(ref_crop, mov_crop, matrix, 1.0, 0.25, 0.25, 0.0625, 4, 8)
    times["refine_translation"] = time.perf_counter() - t
    t = time.perf_counter()
    warp.warp_matrix(mov_crop, matrix, "lanczos3", np.nan)
    times["warp_lanczos3"] = time.perf_counter() - t
    stack = np.stack([calibrate_light(lights[k, y0:y0 + c, x0:x0 + c], bias[y0:y0 + c, x0:x0 + c],
                                      dark[y0:y0 + c, x0:x0 + c], flat[y0:y0 + c, x0:x0 + c], 1.0, 1.0,
                                      master_dark_includes_bias=False) for k in range(n)])
    t = time.perf_counter()
    finite = np.isfinite(stack)
    means = np.array([stack[k][finite[k]].astype(np.float64).mean() for k in range(n)])
    stds = np.array([stack[k][finite[k]].astype(np.float64).std() for k in range(n)])
    weights = np.maximum(np.abs(means) / np.maximum(stds, 1e-6), 1e-6).astype(np.float32)
    weighted_integrate_stack(stack, weights, "winsorized_sigma")
    times["weights_integrate"] = time.perf_counter() - t
    return times


def cpu_step_estimate(data, masters, processes: int):
    """Seconds one full step takes on the host cores (oracle port), composed
    from `processes` concurrent samples: per-frame stages x frames, per-pixel
    stages scaled from their crops.  Returns (Mpix-frames/s over all the
    processes, mean seconds per step, stage seconds per step, description)."""
    import multiprocessing as mp

    global _CPU_DATA
    n, h, w = data.lights.shape
    c = CPU_CROP
    _CPU_DATA = (data.lights, masters.bias, masters.dark, masters.flat, data.truth_matrices)
    rng = np.random.default_rng(0)
    specs = [(1 + k % (n - 1), int(rng.integers(0, h - c + 1)), int(rng.integers(0, w - c + 1)))
             for k in range(processes)]
    if processes <= 1:
        samples = [_cpu_step_sample(specs[0])]
    else:
        # forked workers share the stack without pickling it; this process
        # has not touched CUDA (the reference arm never does)
        with mp.get_context("fork").Pool(processes) as pool:
            samples = pool.map(_cpu_step_sample, specs)
    px_scale = (h * w) / (c * c)
    steps = []
    for s in samples:
        stage = {"calibrate": n * s["calibrate"], "detect_stars": n * s["detect_stars"],
                 "register": (n - 1) * s["register"],
                 "refine_translation": (n - 1) * s["refine_translation"] * px_scale,
                 "warp_lanczos3": (n - 1) * s["warp_lanczos3"] * px_scale,
                 "weights_integrate": s["weights_integrate"] * px_scale}
        steps.append(stage)
    mean = {k: float(np.mean([st[k] for st in steps])) for k in steps[0]}
    step_s = sum(mean.values())
    value = processes * n * h * w / 1e6 / step_s
    desc = (f"{processes} process(es), each: calibrate + detect 2 full {h}x{w} frames, triangle registration of one "
            f"pair, NCC refine + Lanczos3 warp of one {c}x{c} crop pair, weights + winsorized integration of a "
            f"{n}x{c}x{c} crop; composed to one {n}-frame step (per-pixel stages scaled by {px_scale:.0f}x)")
    return value, step_s, mean, desc


def adjoint_report(pipe, dev_raw, reg, truth, h, w, stream) -> dict:
    """Registration accuracy against the synthetic truth, same GPU, same
    frames: triangle asterism (plain), plus the NCC translation grid refine,
    plus the gradient (adjoint-warp) similarity refine started from the
    triangle matrices.  Outside the timed step."""
    import torch

    from glass_gb300.adjoint import RefineConfig, registration_rms_px

    pipe.calibrate_device(dev_raw.data_ptr())  # the timed steps left warped frames behind
    stream.synchronize()
    ok = [k for k in range(1, pipe.frames) if reg["ok"][k]]

    def rms(mats):
        return registration_rms_px([mats[k] for k in ok], [truth[k] for k in ok], h, w)

    def timed(method, reps=3, gradient=None):
        pipe.config.refine_method = method
        pipe.config.gradient_refine = gradient
        try:
            out = pipe.refine(reg["triangle"], 0)
            stream.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                out = pipe.refine(reg["triangle"], 0)
            stream.synchronize()
            return out, 1e3 * (time.perf_counter() - t0) / reps
        finally:
            pipe.config.refine_method = "ncc"
            pipe.config.gradient_refine = None

    ncc, ncc_ms = timed("ncc")
    gn, gn_ms = timed("gradient")
    gn2, gn2_ms = timed("gradient", gradient={"sample_stride": 2, "target_samples": None})
    gn4, gn4_ms = timed("gradient", gradient={"sample_stride": 4, "target_samples": None})
    # the generic autograd path (torch.autograd through the warp adjoint,
    # trust-region Newton over torch ops, one frame at a time) on 4 frames
    sub = ok[:4]
    t0 = time.perf_counter()
    torch_mats, outcomes = pipe.refine_adjoint(reg["triangle"], 0, RefineConfig(model="similarity", loss="ssd"),
                                               frames=sub)
    torch.cuda.synchronize()
    torch_ms = 1e3 * (time.perf_counter() - t0) / max(1, len(sub))

    def rms_sub(mats):
        return registration_rms_px([mats[k] for k in sub], [truth[k] for k in sub], h, w)

    return {"rms_px_vs_truth": {"triangle": rms(reg["triangle"]), "ncc_translation": rms(ncc),
                                "gradient_gauss_newton": rms(gn), "gradient_gauss_newton_stride2": rms(gn2),
                                "gradient_gauss_newton_stride4": rms(gn4)},
            "refine_ms_per_step": {"ncc_translation": ncc_ms, "gradient_gauss_newton": gn_ms,
                                   "gradient_gauss_newton_stride2": gn2_ms,
                                   "gradient_gauss_newton_stride4": gn4_ms},
            "frames_compared": len(ok),
            "autograd_subset": {"frames": len(sub), "ms_per_frame": torch_ms,
                                "rms_px_vs_truth": {"triangle": rms_sub(reg["triangle"]), "ncc_translation":
                                                    rms_sub(ncc), "gradient_gauss_newton": rms_sub(gn),
                                                    "gradient_autograd_ssd": rms_sub(torch_mats)},
                                "evaluations_mean": float(np.mean([o.evaluations for o in outcomes]))
                                if outcomes else 0.0}}


def local_norm_report(pipe, stream, reps: int, peak: float) -> dict:
    """Grid local normalisation (tile 256, the resident default mode) of the
    31 warped frames to the reference: tile statistics (8 B per pixel: source
    and reference) + in-place apply (8 B per pixel), CUDA events."""
    import torch

    idx = list(range(1, pipe.frames))
    run = lambda: pipe.stack.local_normalize_grid(0, idx, 256, 1.0e-6, update_weights=False)  # noqa: E731
    run()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        run()
    e1.record(stream)
    stream.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nbytes = 16 * len(idx) * pipe.height * pipe.width
    achieved = nbytes / (ms / 1e3) / 1e9
    return {"tile": 256, "frames": len(idx), "ms_per_call": ms, "algorithmic_bytes": nbytes,
            "achieved_gbs": achieved, "frac_of_measured_hbm": achieved / peak}


def large_stack_report(reps: int, frames: int = 200, height: int = 1024, width: int = 1024) -> dict:
    """Winsorized 3/3 weighted integration of a 200-frame stack (c5's frame
    count at 1024 x 1024: the warp-per-pixel integrator), seeded noise frames
    with 1 % outliers resident on the device, device simple-SNR weights, CUDA
    events over `reps` launches on the stack's stream."""
    import torch

    from glass_gb300 import _glass_cuda_native as native
    from glass_gb300 import _lib

    stream = torch.cuda.Stream()
    rng = np.random.default_rng(17)
    s = native.ResidentCalibratedStack(frames, height, width)
    try:
        s.set_stream(stream.cuda_stream)
        base = rng.normal(1000.0, 20.0, (8, height, width)).astype(np.float32)
        base[rng.random(base.shape) < 0.01] += 5000.0
        for k in range(frames):
            s.upload_calibrated_frame(k, base[k % 8] + np.float32(k % 5))
        s.compute_frame_weights("simple_snr", None, 1.0e-6, download=False)

        def run():
            s.integrate_async("device", _lib.GG_REJECT_WINSORIZED, 3.0, 3.0, 3, 0.5, "uint16")

        def timed(fn):
            for _ in range(2):
                fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            stream.synchronize()
            return e0.elapsed_time(e1) / reps

        ms = timed(run)
        # the same stack through the fused Lanczos3 warp + integration (small
        # seeded similarities; the frames are sampled, not rewritten)
        mats = np.zeros((frames, 3, 3))
        for k in range(frames):
            t = np.deg2rad(rng.uniform(-0.3, 0.3)) if k else 0.0
            dx, dy = (rng.uniform(-8, 8), rng.uniform(-8, 8)) if k else (0.0, 0.0)
            mats[k] = [[np.cos(t), -np.sin(t), dx], [np.sin(t), np.cos(t), dy], [0.0, 0.0, 1.0]]
        fused_ms = timed(lambda: s.integrate_warped_device_weights(mats, "lanczos3", -1.0,
                                                                   _lib.GG_REJECT_WINSORIZED, 3.0, 3.0, 3, 0.5,
                                                                   "uint16"))
    finally:
        s.close()
    px = height * width
    nbytes = 4 * frames * px + 16 * px
    peak, kind = measured_peak()
    return {"stack": [frames, height, width], "kernel": "integrate_warp_kernel<8, 0>", "ms": ms,
            "fused_lanczos3_ms": fused_ms,
            "algorithmic_bytes": nbytes, "achieved_gbs": nbytes / (ms / 1e3) / 1e9,
            "frac": nbytes / (ms / 1e3) / 1e9 / peak, "peak_source": kind}


def batch_report(reps: int) -> dict:
    """Uneven stacks winsorized-integrated one after another vs batched (one
    launch per frame-count bucket), CUDA events on one stream, seeded noise
    frames resident on the device: four large stacks (25/20/16/12 frames at
    1024x1024, 1536x1024, 1024x768, 2048x512; 25 x 1024^2 is the c4 C shape)
    and sixteen small ones (8-16 frames at 256x256 / 256x320)."""
    large = [(25, 1024, 1024), (20, 1536, 1024), (16, 1024, 768), (12, 2048, 512)]
    small = [(8 + (k % 3) * 4, 256, 256 + 64 * (k % 2)) for k in range(16)]
    return {"large_uneven": _batch_case(large, reps), "many_small": _batch_case(small, reps)}


def _batch_case(shapes, reps: int) -> dict:
    import torch

    from glass_gb300 import _glass_cuda_native as native
    from glass_gb300 import _lib

    stream = torch.cuda.Stream()
    stacks = []
    try:
        rng = np.random.default_rng(3)
        for n, h, w in shapes:
            s = native.ResidentCalibratedStack(n, h, w)
            s.set_stream(stream.cuda_stream)
            frames = rng.normal(1000.0, 20.0, (n, h, w)).astype(np.float32)
            for k in range(n):
                s.upload_calibrated_frame(k, frames[k])
            s.compute_frame_weights("simple_snr", None, 1.0e-6, download=False)
            stacks.append(s)

        def sequential():
            for s in stacks:
                s.integrate_async("device", _lib.GG_REJECT_WINSORIZED, 3.0, 3.0, 3, 0.5, "uint16")

        def batched():
            native.integrate_stacks_batch(stacks, _lib.GG_REJECT_WINSORIZED, 3.0, 3.0, 3, 0.5, "uint16")

        def timed(fn):
            for _ in range(2):
                fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            stream.synchronize()
            return e0.elapsed_time(e1) / reps

        seq_ms, batch_ms = timed(sequential), timed(batched)
        mpix = sum(n * h * w for n, h, w in shapes) / 1e6
        return {"stacks": [list(s) for s in shapes], "sequential_ms": seq_ms, "batched_ms": batch_ms,
                "mpix_frames_per_s_batched": mpix / (batch_ms / 1e3)}
    finally:
        for s in stacks:
            s.close()


def graph_report(pipe, dev_raw, matrices, stream, reps: int) -> dict:
    """calibrate -> weights -> fused warp + winsorized integration with fixed
    matrices: the eager launch sequence against its CUDA-graph replay, same
    stream, CUDA events, inputs larger than L2 (the raw stack and the frames)."""
    import torch

    if pipe.frames > 32:
        return {"skipped": "the fused warp-integration takes at most 32 frames"}
    ptr = dev_raw.data_ptr()

    def timed(fn):
        for _ in range(2):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / reps

    eager_ms = timed(lambda: pipe.step_device_fused(ptr, matrices))
    kernels = pipe.capture_graph(ptr, matrices)
    graph_ms = timed(pipe.launch_graph)
    pipe.stack.destroy_step_graph()
    return {"sequence": "calibrate -> simple-SNR weights -> fused Lanczos3 warp + winsorized integration",
            "eager_ms_per_step": eager_ms, "graph_ms_per_step": graph_ms, "kernels_per_replay": kernels,
            "mpix_frames_per_s_graph": pipe.frames * pipe.height * pipe.width / 1e6 / (graph_ms / 1e3)}


def refinement_by(results: list, frame: int) -> dict:
    for r in results:
        if r.get("frame") == frame:
            return r
    return {}


def run_c5(args) -> int:
    """The full c5 stack resident on one GPU: 200 frames of 9600 x 6422
    (49.3 GB of float32 frames).  Eight distinct seeded raw frames are
    rendered at full size (c5's star, sky and defect model; 2 calibration
    frames of each kind) and cycled over the 200 frame slots on the device, so
    no 24.7 GB host array is needed.  Step: calibrate -> star catalogs ->
    triangle registration -> Gauss-Newton refinement -> Lanczos3 warp ->
    simple-SNR weights -> winsorized 3/3 integration; CUDA events per stage
    over K steps.  About 6000 cosmic-ray hits per frame are as bright as the
    brightest stars, so the catalog keeps the 4096 brightest detections for
    the shape filter to find 80 round stars among them (with 400, fewer than
    ten survive and no frame registers)."""
    import dataclasses

    import torch

    from glass_gb300 import _lib
    from glass_gb300.pipeline import ResidentPipeline, StepConfig, build_masters
    from glass_gb300.synthetic import CONFIGS, generate

    torch.cuda.set_device(0)
    n = args.frames or 200
    unique = 8
    cfg = dataclasses.replace(CONFIGS["c5"], calibration_frames=2)
    data = generate(cfg, unique)
    _, h, w = data.lights.shape
    masters = build_masters(data.bias_frames, data.dark_frames, data.flat_frames)
    pipe = ResidentPipeline(n, h, w, masters, StepConfig(star_max_stars=4096, refine_method="gradient"))
    stream = torch.cuda.Stream()
    pipe.set_stream(stream.cuda_stream)
    dev_raw = torch.from_numpy(data.lights.view(np.int16)).cuda()
    truth = np.asarray([data.truth_matrices[k % unique] for k in range(n)])
    idx_groups = [np.arange(k, min(k + unique, n), dtype=np.int64) for k in range(0, n, unique)]
    reg = {}

    def calibrate():
        for g in idx_groups:
            _lib.call("gg_stack_calibrate_u16_device", pipe.stack.handle, _lib.ptr(g), ctypes.c_int64(g.size),
                      ctypes.c_void_p(dev_raw.data_ptr()), 0, ctypes.byref(pipe._calib_params()))

    def register():
        reg["triangle"], reg["ok"] = pipe.register(0)

    def refine():
        reg["m"] = pipe.refine(reg["triangle"], 0)

    P = h * w
    stages = [("calibrate", calibrate, 6 * n * P + 12 * P), ("detect_stars", pipe.detect, 4 * n * P),
              ("register", register, None), ("refine_gradient", refine, None),
              ("warp_lanczos3", lambda: pipe.warp(reg["m"]), 8 * (n - 1) * P),
              ("weights", pipe.weights, 4 * n * P), ("integrate_winsorized", pipe.integrate, 4 * n * P + 16 * P)]
    for _ in range(max(1, args.warmup)):
        for _, fn, _ in stages:
            fn()
    stream.synchronize()
    events = {name: [] for name, _, _ in stages}
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(args.steps):
        for name, fn, _ in stages:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            events[name].append((e0, e1))
    stop.record(stream)
    stream.synchronize()
    ms = start.elapsed_time(stop) / args.steps
    peak, kind = measured_peak()
    out_stages = {}
    for name, _, nbytes in stages:
        t = statistics.mean(a.elapsed_time(b) for a, b in events[name])
        gbs = None if nbytes is None else nbytes / (t / 1e3) / 1e9
        out_stages[name] = {"ms": t, "algorithmic_bytes": nbytes, "achieved_gbs": gbs,
                            "frac": None if gbs is None else gbs / peak}
    ok = [k for k in range(1, n) if reg["ok"][k]]
    from glass_gb300.adjoint import registration_rms_px

    # ingest: the 200 raw frames from pinned host memory (the 8 distinct
    # frames cycled) -> H2D -> decode + calibration, the reference's
    # host-read/H2D-bound stage
    host_raw = torch.from_numpy(data.lights.view(np.int16)).pin_memory()

    def ingest():
        for g in idx_groups:
            _lib.call("gg_stack_calibrate_u16", pipe.stack.handle, _lib.ptr(g), ctypes.c_int64(g.size),
                      ctypes.c_void_p(host_raw.data_ptr()), 0, ctypes.byref(pipe._calib_params()))

    ingest()
    stream.synchronize()
    i0, i1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    i0.record(stream)
    ingest()
    i1.record(stream)
    stream.synchronize()
    ingest_wall_ms = 1e3 * (time.perf_counter() - t0)
    ingest_ms = i0.elapsed_time(i1)
    raw_bytes = 2 * n * P
    # fused Lanczos3 warp + winsorized integration of the 200 frames (the
    # warp-per-pixel integrator sampling every frame; nothing written to the
    # stack) against the warp + integrate stages above
    calibrate()
    pipe.weights()
    cfg = pipe.config

    def fused():
        pipe.stack.integrate_warped_device_weights(reg["m"], cfg.interpolation, cfg.clamping_threshold, cfg.rejection,
                                                   cfg.low_sigma, cfg.high_sigma, cfg.min_samples,
                                                   cfg.max_reject_fraction, cfg.count_map_dtype)

    fused()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    fused()
    f1.record(stream)
    stream.synchronize()
    fused_ms = f0.elapsed_time(f1)
    calibrate()  # detection statistics of the calibrated (not the warped) frames
    info = pipe.detect(info=True)
    inliers = [r["inliers"] for r in pipe.last_registration]
    rms_tri = registration_rms_px([reg["triangle"][k] for k in ok], [truth[k] for k in ok], h, w)
    rms_gn = registration_rms_px([reg["m"][k] for k in ok], [truth[k] for k in ok], h, w)
    refinement = getattr(pipe, "last_refinement", [])
    per_frame = sorted(((registration_rms_px([reg["m"][k]], [truth[k]], h, w),
                         registration_rms_px([reg["triangle"][k]], [truth[k]], h, w), k) for k in ok), reverse=True)

    line = {"metric": "stacked Mpix-frames/s", "value": n * P / 1e6 / (ms / 1e3), "unit": "Mpix-frames/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (8 distinct seeded raw frames cycled over the frame slots)",
            "config": {"workload": f"c5:{n}x{h}x{w} uint16 -> calibrate -> star catalogs -> triangle registration "
                                   "-> Gauss-Newton refinement -> Lanczos3 warp -> simple_snr weights -> "
                                   "winsorized 3/3 integration",
                       "star_max_stars": 4096,
                       "frames": n, "height": h, "width": w, "unique_raw_frames": unique,
                       "l2": "inputs larger than L2", "peak_source": kind},
            "resident": {"stack_bytes_allocated": pipe.stack.bytes_allocated,
                         "device_bytes_in_use": int(torch.cuda.mem_get_info()[1] - torch.cuda.mem_get_info()[0])},
            "stages": out_stages,
            "fused_warp_integrate": {"ms": fused_ms, "vs_warp_plus_integrate_ms":
                                     out_stages["warp_lanczos3"]["ms"] + out_stages["integrate_winsorized"]["ms"]},
            "ingest_from_pinned_host": {"frames": n, "raw_bytes": raw_bytes, "ms_events": ingest_ms,
                                        "ms_wall": ingest_wall_ms,
                                        "raw_gb_per_s": raw_bytes / (max(ingest_ms, ingest_wall_ms) / 1e3) / 1e9},
            "detection": {"candidates_max": max(r["candidates"] for r in info),
                          "candidates_min": min(r["candidates"] for r in info), "candidate_capacity": 32768,
                          "catalog_stars_min": min(r["stars"] for r in info)},
            "registration": {"frames_ok": len(ok) + 1, "frames": n,
                             "inliers_median": float(np.median(inliers)) if inliers else None,
                             "rms_px_vs_truth": {"triangle": rms_tri, "gradient_gauss_newton": rms_gn},
                             "refine_status": {str(v): sum(1 for r in refinement if r.get("status") == v)
                                               for v in sorted({r.get("status") for r in refinement})},
                             "refine_iterations_mean": (float(np.mean([r["iterations"] for r in refinement]))
                                                        if refinement else None),
                             "refine_last_step_px_median_at_cap": (
                                 float(np.median([r["last_step_px"] for r in refinement
                                                  if r.get("status") == "iteration_cap"]))
                                 if any(r.get("status") == "iteration_cap" for r in refinement) else None),
                             "worst_frames": [{"frame": k, "gradient_px": g, "triangle_px": t,
                                               **{q: refinement_by(refinement, k).get(q)
                                                  for q in ("status", "iterations", "alpha", "sigma", "samples",
                                                            "last_step_px")}}
                                              for g, t, k in per_frame[:6]]}}
    print(json.dumps(line))
    pipe.close()
    return 0


# ---------------------------------------------------------------------------
def main():
    args = parse_args()
    if args.config == "c5" and args.impl == "gb300":
        return run_c5(args)
    rank, world, local = dist_env()
    from glass_gb300.synthetic import CONFIGS, generate

    cfg = CONFIGS[args.config]
    frames = args.frames or cfg.frames
    workload = f"{args.config}:{frames}x{cfg.height}x{cfg.width} uint16 -> calibrate -> star catalogs -> " \
               f"triangle registration -> sub-pixel translation refinement -> Lanczos3 warp -> simple_snr " \
               f"weights -> winsorized 3/3 weighted " \
               f"integration (6 maps)"
    metric = "stacked Mpix-frames/s"

    if args.impl == "reference":
        if rank != 0:
            return 0
        data = generate(cfg, frames)
        from oracle.integration import weighted_integrate_stack  # noqa: F401  (the oracle port)
        bias = data.bias_frames.astype(np.float64).mean(0).astype(np.float32)
        dark = (data.dark_frames.astype(np.float64).mean(0) - bias).astype(np.float32)
        flat = (data.flat_frames.astype(np.float64).mean(0) - bias)
        flat = np.maximum(flat / np.median(flat), 1e-6).astype(np.float32)

        class M:  # noqa: D401
            pass

        m = M()
        m.bias, m.dark, m.flat = bias, dark, flat
        procs = os.cpu_count() or 1
        if args.warmup > 0:  # one untimed sample batch warms the caches and imports
            cpu_step_estimate(data, m, procs)
        values, step_s, desc, stages = [], [], "", {}
        for _ in range(args.steps):
            v, s, stages, desc = cpu_step_estimate(data, m, procs)
            values.append(v)
            step_s.append(s)
        value = float(np.mean(values))
        line = {
            "metric": metric, "value": value, "unit": "Mpix-frames/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(step_s)) / procs,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": workload, "sample": desc},
            "stages_s_per_step_one_process": stages,
            "cpu_baseline": {"value": value, "unit": "Mpix-frames/s", "cores": procs, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": "Mpix-frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return 0

    import torch

    torch.cuda.set_device(local)
    replicas.init("nccl", torch.device("cuda", local))
    from glass_gb300 import _lib
    from glass_gb300.pipeline import DEFAULT_REFINE, ResidentPipeline, StepConfig, build_masters

    data = generate(cfg, frames)
    n, h, w = data.lights.shape
    masters = build_masters(data.bias_frames, data.dark_frames, data.flat_frames)
    pipe = ResidentPipeline(n, h, w, masters, StepConfig(refine=dict(DEFAULT_REFINE)))
    stream = torch.cuda.Stream()
    pipe.set_stream(stream.cuda_stream)
    dev_raw = torch.from_numpy(data.lights.view(np.int16)).to(f"cuda:{local}")
    torch.cuda.synchronize()

    barrier = replicas.barrier

    # ---- device-resident throughput ("value") ----
    P = h * w
    reg = {}

    def register():
        reg["triangle"], reg["ok"] = pipe.register(0)

    def refine():
        reg["matrices"] = pipe.refine(reg["triangle"], 0)

    # NCC refine: 8 B per sampled pixel per candidate (reference + moving
    # sample), coarse and fine grids, every frame but the reference
    rp = DEFAULT_REFINE
    n_coarse = len(np.arange(-rp["search_radius_px"], rp["search_radius_px"] + rp["coarse_step_px"] * 0.5,
                             rp["coarse_step_px"], dtype=np.float32)) ** 2
    n_fine = len(np.arange(-rp["fine_radius_px"], rp["fine_radius_px"] + rp["fine_step_px"] * 0.5,
                           rp["fine_step_px"], dtype=np.float32)) ** 2

    def sampled(stride):
        return -(-w // stride) * -(-h // stride)

    refine_bytes = 8 * (n - 1) * (n_coarse * sampled(rp["coarse_sample_stride"]) +
                                  n_fine * sampled(rp["final_sample_stride"]))
    stages = [
        ("calibrate", lambda: pipe.calibrate_device(dev_raw.data_ptr()), 6 * n * P + 12 * P),
        ("detect_stars", pipe.detect, 4 * n * P),
        ("register", register, None),
        ("refine_translation", refine, refine_bytes),
        ("warp_lanczos3", lambda: pipe.warp(reg["matrices"]), 8 * (n - 1) * P),
        ("weights", pipe.weights, 4 * n * P),
        ("integrate_winsorized", pipe.integrate, 4 * n * P + 16 * P),
    ]
    for _ in range(args.warmup):
        for _, fn, _ in stages:
            fn()
    stream.synchronize()
    barrier()
    torch.cuda.synchronize()
    launches0 = _lib.kernel_launches()
    events = {name: [] for name, _, _ in stages}
    with ClockSampler(local) as clocks:
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        clocks.mark_start()
        start.record(stream)
        for _ in range(args.steps):
            for name, fn, _ in stages:
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                events[name].append((e0, e1))
        stop.record(stream)
        stream.synchronize()
        clocks.mark_stop()
    torch.cuda.synchronize()
    barrier()
    launches = _lib.kernel_launches() - launches0
    elapsed_ms = start.elapsed_time(stop)
    stage_ms = {name: statistics.mean(a.elapsed_time(b) for a, b in ev) for name, ev in events.items()}
    elapsed_ms = replicas.max_over_ranks(elapsed_ms, torch.device("cuda", local))
    mpix_frames = n * h * w / 1e6
    value = replicas.replica_throughput(world, mpix_frames, args.steps, elapsed_ms / 1e3)

    # ---- end to end through the public API (host pinned in, host maps out) ----
    truth = np.asarray(data.truth_matrices, dtype=np.float64)
    probe = np.array([[0.0, 0.0, 1.0], [w - 1.0, 0.0, 1.0], [0.0, h - 1.0, 1.0], [w - 1.0, h - 1.0, 1.0]])
    def corner_err(mats):
        return max(float(np.abs(probe @ (mats[k] - truth[k]).T).max()) for k in range(n))

    registration = {"frames_ok": int(reg["ok"].sum()), "frames": n,
                    "max_corner_error_px_vs_truth": {"triangle": corner_err(reg["triangle"]),
                                                     "refined": corner_err(reg["matrices"])}}
    if not args.no_adjoint:
        registration.update(adjoint_report(pipe, dev_raw, reg, truth, h, w, stream))
    graph = graph_report(pipe, dev_raw, reg["matrices"], stream, max(3, args.steps))
    local_norm = local_norm_report(pipe, stream, max(3, args.steps), measured_peak()[0])
    batch = batch_report(max(3, args.steps))
    large = large_stack_report(max(3, args.steps))
    pinned =torch.from_numpy(data.lights.view(np.int16)).pin_memory().numpy().view(np.uint16)
    # reused pinned destinations for the six maps (master, weight f32; coverage,
    # low, high uint16; dq int16)
    map_out = tuple(torch.empty((h, w), dtype=dt).pin_memory().numpy() for dt in (torch.float32, torch.float32))
    map_out += tuple(torch.empty((h, w), dtype=torch.int16).pin_memory().numpy().view(np.uint16) for _ in range(3))
    map_out += (torch.empty((h, w), dtype=torch.int16).pin_memory().numpy(),)
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(2):
        maps = pipe.step_host(pinned, register=True, out=map_out)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        maps = pipe.step_host(pinned, register=True, out=map_out)
    t1 = time.perf_counter()
    e2e_s = replicas.max_over_ranks(t1 - t0, torch.device("cuda", local))
    h2d = int(pinned.nbytes)
    d2h = int(sum(m.nbytes for m in maps if m is not None))
    e2e_value = replicas.replica_throughput(world, mpix_frames, e2e_steps, e2e_s)
    if not args.no_adjoint:
        # the same end-to-end step with the gradient refinement in place of the grid search
        pipe.config.refine_method = "gradient"
        for _ in range(2):
            pipe.step_host(pinned, register=True, out=map_out)
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            pipe.step_host(pinned, register=True, out=map_out)
        gn_s = replicas.max_over_ranks(time.perf_counter() - t0, torch.device("cuda", local))
        pipe.config.refine_method = "ncc"
        registration["e2e_mpix_frames_per_s"] = {
            "ncc_translation": e2e_value,
            "gradient_gauss_newton": replicas.replica_throughput(world, mpix_frames, e2e_steps, gn_s)}

    if rank != 0:
        return 0
    peak, peak_kind = measured_peak()
    kernels = {}
    for name, _, nbytes in stages:
        ms = stage_ms[name]
        if nbytes is None:  # latency-bound catalog work: no HBM roofline
            kernels[name] = {"ms": ms, "algorithmic_bytes": None, "achieved_gbs": None, "frac": None}
            continue
        gbs = nbytes / (ms / 1e3) / 1e9
        kernels[name] = {"ms": ms, "algorithmic_bytes": nbytes, "achieved_gbs": gbs, "frac": gbs / peak}
    top = max((k for k in kernels if kernels[k]["algorithmic_bytes"]), key=lambda k: kernels[k]["ms"])
    cpu = None
    if not args.no_cpu_baseline:
        t_cpu = time.perf_counter()
        rate, step_s, cpu_stages, desc = cpu_step_estimate(data, masters, 1)
        cpu = {"value": rate, "unit": "Mpix-frames/s", "cores": 1, "kind": "port",
               "sample": f"{desc}; sample took {time.perf_counter() - t_cpu:.1f} s, one step {step_s:.1f} s",
               "stages_s_per_step": cpu_stages}
    line = {
        "metric": metric,
        "value": value,
        "unit": "Mpix-frames/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": elapsed_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded generator, benchmark-config shapes and noise model)",
        "config": {"workload": workload, "frames": n, "height": h, "width": w,
                   "l2": "inputs larger than L2 (stack %.0f MB > 129 MB)" % (4 * n * h * w / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "kernel": top, "achieved": kernels[top]["achieved_gbs"], "peak": peak,
                     "unit": "GB/s", "frac": kernels[top]["frac"], "peak_source": peak_kind,
                     "traffic": profile_traffic(f"{top}_c2.md"),
                     "algorithmic_bytes_per_launch": kernels[top]["algorithmic_bytes"],
                     "launch_ms": kernels[top]["ms"]},
        "stages": kernels,
        "registration": registration,
        "graph_step": graph,
        "local_normalization": local_norm,
        "batched_stacks": batch,
        "large_stack_integration": large,
        "autotune": _lib.autotune_entries(),
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "Mpix-frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": 1e3 * e2e_s / e2e_steps},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line))
    pipe.close()
    replicas.shutdown()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
