"""Benchmark of the resident light-stack hot path on GB300.

Workload (default, c5): 200 uint16 frames of 9600 x 6422 (seeded synthetic,
rendered on the device: ~20,000 stars, sky drift, cosmic rays, 7 thin-cloud
frames; 20 bias / dark / flat frames) resident on one GPU -> fused decode +
calibration -> star catalogs -> triangle registration -> Gauss-Newton
refinement -> registration quality -> Lanczos3 warp -> simple_snr weights ->
winsorized sigma-clip weighted integration into the six maps.  Metric:
stacked Mpix-frames/s (N*H*W/1e6 per step / step time), plus the HBM roofline
of the dominant kernel, the end-to-end rate from pinned host memory to host
maps, and the CPU baseline (the oracle port of the reference's CPU path on a
bounded sample).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--config c5|c2|c1]

Under torchrun each rank processes its own stack (replicas: the path has no
exchange step), value = all ranks' Mpix-frames / max-over-ranks time.
`--impl reference` times the CPU oracle port of the reference algorithm on the
host cores instead (rank 0 only).
"""

from __future__ import annotations

import argparse
import ctypes
import gc
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
    p.add_argument("--config", default="c5", choices=["c1", "c2", "c5"],
                   help="c5 (default): the full 200 x 9600 x 6422 stack resident on one GPU; c1/c2: smaller stacks "
                        "with the side reports")
    p.add_argument("--frames", type=int, default=0, help="override frame count (smaller smoke runs)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-adjoint", action="store_true", help="skip the gradient-refinement registration report")
    p.add_argument("--no-side", action="store_true", help="c5: skip the c2 side report")
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


def settle_host_heap() -> None:
    """Collects once and moves every object alive now into the permanent
    generation (gc.freeze), so the cyclic collector later scans only objects
    made after this point.  A full collection over a heap with torch loaded
    takes about 50 ms; landing between two host-synchronised stages of a
    timed step (registration, refinement, quality read their results back)
    it leaves the GPU idle for that long.  Called before each timed region,
    after setup and warm-up."""
    gc.collect()
    gc.freeze()


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
CPU_TILE = 384  # side of the crop every frame of the CPU sample is cut to
_SAMPLE = None  # per worker process: the tile stack, its masters and truth


def cpu_sample_config(name: str, tile: int = CPU_TILE):
    """`name`'s model on a tile x tile crop: the same frame count, noise,
    defects and transforms, the star count scaled by area."""
    import dataclasses

    from glass_gb300.synthetic import CONFIGS

    cfg = CONFIGS[name]
    stars = max(8, int(round(cfg.stars * tile * tile / (cfg.height * cfg.width))))
    return dataclasses.replace(cfg, height=tile, width=tile, stars=stars)


def _sample_load(path: str) -> None:
    global _SAMPLE
    with np.load(path) as z:
        _SAMPLE = {k: z[k] for k in z.files}


def _sample_frames(job):
    """calibrate -> star catalog -> triangle registration to the reference
    catalog -> Lanczos3 warp -> frame statistics, for a chunk of frames
    (oracle port; the reference's CPU path for these stages)."""
    from oracle import registration, stars, warp
    from oracle.calibration import calibrate_light

    frames, ref_catalog = job
    d = _SAMPLE
    out = []
    for k in frames:
        cal = calibrate_light(d["lights"][k], d["bias"], d["dark"], d["flat"], 300.0, 300.0,
                              master_dark_includes_bias=False)
        found = stars.detect_stars(cal, threshold_sigma=5.0, max_stars=400)
        catalog = [(s[0], s[1]) for s in found if s[5] is not None and s[5] <= 0.8][:80]
        ok = k == 0
        if k:
            reg = registration.estimate_triangle_asterism_transform(ref_catalog, catalog)
            ok = reg["status"] == "ok"
            matrix = np.asarray(reg["matrix"], dtype=np.float64) if ok else d["truth"][k]
            cal, _cov = warp.warp_matrix(cal, matrix.astype(np.float32), "lanczos3", np.nan)
        finite = np.isfinite(cal)
        vals = cal[finite].astype(np.float64)
        mean, std = (float(vals.mean()), float(vals.std())) if vals.size else (0.0, 0.0)
        weight = max(abs(mean) / std, 1.0e-6) if std > 1.0e-6 else (1.0e6 if vals.size else 0.0)
        out.append((int(k), cal, float(weight) if ok else 0.0))
    return out


def _sample_integrate(job):
    from oracle.integration import weighted_integrate_stack

    band, weights = job
    return weighted_integrate_stack(band, weights, "winsorized_sigma")[0]


class CpuSample:
    """The oracle port of the reference's CPU path run on a bounded sample of
    the workload: every frame of `config_name` cut to a tile x tile crop of
    the same model, through calibration, star catalogs, triangle registration,
    Lanczos3 warp, simple_snr weights and winsorized 3/3 integration, spread
    over `processes` host processes (frames, then row bands).  One step() is
    one pass over the sample; its throughput is the sample's Mpix-frames over
    the step's wall time.  `start` is "fork" only in a process that has not
    touched CUDA; after CUDA it must be "spawn"."""

    def __init__(self, config_name: str, processes: int, start: str, tile: int = CPU_TILE):
        import multiprocessing as mp

        from glass_gb300.synthetic import generate
        from oracle.calibration import calibrate_light
        from oracle import stars

        cfg = cpu_sample_config(config_name, tile)
        data = generate(cfg)
        bias = data.bias_frames.astype(np.float64).mean(0).astype(np.float32)
        dark = (data.dark_frames.astype(np.float64).mean(0) - bias).astype(np.float32)
        flat = data.flat_frames.astype(np.float64).mean(0) - bias
        flat = np.maximum(flat / np.median(flat), 1.0e-6).astype(np.float32)
        self.frames, self.tile, self.processes = cfg.frames, tile, processes
        self.path = tempfile.NamedTemporaryFile(suffix=".npz", delete=False).name
        np.savez(self.path, lights=data.lights, bias=bias, dark=dark, flat=flat, truth=data.truth_matrices)
        _sample_load(self.path)
        ref = calibrate_light(data.lights[0], bias, dark, flat, 300.0, 300.0, master_dark_includes_bias=False)
        found = stars.detect_stars(ref, threshold_sigma=5.0, max_stars=400)
        self.ref_catalog = [(s[0], s[1]) for s in found if s[5] is not None and s[5] <= 0.8][:80]
        self.pool = mp.get_context(start).Pool(processes, initializer=_sample_load, initargs=(self.path,))
        self.description = (f"{self.frames} frames x {tile}x{tile} crop of the {config_name} model (stars scaled by "
                            f"area), oracle port of calibrate -> detect_stars -> triangle registration -> Lanczos3 "
                            f"warp -> simple_snr weights -> winsorized 3/3 integration on {processes} host "
                            f"process(es); no sub-pixel refinement (the reference CPU path has none)")

    def step(self) -> float:
        """One pass over the sample; returns its wall seconds."""
        t0 = time.perf_counter()
        chunks = [list(range(k, self.frames, self.processes)) for k in range(self.processes)]
        results = self.pool.map(_sample_frames, [(c, self.ref_catalog) for c in chunks if c])
        stack = np.empty((self.frames, self.tile, self.tile), np.float32)
        weights = np.zeros(self.frames, np.float32)
        for part in results:
            for k, frame, w in part:
                stack[k] = frame
                weights[k] = w
        bands = np.array_split(np.arange(self.tile), self.processes)
        self.pool.map(_sample_integrate, [(np.ascontiguousarray(stack[:, b]), weights) for b in bands if b.size])
        return time.perf_counter() - t0

    def mpix_frames(self) -> float:
        return self.frames * self.tile * self.tile / 1e6

    def close(self) -> None:
        self.pool.close()
        self.pool.join()
        try:
            os.unlink(self.path)
        except OSError:
            pass


def cpu_baseline_line(config_name: str, processes: int, start: str, steps: int = 1) -> dict:
    """cpu_baseline of the bench line: `steps` sample passes after one warm-up pass."""
    sample = CpuSample(config_name, processes, start)
    try:
        sample.step()
        secs = [sample.step() for _ in range(steps)]
    finally:
        sample.close()
    mean = float(np.mean(secs))
    return {"value": sample.mpix_frames() / mean, "unit": "Mpix-frames/s", "cores": processes, "kind": "port",
            "sample": f"{sample.description}; {mean:.2f} s per pass"}


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

    if pipe.frames > 512:
        return {"skipped": "the captured step graph takes at most 512 frames"}
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


C5_CLOUD_SLOTS = (23, 57, 88, 104, 131, 162, 190)  # the 7 thin-cloud frames (frame 0 is the reference)
# pixel-agreement gate of the c5 run: the reference's score with its default
# 200 ADU RMS scale, sampled every 4th pixel; the minimum (a plan setting in
# the reference, no default) sits between the clear frames' scores (cosmic
# rays dominate their RMS) and the thin-cloud frames' (2x sky)
C5_AGREEMENT = {"min_score": 0.02, "rms_scale_adu": 200.0, "action": "fail", "min_weight": 0.0, "sample_stride": 4}
C5_WORKLOAD = ("uint16 -> calibrate (20 bias/dark/flat) -> star catalogs -> triangle registration -> Gauss-Newton "
               "refinement -> registration quality (agreement score) -> Lanczos3 warp -> simple_snr weights -> "
               "winsorized 3/3 weighted integration (6 maps)")


def c5_config(n: int, h: int, w: int) -> dict:
    return {"workload": f"c5:{n}x{h}x{w} {C5_WORKLOAD}", "frames": n, "height": h, "width": w,
            "thin_cloud_frames": list(C5_CLOUD_SLOTS), "calibration_frames_per_kind": 20,
            "agreement_min_score": C5_AGREEMENT["min_score"],
            "l2": "inputs larger than L2 (raw stack %.1f GB, frames %.1f GB > 129 MB)" % (2 * n * h * w / 1e9,
                                                                                         4 * n * h * w / 1e9),
            "parallelism": "single GPU"}


def run_c5(args) -> int:
    """The headline: the full c5 stack resident on one GPU - 200 uint16
    frames of 9600 x 6422 (49.3 GB as float32 frames), 20 bias / dark / flat
    frames, ~20,000 stars per frame, sky drift +/-15 %, cosmic rays 1e-4,
    +/-40 px and +/-0.3 deg, and exactly 7 thin-cloud frames (50 % flux,
    2x sky) that the registration-quality policy must weight 0.  Every frame
    is rendered on the device (seeded).  `value`: CUDA events around K device
    steps on the raw stack already in HBM; `e2e`: the same step through the
    public API from pinned host uint16 to host maps."""
    import torch

    from glass_gb300 import _lib
    from glass_gb300.adjoint import registration_rms_px
    from glass_gb300.pipeline import ResidentPipeline, StepConfig, build_masters
    from glass_gb300.synthetic import CONFIGS, generate_device

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    replicas.init("nccl", torch.device("cuda", local))
    cfg = CONFIGS["c5"]
    n = args.frames or cfg.frames
    slots = [k for k in C5_CLOUD_SLOTS if k < n]
    t_gen = time.perf_counter()
    data = generate_device(cfg, n, cloud_slots=slots, device=f"cuda:{local}")
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t_gen
    _, h, w = data.lights.shape
    P = h * w
    masters = build_masters(data.bias_frames, data.dark_frames, data.flat_frames)
    pipe = ResidentPipeline(n, h, w, masters, StepConfig(star_max_stars=4096, refine_method="gradient",
                                                         agreement=dict(C5_AGREEMENT)))
    stream = torch.cuda.Stream()
    pipe.set_stream(stream.cuda_stream)
    dev_raw = data.lights
    truth = data.truth_matrices
    reg = {}

    def register():
        reg["triangle"], reg["ok"] = pipe.register(0)

    def refine():
        reg["m"] = pipe.refine(reg["triangle"], 0)

    def assess():
        reg["quality"] = pipe.assess(reg["m"], 0)

    sampled = -(-h // C5_AGREEMENT["sample_stride"]) * -(-w // C5_AGREEMENT["sample_stride"])
    stages = [("calibrate", lambda: pipe.calibrate_device(dev_raw.data_ptr()), 6 * n * P + 12 * P),
              ("detect_stars", pipe.detect, 4 * n * P),
              ("register", register, None),
              ("refine_gradient", refine, None),
              ("registration_quality", assess, 8 * (n - 1) * sampled),
              ("warp_lanczos3", lambda: pipe.warp(reg["m"]), 8 * (n - 1) * P),
              ("weights", pipe.weights, 4 * n * P),
              ("integrate_winsorized", pipe.integrate, 4 * n * P + 16 * P)]
    for _ in range(max(1, args.warmup)):
        for _, fn, _ in stages:
            fn()
    stream.synchronize()
    settle_host_heap()
    replicas.barrier()
    torch.cuda.synchronize()
    launches0 = _lib.kernel_launches()
    events = {name: [] for name, _, _ in stages}
    with ClockSampler(local) as clocks:
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clocks.mark_start()
        start.record(stream)
        for _ in range(args.steps):
            torch.cuda.nvtx.range_push("timed_step")  # lets a profiler keep only the timed steps' kernels
            for name, fn, _ in stages:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                events[name].append((e0, e1))
            torch.cuda.nvtx.range_pop()
        stop.record(stream)
        stream.synchronize()
        clocks.mark_stop()
    torch.cuda.synchronize()
    replicas.barrier()
    launches = _lib.kernel_launches() - launches0
    elapsed_ms = replicas.max_over_ranks(start.elapsed_time(stop), torch.device("cuda", local))
    mpix = n * P / 1e6
    value = replicas.replica_throughput(world, mpix, args.steps, elapsed_ms / 1e3)
    peak, peak_kind = measured_peak()
    out_stages = {}
    for name, _, nbytes in stages:
        t = statistics.mean(a.elapsed_time(b) for a, b in events[name])
        gbs = None if nbytes is None else nbytes / (t / 1e3) / 1e9
        out_stages[name] = {"ms": t, "algorithmic_bytes": nbytes, "achieved_gbs": gbs,
                            "frac": None if gbs is None else gbs / peak}
    weights = pipe.stack.device_frame_weights()
    ok = [k for k in range(1, n) if reg["ok"][k]]

    # ---- end to end through the public API: pinned host uint16 in, host maps out ----
    # reused page-locked destinations of the six maps, allocated before the
    # 24.7 GB raw buffer; the tensors stay referenced for the whole loop
    map_tensors = [torch.empty((h, w), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    map_tensors += [torch.empty((h, w), dtype=torch.int16, pin_memory=True) for _ in range(4)]
    map_out = tuple(t.numpy() for t in map_tensors[:2])
    map_out += tuple(t.numpy().view(np.uint16) for t in map_tensors[2:5])
    map_out += (map_tensors[5].numpy(),)
    pinned = torch.empty((n, h, w), dtype=torch.int16, pin_memory=True)
    for k in range(n):
        pinned[k].copy_(dev_raw[k])
    host_raw = pinned.numpy().view(np.uint16)
    e2e_steps = max(3, min(args.steps, 10))
    pipe.step_host(host_raw, register=True, out=map_out)
    settle_host_heap()
    replicas.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        # the next step's raw frames start uploading once this step has
        # calibrated its own (every step still copies its 24.7 GB inside the
        # timed region; the last step prefetches nothing)
        maps = pipe.step_host(host_raw, register=True, out=map_out,
                              prefetch=host_raw if k + 1 < e2e_steps else None)
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0, torch.device("cuda", local))
    e2e_value = replicas.replica_throughput(world, mpix, e2e_steps, e2e_s)
    h2d = int(host_raw.nbytes)
    d2h = int(sum(m.nbytes for m in maps if m is not None))
    e2e_weights = pipe.stack.device_frame_weights()
    del pinned, host_raw, map_tensors

    rms_tri = registration_rms_px([reg["triangle"][k] for k in ok], [truth[k] for k in ok], h, w)
    rms_gn = registration_rms_px([reg["m"][k] for k in ok], [truth[k] for k in ok], h, w)
    refinement = getattr(pipe, "last_refinement", [])
    qual = reg.get("quality", [])
    cloud = [int(k) for k in slots]
    registration = {
        "frames_ok": len(ok) + 1, "frames": n,
        "inliers_median": float(np.median([r["inliers"] for r in pipe.last_registration])),
        "rms_px_vs_truth": {"triangle": rms_tri, "gradient_gauss_newton": rms_gn},
        "refine_status": {str(v): sum(1 for r in refinement if r.get("status") == v)
                          for v in sorted({r.get("status") for r in refinement})},
        "quality": {"thin_cloud_frames": cloud,
                    "thin_cloud_weights": [float(weights[k]) for k in cloud],
                    "zero_weight_frames": [int(k) for k in range(n) if weights[k] <= 0.0],
                    "e2e_zero_weight_frames": [int(k) for k in range(n) if e2e_weights[k] <= 0.0],
                    "score_clear": _quantiles([q["score"] for q in qual if q.get("score") is not None
                                               and q["frame"] not in cloud]),
                    "score_cloud": _quantiles([q["score"] for q in qual if q.get("score") is not None
                                               and q["frame"] in cloud])}}
    stack_bytes = pipe.stack.bytes_allocated
    pipe.close()
    del dev_raw, data
    torch.cuda.empty_cache()
    side = {}
    if not args.no_side:
        for name, fn in (("c2", lambda: c2_side_report(local, max(3, min(args.steps, 10)))),
                         ("c3", lambda: c3_side_report(local)), ("c4", lambda: c4_side_report(local))):
            try:
                side[name] = fn()
            except Exception as exc:  # a side report must not lose the headline line
                side[name] = {"error": f"{type(exc).__name__}: {exc}"}
            torch.cuda.empty_cache()
    if rank != 0:
        replicas.shutdown()
        return 0
    top = max((k for k in out_stages if out_stages[k]["algorithmic_bytes"]), key=lambda k: out_stages[k]["ms"])
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline_line("c5", os.cpu_count() or 1, "spawn")
    line = {
        "metric": "stacked Mpix-frames/s", "value": value, "unit": "Mpix-frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (every frame rendered on the device from the seeded c5 model)",
        "config": c5_config(n, h, w),
        "roofline": {"bound": "hbm", "kernel": top, "achieved": out_stages[top]["achieved_gbs"], "peak": peak,
                     "unit": "GB/s", "frac": out_stages[top]["frac"], "peak_source": peak_kind,
                     "traffic": profile_traffic(f"{top}_c5.md"),
                     "algorithmic_bytes_per_launch": out_stages[top]["algorithmic_bytes"],
                     "launch_ms": out_stages[top]["ms"]},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "Mpix-frames/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": 1e3 * e2e_s / e2e_steps},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "stages": out_stages,
        "registration": registration,
        "resident": {"stack_bytes_allocated": stack_bytes, "generate_s": gen_s},
        "side_reports": side,
    }
    print(json.dumps(line))
    replicas.shutdown()
    return 0


def _quantiles(values) -> dict:
    if not values:
        return {}
    v = np.asarray(values, dtype=np.float64)
    return {"min": float(v.min()), "median": float(np.median(v)), "max": float(v.max()), "n": int(v.size)}


def c2_side_report(local: int, steps: int) -> dict:
    """The 32 x 2048 x 2048 stack (c2 model, rendered on the device): the same
    device step as the headline (Gauss-Newton refinement, quality policy in
    audit mode), CUDA events over `steps` steps."""
    import torch

    from glass_gb300.pipeline import ResidentPipeline, StepConfig, build_masters
    from glass_gb300.synthetic import generate_device

    data = generate_device("c2", device=f"cuda:{local}")
    n, h, w = data.lights.shape
    masters = build_masters(data.bias_frames, data.dark_frames, data.flat_frames)
    pipe = ResidentPipeline(n, h, w, masters, StepConfig(refine_method="gradient"))
    stream = torch.cuda.Stream()
    pipe.set_stream(stream.cuda_stream)
    try:
        def step():
            pipe.calibrate_device(data.lights.data_ptr())
            pipe.detect()
            m, _ = pipe.register(0)
            m = pipe.refine(m, 0)
            pipe.assess(m, 0)
            pipe.warp(m)
            pipe.weights()
            pipe.integrate()

        for _ in range(2):
            step()
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1) / steps
    finally:
        pipe.close()
    return {"workload": f"c2:{n}x{h}x{w} (same step as the headline)", "ms_per_step": ms,
            "mpix_frames_per_s": n * h * w / 1e6 / (ms / 1e3), "steps": steps}


def c3_side_report(local: int, frames: int = 64, size: int = 4096) -> dict:
    """Differentiable registration on 64 calibrated float32 frames of 4096 x
    4096 (~30 stars per 128 x 128, true affine = I + N(0, 1e-3) on the
    linear terms, +-0.5 px shifts): the catalog-matching start (triangle
    similarity, the plain registration; and the same catalogs with the affine
    model, alone and followed by the device Gauss-Newton) against three
    refinements on the same
    GPU and frames - the NCC translation grid (the reference's), the device
    Gauss-Newton (affine model, 20 steps at most) and L-BFGS on the masked NCC of the star
    regions with every gradient from the hand-written warp adjoint behind
    torch.autograd (20 evaluations at most; timed after one untimed warm-up
    call) - as RMS distance to the true maps (px) and wall time."""
    import torch

    from glass_gb300.adjoint import LbfgsConfig, refine_affine_lbfgs, registration_rms_px, star_region_mask
    from glass_gb300.pipeline import DEFAULT_REFINE, Masters, ResidentPipeline, StepConfig
    from glass_gb300.synthetic import render_affine_device

    dev = f"cuda:{local}"
    images, truth = render_affine_device(frames, size, size, device=dev)
    pipe = ResidentPipeline(frames, size, size, Masters(None, None, None),
                            StepConfig(refine=dict(DEFAULT_REFINE)))
    stream = torch.cuda.Stream()
    pipe.set_stream(stream.cuda_stream)
    try:
        for k in range(frames):
            pipe.stack.upload_calibrated_frame(k, images[k].cpu().numpy())
        del images
        torch.cuda.synchronize()

        def timed(fn):
            stream.synchronize()
            t0 = time.perf_counter()
            out = fn()
            stream.synchronize()
            torch.cuda.synchronize()
            return out, time.perf_counter() - t0

        def catalog():
            pipe.detect()
            return pipe.register(0)

        (tri, ok), t_plain = timed(catalog)
        good = [k for k in range(1, frames) if ok[k]]

        def rms(mats):
            return registration_rms_px([mats[k] for k in good], [truth[k] for k in good], size, size)

        out = {"frames": frames, "size": size, "registered": len(good) + 1,
               "plain_catalog_similarity": {"rms_px": rms(tri), "s": t_plain}}
        # the same catalogs with the reference's affine model
        pipe.config.registration_model = "affine"
        (aff, ok_aff), t_aff = timed(lambda: pipe.register(0))
        pipe.config.registration_model = "similarity"
        out["plain_catalog_affine"] = {"rms_px": rms(aff), "s": t_aff,
                                       "registered": int(sum(ok_aff[k] for k in range(1, frames))) + 1}
        pipe.config.refine_method = "ncc"
        ncc, t = timed(lambda: pipe.refine(tri, 0))
        out["ncc_translation_grid"] = {"rms_px": rms(ncc), "s": t}
        pipe.config.refine_method = "gradient"
        pipe.config.gradient_refine = {"model": "affine", "iterations": 20}
        gn, t = timed(lambda: pipe.refine(tri, 0))
        out["device_gauss_newton_affine"] = {"rms_px": rms(gn), "s": t}
        # Gauss-Newton from the affine catalog solution (inside its capture range)
        gna, t = timed(lambda: pipe.refine(aff, 0))
        out["affine_catalog_then_gauss_newton"] = {"rms_px": rms(gna), "s": t + t_aff}
        ref = pipe.stack.frame_tensor(0)
        cfg = LbfgsConfig(iterations=20)

        def lbfgs():
            mask = star_region_mask(ref, cfg.star_sigma, cfg.star_radius_px, cfg.border_px)
            mats = np.array(tri, dtype=np.float64, copy=True)
            evals = []
            with torch.cuda.stream(stream):
                for k in good:
                    res = refine_affine_lbfgs(ref, pipe.stack.frame_tensor(k), tri[k], cfg, mask=mask)
                    mats[k] = res.matrix
                    evals.append(res.evaluations)
            return mats, evals

        # one untimed call first: the first autograd / L-BFGS use in a process
        # costs seconds of one-time setup that no later frame pays
        with torch.cuda.stream(stream):
            refine_affine_lbfgs(ref, pipe.stack.frame_tensor(good[0]), tri[good[0]], LbfgsConfig(iterations=2))
        (adj, evals), t = timed(lbfgs)
        out["adjoint_lbfgs_masked_ncc"] = {"rms_px": rms(adj), "s": t, "evaluations_mean": float(np.mean(evals)),
                                           "evaluations_max": int(np.max(evals))}
        return out
    finally:
        pipe.close()


C4_STACKS = (  # name, frames, height, width, interpolation, rejection
    ("A", 40, 2000, 3000, "bilinear", "winsorized"),
    ("B", 120, 4000, 6000, "lanczos3", "winsorized"),
    ("C", 25, 1024, 1024, "lanczos3", "linear_fit"),
)


def c4_side_report(local: int, reps: int = 3) -> dict:
    """Batched uneven stacks: A 40 x 3000 x 2000 (bilinear, winsorized 3/3),
    B 120 x 6000 x 4000 (Lanczos3, winsorized 3/3) and C 25 x 1024 x 1024
    (Lanczos3, linear-fit clipping), raw uint16 rendered with the 8-frame
    config's noise model (30 stars per 128 x 128, sky 1000, pedestal 500,
    integer shifts +-5 px, 4 calibration frames of each kind).  Each stack's
    calibrate -> simple_snr weights -> warp -> rejection + integration runs
    eagerly stack after stack (CUDA events per stack) and as one CUDA graph
    of all three (gg_stacks_graph_capture); the replayed maps are compared
    with the eager ones bit for bit."""
    import dataclasses

    import torch

    from glass_gb300 import _glass_cuda_native as native
    from glass_gb300 import _lib
    from glass_gb300.pipeline import build_masters
    from glass_gb300.synthetic import CONFIGS, generate_device

    rejections = {"winsorized": _lib.GG_REJECT_WINSORIZED, "linear_fit": _lib.GG_REJECT_LINEAR_FIT}
    interps = {"bilinear": _lib.GG_INTERP_BILINEAR, "lanczos3": _lib.GG_INTERP_LANCZOS3}
    stream = torch.cuda.Stream()
    peak, _ = measured_peak()
    stacks, raws, mats, steps = [], [], [], []
    try:
        for k, (name, n, h, w, interp, rej) in enumerate(C4_STACKS):
            cfg = dataclasses.replace(CONFIGS["c1"], frames=n, height=h, width=w,
                                      stars=int(round(30 * h * w / 128.0 ** 2)), seed=40 + k)
            data = generate_device(cfg, n, device=f"cuda:{local}")
            masters = build_masters(data.bias_frames, data.dark_frames, data.flat_frames)
            s = native.ResidentCalibratedStack(n, h, w)
            s.set_stream(stream.cuda_stream)
            s.set_calibration_masters(masters.bias, masters.dark, masters.flat)
            stacks.append(s)
            raws.append(data.lights)
            mats.append(np.asarray(data.truth_matrices))
            steps.append({"stack": s, "dev_raw": data.lights.data_ptr(), "matrices": mats[-1],
                          "interpolation": interp, "rejection": rejections[rej],
                          "calib": _lib.CalibParams(0, 1.0, 1.0e-6, 0.0)})
        torch.cuda.synchronize()

        def eager(k):
            st, s = steps[k], stacks[k]
            n = s.frame_count
            idx = np.arange(n, dtype=np.int64)
            _lib.call("gg_stack_calibrate_u16_device", s.handle, _lib.ptr(idx), ctypes.c_int64(n),
                      ctypes.c_void_p(st["dev_raw"]), 0, ctypes.byref(st["calib"]))
            s.compute_frame_weights("simple_snr", None, 1.0e-6, download=False)
            moving = np.array([f for f in range(n) if not np.array_equal(mats[k][f], np.eye(3))], dtype=np.int64)
            s.warp_frames_async(moving, mats[k][moving], interps[st["interpolation"]], np.nan, -1.0, False)
            s.integrate_async("device", st["rejection"], 3.0, 3.0, 3, 0.5, "uint16")

        for k in range(len(stacks)):  # warm-up (autotuner, buffers)
            eager(k)
        stream.synchronize()
        per_stack = {}
        eager_maps = []
        t_seq = 0.0
        for k, (name, n, h, w, interp, rej) in enumerate(C4_STACKS):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                eager(k)
            e1.record(stream)
            stream.synchronize()
            ms = e0.elapsed_time(e1) / reps
            t_seq += ms
            eager_maps.append(stacks[k].download_maps("full", include_dq=True))
            P = h * w
            warped = sum(1 for f in range(n) if not np.array_equal(mats[k][f], np.eye(3)))
            nbytes = (6 * n * P + 12 * P) + 4 * n * P + 8 * warped * P + (4 * n * P + 16 * P)
            per_stack[name] = {"frames": n, "height": h, "width": w, "interpolation": interp, "rejection": rej,
                               "ms": ms, "mpix_frames_per_s": n * P / 1e6 / (ms / 1e3),
                               "algorithmic_bytes": nbytes, "achieved_gbs": nbytes / (ms / 1e3) / 1e9,
                               "frac_of_measured_hbm": nbytes / (ms / 1e3) / 1e9 / peak}
        graph = native.StacksGraph(steps, stream.cuda_stream)
        try:
            graph.launch()
            stream.synchronize()
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            for _ in range(reps):
                graph.launch()
            g1.record(stream)
            stream.synchronize()
            t_graph = g0.elapsed_time(g1) / reps
            identical = all(all(np.array_equal(a, b) for a, b in zip(stacks[k].download_maps("full", include_dq=True),
                                                                  eager_maps[k]))
                            for k in range(len(stacks)))
            kernels = graph.kernel_count
        finally:
            graph.close()
        total = sum(v["frames"] * v["height"] * v["width"] for v in per_stack.values())
        return {"stacks": per_stack, "sequential_eager_ms": t_seq, "graph_ms": t_graph,
                "graph_kernels": kernels, "graph_maps_identical_to_eager": identical,
                "mpix_frames_per_s_graph": total / 1e6 / (t_graph / 1e3)}
    finally:
        for s in stacks:
            s.close()


def run_reference(args) -> int:
    """--impl reference: the oracle port of the reference's CPU path (the
    reference itself is not on the GPU host) on all host cores, rank 0 only,
    no CUDA.  Each step is one pass over the bounded sample of the workload
    (every frame cut to a 384 x 384 crop of the same model); `value` is the
    sample's Mpix-frames over the mean step time."""
    rank, _world, _local = dist_env()
    if rank != 0:
        return 0
    from glass_gb300.synthetic import CONFIGS

    cfg = CONFIGS[args.config]
    n = args.frames or cfg.frames
    procs = os.cpu_count() or 1
    sample = CpuSample(args.config, procs, "fork")
    try:
        for _ in range(args.warmup):
            sample.step()
        settle_host_heap()
        secs = [sample.step() for _ in range(args.steps)]
    finally:
        sample.close()
    step_s = float(np.mean(secs))
    value = sample.mpix_frames() / step_s
    config = c5_config(n, cfg.height, cfg.width) if args.config == "c5" else c2_config(args.config, n, cfg)
    line = {"metric": "stacked Mpix-frames/s", "value": value, "unit": "Mpix-frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": config,
            "cpu_baseline": {"value": value, "unit": "Mpix-frames/s", "cores": procs, "kind": "port",
                             "sample": sample.description},
            "e2e": {"value": value, "unit": "Mpix-frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def c2_config(name: str, n: int, cfg) -> dict:
    return {"workload": f"{name}:{n}x{cfg.height}x{cfg.width} uint16 -> calibrate -> star catalogs -> triangle "
                        f"registration -> sub-pixel translation refinement -> Lanczos3 warp -> simple_snr weights -> "
                        f"winsorized 3/3 weighted integration (6 maps)",
            "frames": n, "height": cfg.height, "width": cfg.width,
            "l2": "inputs larger than L2 (stack %.0f MB > 129 MB)" % (4 * n * cfg.height * cfg.width / 1e6),
            "parallelism": "single GPU"}


# ---------------------------------------------------------------------------
def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "c5":
        return run_c5(args)
    return run_c2(args)


def run_c2(args) -> int:
    """--config c1 / c2: the smaller stack with the NCC candidate-grid
    refinement (the reference's resident default) and the side reports
    (registration accuracy, CUDA graph, local normalisation, batched stacks,
    200-frame integration, autotune)."""
    rank, world, local = dist_env()
    from glass_gb300.synthetic import CONFIGS, generate

    cfg = CONFIGS[args.config]
    frames = args.frames or cfg.frames
    metric = "stacked Mpix-frames/s"
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
    settle_host_heap()
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
    settle_host_heap()
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
        cpu = cpu_baseline_line(args.config, os.cpu_count() or 1, "spawn")
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
        "config": dict(c2_config(args.config, n, cfg), parallelism="replicas" if world > 1 else "single GPU"),
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
