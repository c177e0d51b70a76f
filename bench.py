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
    p.add_argument("--config", default="c2", choices=["c1", "c2"])
    p.add_argument("--frames", type=int, default=0, help="override frame count (smaller smoke runs)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
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
def _cpu_tile_job(args):
    raw, bias, dark, flat, scale, rejection = args
    from oracle.calibration import calibrate_light
    from oracle.integration import weighted_integrate_stack

    frames = np.stack([calibrate_light(raw[i], bias, dark, flat, 1.0, 1.0 / scale,
                                       master_dark_includes_bias=False) for i in range(raw.shape[0])])
    valid = np.isfinite(frames)
    means = np.array([frames[i][valid[i]].astype(np.float64).mean() for i in range(frames.shape[0])])
    stds = np.array([frames[i][valid[i]].astype(np.float64).std() for i in range(frames.shape[0])])
    weights = np.maximum(np.abs(means) / np.maximum(stds, 1e-6), 1e-6).astype(np.float32)
    weighted_integrate_stack(frames, weights, rejection)
    return int(raw.size)


def cpu_baseline(data, masters, seconds: float, processes: int):
    """Times the oracle port on crops of the workload for ~`seconds`."""
    import multiprocessing as mp

    n, h, w = data.lights.shape
    tile = 256
    jobs = []
    rng = np.random.default_rng(0)
    for _ in range(4096):
        y = int(rng.integers(0, h - tile + 1))
        x = int(rng.integers(0, w - tile + 1))
        sl = (slice(y, y + tile), slice(x, x + tile))
        jobs.append((data.lights[:, sl[0], sl[1]].copy(),
                     None if masters.bias is None else masters.bias[sl],
                     None if masters.dark is None else masters.dark[sl],
                     None if masters.flat is None else masters.flat[sl], 1.0, "winsorized_sigma"))
    done_px = 0
    start = time.perf_counter()
    if processes <= 1:
        for job in jobs:
            done_px += _cpu_tile_job(job)
            if time.perf_counter() - start >= seconds:
                break
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(processes) as pool:
            for px in pool.imap_unordered(_cpu_tile_job, jobs, chunksize=1):
                done_px += px
                if time.perf_counter() - start >= seconds:
                    pool.terminate()
                    break
    elapsed = time.perf_counter() - start
    return done_px / 1e6 / elapsed, elapsed, done_px


# ---------------------------------------------------------------------------
def main():
    args = parse_args()
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
        per_step = []
        for _ in range(args.warmup):
            cpu_baseline(data, m, 1.0, procs)
        for _ in range(args.steps):
            rate, elapsed, px = cpu_baseline(data, m, max(2.0, args.cpu_seconds / max(args.steps, 1)), procs)
            per_step.append((rate, elapsed, px))
        total_px = sum(p for _, _, p in per_step)
        total_t = sum(t for _, t, _ in per_step)
        value = total_px / 1e6 / total_t
        line = {
            "metric": metric, "value": value, "unit": "Mpix-frames/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total_t / max(len(per_step), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": workload, "sample": "random 256x256 crops x all frames"},
            "cpu_baseline": {"value": value, "unit": "Mpix-frames/s", "cores": procs, "kind": "port",
                             "sample": f"{total_px / 1e6:.1f} Mpix-frames in 256x256 crops of the workload"},
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

    stages = [
        ("calibrate", lambda: pipe.calibrate_device(dev_raw.data_ptr()), 6 * n * P + 12 * P),
        ("detect_stars", pipe.detect, 4 * n * P),
        ("register", register, None),
        ("refine_translation", refine, None),
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
    pinned = torch.from_numpy(data.lights.view(np.int16)).pin_memory().numpy().view(np.uint16)
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
        rate, elapsed, px = cpu_baseline(data, masters, args.cpu_seconds, 1)
        cpu = {"value": rate, "unit": "Mpix-frames/s", "cores": 1, "kind": "port",
               "sample": f"{px / 1e6:.1f} Mpix-frames (random 256x256 crops x {n} frames) in {elapsed:.1f} s, "
                         "oracle calibrate + simple_snr weights + winsorized integration"}
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
