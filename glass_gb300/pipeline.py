"""Host orchestration of the resident hot path on one GPU.

Mirrors the order of the resident run (src/glass/engine/resident_cuda.py:
ResidentCalibratedStack at :7667, set_calibration_masters :8542, calibrate
:8974-9280, star catalogs :10798-10950, triangle match :11220-11400, warp
:11466/12505, weights :12762-12785, integrate :13294-13460) for a stack whose
raw frames are already in memory.  Every stage is a call into
libglass_gb300.so; all work is enqueued on the stack's stream, so a whole
step can run without a host synchronisation (and be captured in a CUDA
graph) until the maps are downloaded.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from glass_gb300 import _lib
from glass_gb300._glass_cuda_native import ResidentCalibratedStack


@dataclass
class Masters:
    bias: np.ndarray | None
    dark: np.ndarray | None
    flat: np.ndarray | None


def build_masters(bias_frames: np.ndarray | None, dark_frames: np.ndarray | None,
                  flat_frames: np.ndarray | None, flat_floor: float = 1.0e-6, method: str = "mean",
                  low_sigma: float = 3.0, high_sigma: float = 3.0) -> Masters:
    """Master bias / dark / flat on the GPU (cpu/master_frames.py:97-165;
    resident _stack_resident_master_array_with_resident_cuda_{mean,
    hardened_winsorized}, resident_cuda.py:6150, 6351).

    Each master is the mean of its frames ("mean": the stack integrator with
    no rejection, float64-exact sums) or their winsorized sigma-clipped mean
    ("winsorized": low_sigma / high_sigma, min 3 samples, at most half
    rejected); the dark has the master bias subtracted and the flat is
    bias-subtracted, divided by its median and floored.
    """
    if method not in ("mean", "winsorized"):
        raise ValueError("method must be mean or winsorized")

    def combine(frames: np.ndarray) -> np.ndarray:
        n, h, w = frames.shape
        stack = ResidentCalibratedStack(n, h, w)
        try:
            raw = np.ascontiguousarray(frames.astype(np.uint16, copy=False))
            params = _lib.CalibParams(1, 1.0, 1.0e-6, 0.0)
            idx = np.arange(n, dtype=np.int64)
            _lib.call("gg_stack_calibrate_u16", stack.handle, _lib.ptr(idx), ctypes.c_int64(n), _lib.ptr(raw), 0,
                      ctypes.byref(params))
            if method == "mean":
                master, _ = stack.integrate_mean()
            else:
                master = stack.integrate_hardened_winsorized_sigma(None, low_sigma, high_sigma, 3, 0.5,
                                                                   download_mode="master_only")[0]
        finally:
            stack.close()
        return master

    bias = combine(bias_frames) if bias_frames is not None else None
    dark = None
    if dark_frames is not None:
        dark = combine(dark_frames)
        if bias is not None:
            dark = (dark - bias).astype(np.float32)
    flat = None
    if flat_frames is not None:
        flat = combine(flat_frames)
        if bias is not None:
            flat = (flat - bias).astype(np.float32)
        norm = float(np.median(flat))
        if abs(norm) < flat_floor:
            raise ValueError("flat normalization is below flat_floor")
        flat = np.maximum(flat / norm, flat_floor).astype(np.float32)
    return Masters(bias, dark, flat)


@dataclass
class StepConfig:
    rejection: int = _lib.GG_REJECT_WINSORIZED
    low_sigma: float = 3.0
    high_sigma: float = 3.0
    min_samples: int = 3
    max_reject_fraction: float = 0.5
    weighting: str = "simple_snr"
    count_map_dtype: str = "uint16"
    interpolation: str = "lanczos3"
    clamping_threshold: float = -1.0
    light_exposure_s: float = 300.0
    dark_exposure_s: float | None = 300.0
    # star catalogs + triangle registration (resident_cuda.py:10790-11400)
    star_threshold_sigma: float = 5.0
    star_max_stars: int = 400
    # registration catalog = first 80 detections that look like stars: cosmic
    # ray streaks are elongated (eccentricity near 1), stars round
    catalog_min_fwhm: float = 0.0
    catalog_max_eccentricity: float = 0.8
    # 0: the reference's global median / MAD threshold; 8..64: background
    # mesh of that cell size (local threshold, local background per star)
    background_mesh_cell: int = 0
    # grid local normalisation between warp and integration (the resident
    # grid_mean_std mode; 256 is the reference CLI's tile), 0 = off
    local_normalization_tile: int = 0
    registration_tolerance_px: float = 3.0
    registration_min_inliers: int = 6
    # "similarity" (the resident triangle path) or "affine" (3-point affine
    # hypotheses and least-squares affine refits, cpu/registration.py:106-119)
    registration_model: str = "similarity"
    # sub-pixel translation refinement of the triangle matrices (a coarse
    # +-1 px grid of 0.25 px at stride 4, then +-0.25 px of 0.0625 px at
    # stride 8: the resident run's settings); None skips it
    refine: dict | None = None
    # "ncc": the reference's translation grid search (refine above);
    # "gradient": device Gauss-Newton on the masked sum of squares with the
    # warp adjoint's derivatives (gradient_refine below)
    refine_method: str = "ncc"
    gradient_refine: dict | None = None
    # registration-quality weighting (glass_gb300.quality): pixel-agreement
    # score of each frame's final matrix against the reference (NCC and RMS
    # of the alignment metrics at `sample_stride`), its minimum (None: audit
    # only), the action on a miss and the downweight floor; then the
    # inlier / fit-RMS gate ("auto": exclude for this triangle mode)
    agreement: dict | None = None
    quality_action: str = "auto"
    quality_min_inliers: int = 4
    quality_max_rms_px: float | None = None


DEFAULT_AGREEMENT = {"min_score": None, "rms_scale_adu": 200.0, "action": "fail", "min_weight": 0.0,
                     "sample_stride": 8}

DEFAULT_REFINE = {"search_radius_px": 1.0, "coarse_step_px": 0.25, "fine_radius_px": 0.25, "fine_step_px": 0.0625,
                  "coarse_sample_stride": 4, "final_sample_stride": 8}

# similarity model, Lanczos3 derivatives, every 3rd row and column (or, on a
# frame where that grid would exceed target_samples, whole rows spaced to
# about target_samples pixels), three noise passes on a grid twice as coarse,
# at most five steps, stop below 1e-3 px
# Gauss-Newton defaults.  On the 200-frame 9600 x 6422 stack (registration
# error 0.0146 px RMS against the rendered truth) three statistics passes and
# a 1e-3 px step tolerance gave the same error in 33.6 ms with 6 frames at the
# iteration cap; two passes and 3e-3 px take 27.6 ms and every frame converges.
DEFAULT_GRADIENT_REFINE = {"model": "similarity", "interpolation": "lanczos3", "sample_stride": 3,
                           "target_samples": 1_000_000, "stats_passes": 2, "iterations": 5, "min_samples": 256,
                           "clip_sigma": 5.0, "mask_shift_px": 1.0, "tolerance_px": 3.0e-3, "max_step_px": 2.0}


def gradient_sample_grid(params: dict, height: int, width: int) -> tuple[int, int]:
    """(sample_stride, row_stride) of the gradient refinement on a frame of
    height x width: the square grid of params["sample_stride"] while it holds
    at most params["target_samples"] pixels (None: no limit), else whole rows
    (column step 1) spaced so that about target_samples pixels are sampled.
    A warp then reads consecutive pixels of a row and its Lanczos windows
    overlap, where a sparse square grid touches one pixel per 32-byte sector
    and re-reads nothing."""
    stride = int(params["sample_stride"])
    target = params.get("target_samples")
    if target and -(-height // stride) * -(-width // stride) > target:
        rows = int(np.ceil(height * width / float(target)))
        return 1, int(min(max(rows, 1), 4096))
    return stride, stride


class ResidentPipeline:
    """One resident stack plus the per-step stage sequence."""

    def __init__(self, frames: int, height: int, width: int, masters: Masters, config: StepConfig | None = None):
        self.stack = ResidentCalibratedStack(frames, height, width)
        self.stack.set_calibration_masters(masters.bias, masters.dark, masters.flat)
        self.config = config or StepConfig()
        self.frames = frames
        self.height = height
        self.width = width
        self._indices = np.arange(frames, dtype=np.int64)
        self._params = None
        self.staged_chunks = 1

    def set_stream(self, cuda_stream: int | None) -> None:
        self.stack.set_stream(cuda_stream)

    def _calib_params(self) -> _lib.CalibParams:
        if self._params is None:
            cfg = self.config
            has_dark = bool(self.stack._info().has_dark)
            scale = 1.0
            if has_dark and cfg.dark_exposure_s not in (None, 0):
                scale = float(cfg.light_exposure_s) / float(cfg.dark_exposure_s)
            # build_masters subtracts the bias from the dark, so the bias is
            # removed separately (master_dark_includes_bias = False).
            self._params = _lib.CalibParams(0, scale, 1.0e-6, 0.0)
        return self._params

    # ---- stages (all asynchronous on the stack stream) ------------------------
    def calibrate_device(self, dev_raw_ptr: int) -> None:
        """uint16 frames already in device memory -> calibrated stack."""
        _lib.call("gg_stack_calibrate_u16_device", self.stack.handle, _lib.ptr(self._indices),
                  ctypes.c_int64(self.frames), ctypes.c_void_p(dev_raw_ptr), 0, ctypes.byref(self._calib_params()))

    def upload_raw(self, host_raw: np.ndarray) -> None:
        """Enqueues the host-to-device copies of every frame's raw uint16
        samples (page-locked host memory) and returns at once; calibrate_staged
        then waits, on the device, for the frames it calibrates."""
        _lib.call("gg_stack_upload_raw_u16", self.stack.handle, _lib.ptr(self._indices), ctypes.c_int64(self.frames),
                  _lib.ptr(host_raw))

    def calibrate_staged(self, frames) -> None:
        """Calibrates `frames` from their staged raw samples (upload_raw)."""
        idx = np.ascontiguousarray(np.asarray(frames, dtype=np.int64))
        _lib.call("gg_stack_calibrate_u16_staged", self.stack.handle, _lib.ptr(idx), ctypes.c_int64(idx.size), 0,
                  ctypes.byref(self._calib_params()))

    def calibrate_host(self, host_raw: np.ndarray) -> None:
        """uint16 frames in host memory (pinned for full-speed copies)."""
        _lib.call("gg_stack_calibrate_u16", self.stack.handle, _lib.ptr(self._indices),
                  ctypes.c_int64(self.frames), _lib.ptr(host_raw), 0, ctypes.byref(self._calib_params()))

    def detect(self, info: bool = False, frames=None) -> list[dict] | None:
        """Star catalogs of every frame (or of `frames`); they stay on the
        device for register().  info=True also returns each frame's background
        statistics, candidate count and catalog size."""
        cfg = self.config
        indices = self._indices if frames is None else np.ascontiguousarray(np.asarray(frames, dtype=np.int64))
        params = _lib.StarParams(float(cfg.star_threshold_sigma), int(cfg.star_max_stars), 4, 2.0, np.nan, np.nan,
                                 float(cfg.catalog_min_fwhm), float(cfg.catalog_max_eccentricity),
                                 int(cfg.background_mesh_cell))
        host_info = (_lib.StarFrameInfo * indices.size)() if info else None
        counts = np.zeros(indices.size, dtype=np.int32) if info else None
        _lib.call("gg_stack_detect_stars", self.stack.handle, _lib.ptr(indices), ctypes.c_int64(indices.size),
                  ctypes.byref(params), None, None if counts is None else _lib.ptr(counts), host_info)
        if not info:
            return None
        return [{"frame": int(k), "median": float(r.median), "noise": float(r.noise), "threshold": float(r.threshold),
                 "candidates": int(r.candidates), "stars": int(counts[pos])}
                for pos, (k, r) in enumerate(zip(indices, host_info))]

    def register(self, reference_index: int = 0, frames=None) -> tuple[np.ndarray, np.ndarray]:
        """Triangle registration of every frame to the reference frame from the
        device catalogs -> (matrices [frames, 3, 3], ok [frames]).  Frames that
        fail keep the identity matrix and are weighted 0 by weights().  With
        `frames`, only those are registered and the earlier results of the
        others are kept (chunked processing; start with a call that includes
        the reference frame or with frames=None)."""
        cfg = self.config
        models = {"similarity": _lib.GG_TRANSFORM_SIMILARITY, "affine": _lib.GG_TRANSFORM_AFFINE}
        if cfg.registration_model not in models:
            raise ValueError("registration_model must be similarity or affine")
        params = _lib.RegisterParams(models[cfg.registration_model], int(cfg.registration_min_inliers),
                                     float(cfg.registration_tolerance_px), 0.1, 80, 5, 1200, 1500)
        subset = list(range(self.frames)) if frames is None else [int(k) for k in frames]
        idx = np.array([i for i in subset if i != reference_index], dtype=np.int64)
        fresh = frames is None or reference_index in subset or getattr(self, "_reg_matrices", None) is None
        if fresh:
            self._reg_matrices = np.tile(np.eye(3), (self.frames, 1, 1))
            self._registered = np.ones(self.frames, dtype=bool)
            self._accepted = self._registered.copy()
            self._multipliers = np.ones(self.frames, dtype=np.float64)
            self.last_registration = []
            self.last_refinement = []
            self.last_quality = []
        matrices, ok = self._reg_matrices, self._registered
        if idx.size:
            out = (_lib.Registration * idx.size)()
            _lib.call("gg_stack_register_frames", self.stack.handle, ctypes.c_int64(int(reference_index)),
                      _lib.ptr(idx), ctypes.c_int64(idx.size), ctypes.byref(params), out)
            for pos, k in enumerate(idx):
                ok[k] = out[pos].status == 1
                matrices[k] = np.asarray(out[pos].matrix, dtype=np.float64).reshape(3, 3) if ok[k] else np.eye(3)
                self._accepted[k] = ok[k]
                self._multipliers[k] = 1.0
            self.last_registration = [r for r in self.last_registration if r["frame"] not in set(idx.tolist())] + [
                {"frame": int(k), "status": int(r.status), "inliers": int(r.inliers), "matches": int(r.matches),
                 "descriptors_reference": int(r.descriptors_reference),
                 "descriptors_moving": int(r.descriptors_moving), "rms_px": float(r.rms_px)}
                for k, r in zip(idx, out)]
        return matrices.copy(), ok.copy()

    def refine(self, matrices: np.ndarray, reference_index: int = 0, frames=None) -> np.ndarray:
        """Sub-pixel translation refinement (config.refine) of the registered
        frames' matrices (all, or `frames`) against the reference frame;
        returns new matrices."""
        cfg = self.config
        ok = getattr(self, "_registered", None)
        out = np.array(matrices, dtype=np.float64, copy=True)
        subset = range(self.frames) if frames is None else [int(k) for k in frames]
        good = np.array([k for k in subset if k != reference_index and (ok is None or ok[k])], dtype=np.int64)
        if cfg.refine_method == "gradient":
            if good.size == 0:
                return out
            gp = dict(DEFAULT_GRADIENT_REFINE, **(cfg.gradient_refine or {}))
            gp["sample_stride"], gp["row_stride"] = gradient_sample_grid(gp, self.height, self.width)
            gp.pop("target_samples", None)
            res = self.stack.refine_matrix_gradient_batch_to_reference(reference_index, good, out[good], **gp)
            done = set(good.tolist()) if frames is not None else None
            kept = [r for r in getattr(self, "last_refinement", []) if done is not None and r["frame"] not in done]
            self.last_refinement = kept + [dict(r, frame=int(k)) for k, r in zip(good, res)]
            for k, r in zip(good, res):
                if r["ok"]:
                    out[k] = r["matrix"]
            return out
        if cfg.refine_method != "ncc":
            raise ValueError("refine_method must be ncc or gradient")
        if not cfg.refine or good.size == 0:
            return out
        r = cfg.refine
        params = _lib.RefineParams(float(r["search_radius_px"]), float(r["coarse_step_px"]), float(r["fine_radius_px"]),
                                   float(r["fine_step_px"]), int(r["coarse_sample_stride"]),
                                   int(r["final_sample_stride"]))
        res = (_lib.RefineResult * good.size)()
        seeds = np.ascontiguousarray(out[good])
        _lib.call("gg_stack_refine_translation", self.stack.handle, ctypes.c_int64(int(reference_index)),
                  _lib.ptr(good), ctypes.c_int64(good.size), _lib.ptr(seeds), ctypes.byref(params), res)
        for pos, k in enumerate(good):
            out[k] = np.asarray(res[pos].matrix, dtype=np.float64).reshape(3, 3)
        return out

    def refine_adjoint(self, matrices: np.ndarray, reference_index: int = 0, config=None,
                       frames: list[int] | None = None) -> tuple[np.ndarray, list]:
        """Gradient refinement (glass_gb300.adjoint.refine_affine: torch
        autograd through the warp adjoint) of the registered frames' matrices
        (all, or `frames`) against the reference frame, on the calibrated
        frames in place (run it before warp()).  Returns the new matrices and
        the per-frame outcomes."""
        from glass_gb300.adjoint import refine_affine

        ok = getattr(self, "_registered", None)
        out = np.array(matrices, dtype=np.float64, copy=True)
        ref = self.stack.frame_tensor(reference_index)
        outcomes = []
        for k in range(self.frames) if frames is None else frames:
            if k == reference_index or (ok is not None and not ok[k]):
                continue
            res = refine_affine(ref, self.stack.frame_tensor(k), out[k], config)
            out[k] = res.matrix
            outcomes.append(res)
        return out, outcomes

    def assess(self, matrices: np.ndarray, reference_index: int = 0, frames=None) -> list[dict]:
        """Registration quality of every registered frame (or of `frames`)
        under its final matrix (run before warp()): the inlier / fit-RMS gate,
        then the pixel-agreement score and policy.  Frames that fail get
        weight 0 in weights(); downweighted frames get the policy's
        multiplier.  Returns one record per assessed moving frame (one host
        synchronisation)."""
        from glass_gb300 import quality

        cfg = self.config
        ag = dict(DEFAULT_AGREEMENT, **(cfg.agreement or {}))
        registered = getattr(self, "_registered", np.ones(self.frames, dtype=bool))
        subset = range(self.frames) if frames is None else [int(k) for k in frames]
        if frames is None or not hasattr(self, "_accepted"):
            ok = registered.copy()
            mult = np.ones(self.frames, dtype=np.float64)
        else:
            ok = self._accepted.copy()
            mult = self._multipliers.copy()
            for k in subset:
                ok[k] = registered[k]
                mult[k] = 1.0
        regs = {r["frame"]: r for r in getattr(self, "last_registration", [])}
        records = []
        for k in subset:
            if k == reference_index or not ok[k] or k not in regs:
                continue
            r = regs[k]
            gate = quality.registration_quality("ok", r["inliers"], r["rms_px"], "similarity_cuda_triangle",
                                                cfg.quality_action, cfg.quality_min_inliers, cfg.quality_max_rms_px)
            if not gate["accepted"]:
                ok[k] = False
            records.append({"frame": k, "gate": gate})
        idx = np.array([rec["frame"] for rec in records if ok[rec["frame"]]], dtype=np.int64)
        metrics = self.stack.matrix_alignment_metrics(reference_index, idx, np.asarray(matrices)[idx],
                                                      int(ag["sample_stride"])) if idx.size else []
        by_frame = dict(zip(idx.tolist(), metrics))
        for rec in records:
            k = rec["frame"]
            if k not in by_frame:
                continue
            m = by_frame[k]
            q = quality.agreement_quality(m["ncc"], m["rms"], regs[k]["rms_px"], ag["rms_scale_adu"], ag["min_score"])
            pol = quality.agreement_policy(q, ag["action"], ag["min_weight"])
            rec.update(score=q["score"], pixel_ncc=q["pixel_ncc"], pixel_rms_adu=q["pixel_rms_adu"],
                       status=pol["status"], multiplier=pol["weight_multiplier"])
            if pol["hard_failure"]:
                ok[k] = False
            elif pol["weight_multiplier"] < 1.0:
                mult[k] = pol["weight_multiplier"]
        self._accepted = ok
        self._multipliers = mult
        if frames is None:
            self.last_quality = records
        else:
            done = {rec["frame"] for rec in records}
            self.last_quality = [r for r in getattr(self, "last_quality", []) if r["frame"] not in done] + records
        return records

    def warp(self, matrices: np.ndarray, reference_index: int = 0, frames=None) -> None:
        """Warps every frame (or every one of `frames`) but the reference
        through its moving->reference matrix."""
        ok = getattr(self, "_registered", None)
        subset = range(self.frames) if frames is None else [int(k) for k in frames]
        idx = np.array([i for i in subset if i != reference_index and (ok is None or ok[i])], dtype=np.int64)
        if idx.size == 0:
            return
        mats = np.ascontiguousarray(np.asarray(matrices, dtype=np.float64)[idx])
        interp = _lib.GG_INTERP_LANCZOS3 if self.config.interpolation == "lanczos3" else _lib.GG_INTERP_BILINEAR
        self.stack.warp_frames_async(idx, mats, interp, np.nan, self.config.clamping_threshold, False)

    def weights(self) -> None:
        """Frame weights on the device: simple_snr (or unit) times the
        registration-quality multiplier; 0 for frames that failed
        registration or its quality checks (assess())."""
        ok = getattr(self, "_accepted", getattr(self, "_registered", None))
        prior = None
        if ok is not None:
            mult = getattr(self, "_multipliers", np.ones(self.frames))
            prior = np.where(ok, mult, 0.0).astype(np.float32)
        self.stack.compute_frame_weights(self.config.weighting, prior, 1.0e-6, download=False)

    def local_normalize(self, reference_index: int = 0) -> None:
        """Grid local normalisation (config.local_normalization_tile) of every
        registered frame to the reference frame, after the warp and the
        weights (a frame without paired finite pixels gets weight 0)."""
        tile = int(self.config.local_normalization_tile)
        if tile <= 0:
            return
        ok = getattr(self, "_registered", None)
        idx = [k for k in range(self.frames) if k != reference_index and (ok is None or ok[k])]
        self.stack.local_normalize_grid(reference_index, idx, tile, 1.0e-6, update_weights=True)

    def integrate(self) -> None:
        cfg = self.config
        self.stack.integrate_async("device", cfg.rejection, cfg.low_sigma, cfg.high_sigma, cfg.min_samples,
                                   cfg.max_reject_fraction, cfg.count_map_dtype)

    def capture_graph(self, dev_raw_ptr: int, matrices: np.ndarray) -> int:
        """Captures calibrate -> weights -> fused warp + rejection + integration
        with fixed matrices into a CUDA graph (at most 512 frames); returns the
        number of kernels one replay launches."""
        cfg = self.config
        return self.stack.capture_step_graph(dev_raw_ptr, matrices, self._calib_params(), cfg.interpolation,
                                             cfg.clamping_threshold, cfg.weighting, cfg.rejection, cfg.low_sigma,
                                             cfg.high_sigma, cfg.min_samples, cfg.max_reject_fraction,
                                             cfg.count_map_dtype)

    def launch_graph(self) -> None:
        self.stack.launch_step_graph()

    def step_device_fused(self, dev_raw_ptr: int, matrices: np.ndarray) -> None:
        """The eager launch sequence that capture_graph records."""
        cfg = self.config
        self.calibrate_device(dev_raw_ptr)
        self.weights()
        self.stack.integrate_warped_device_weights(matrices, cfg.interpolation, cfg.clamping_threshold, cfg.rejection,
                                                   cfg.low_sigma, cfg.high_sigma, cfg.min_samples,
                                                   cfg.max_reject_fraction, cfg.count_map_dtype)

    def step_device(self, dev_raw_ptr: int, matrices: np.ndarray | None = None) -> None:
        self.calibrate_device(dev_raw_ptr)
        if matrices is not None:
            self.warp(matrices)
        self.weights()
        self.local_normalize()
        self.integrate()

    def frame_chunks(self, parts: int | None = None) -> list[list[int]]:
        """Frame chunks of the staged step: `parts` (default
        self.staged_chunks) runs of consecutive frames (the first holds the
        reference frame 0, whose catalog every registration needs).  Few,
        large chunks: the catalog and registration kernels run one CTA per
        frame, so small chunks leave SMs idle.  On the 9600 x 6422 x 200 stack
        a step whose raw frames were prefetched behind the previous step's
        integration took 379 ms end to end in one chunk (the device step
        alone: 379 ms); a step that uploads its own 24.7 GB took 535 ms in one
        chunk, 468 ms in two, 465 ms in three and 483 ms in eight.  One chunk
        stays the default: the registration-quality sums are split over a
        number of CTAs that depends on the frames sharing a launch, so a
        chunked step reproduces an unchunked one to rounding, not bit for
        bit."""
        parts = self.staged_chunks if parts is None else parts
        parts = max(1, min(int(parts), self.frames))
        bounds = [round(i * self.frames / parts) for i in range(parts + 1)]
        return [list(range(a, b)) for a, b in zip(bounds[:-1], bounds[1:]) if b > a]

    def step_host(self, host_raw: np.ndarray, matrices: np.ndarray | None = None, register: bool = False,
                  out: tuple | None = None, staged: bool = True, prefetch: np.ndarray | None = None):
        """Public-API step from host memory to host maps (end to end).  With
        register=True the matrices come from detect() + register() + refine()
        + assess().  With staged=True (page-locked host_raw) the raw frames of
        the whole stack are uploaded on the copy stream up front and the
        per-frame stages run chunk by chunk (frame_chunks) while the later
        chunks are still in flight, so the host-to-device copy overlaps the
        step's own work; the integration waits for every frame.  `prefetch`
        (page-locked, the next step's raw frames) starts the next step's
        upload once this step's integration is enqueued, so it runs behind
        this step's weights, integration and download; the next step_host call
        with that same buffer then skips its upload (the buffer must not
        change in between).  `out` optionally supplies the six map buffers
        (see download_maps)."""
        if staged and register:
            pending = getattr(self, "_prefetched", None)
            self._prefetched = None
            if pending != host_raw.ctypes.data:
                self.upload_raw(host_raw)
            for chunk in self.frame_chunks():
                self.calibrate_staged(chunk)
                self.detect(frames=chunk)
                mats, _ok = self.register(0, frames=chunk)
                mats = self.refine(mats, 0, frames=chunk)
                self.assess(mats, 0, frames=chunk)
                self.warp(mats, 0, frames=chunk)
        else:
            self.calibrate_host(host_raw)
            if register:
                self.detect()
                matrices, _ok = self.register()
                matrices = self.refine(matrices)
                self.assess(matrices)
            if matrices is not None:
                self.warp(matrices)
        self.weights()
        self.local_normalize()
        self.integrate()
        if staged and register and prefetch is not None:
            # enqueued behind the integration: the copies run on the copy
            # stream while the stack stream integrates and downloads
            self.upload_raw(prefetch)
            self._prefetched = prefetch.ctypes.data
        return self.stack.download_maps("full", include_dq=True, out=out)

    def close(self) -> None:
        self.stack.close()
