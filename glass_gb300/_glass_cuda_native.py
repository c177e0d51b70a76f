"""Drop-in replacement for GLASS's ``_glass_cuda_native`` extension module.

GLASS loads its CUDA backend with ``importlib.import_module("_glass_cuda_native")``
(src/glass_cuda.py:31-44) and reaches it through the names that the pybind11
module exports (cpp/src/native_bindings.cpp:20383-21200).  This module offers
those names on top of libglass_gb300.so (include/glass_gb300.h) through ctypes,
so src/glass_cuda.py, src/glass/engine/resident_cuda.py and ``glass run
--backend cuda`` run unchanged.  ``glass_gb300.install_drop_in()`` registers it
under the reference's module name.

Error behaviour follows the reference: argument errors raise ValueError
(std::invalid_argument), bad frame indices IndexError (std::out_of_range),
state and CUDA failures RuntimeError (check_cuda, native_bindings.cpp:1011).
Callers feature-gate with ``hasattr`` (glass_cuda.py:2740-2760), so methods
that are not provided here make the façade raise its own clear RuntimeError.
"""

from __future__ import annotations

import ctypes
import weakref
from time import perf_counter
from typing import Any

import numpy as np

from glass_gb300 import _lib

_lib.load()

__all__ = [
    "RawFitsReadQueue",
    "ResidentCalibratedStack",
    "calibrate_tile_f32",
    "integrate_stacks_batch",
    "cuda_available",
    "get_device_info",
    "host_pinned_empty_f32",
    "host_pinned_empty_u8",
    "list_devices",
    "resident_dq_map_count_maps_i16",
]


# ---------------------------------------------------------------------------
# module functions
# ---------------------------------------------------------------------------
def cuda_available() -> bool:
    flag = ctypes.c_int(0)
    _lib.call("gg_cuda_available", ctypes.byref(flag))
    return bool(flag.value)


def get_device_info(device_id: int = 0) -> dict[str, Any]:
    info = _lib.DeviceInfo()
    _lib.call("gg_device_info", int(device_id), ctypes.byref(info))
    return {
        "device_id": int(device_id),
        "name": info.name.decode("utf-8", "replace"),
        "compute_capability": f"{info.major}.{info.minor}",
        "major": int(info.major),
        "minor": int(info.minor),
        "multiprocessor_count": int(info.multiprocessor_count),
        "total_memory_bytes": int(info.total_global_mem),
        "l2_cache_bytes": int(info.l2_cache_bytes),
        "shared_memory_per_block_optin": int(info.shared_mem_per_block_optin),
    }


def list_devices() -> list[dict[str, Any]]:
    count = ctypes.c_int(0)
    _lib.call("gg_device_count", ctypes.byref(count))
    return [get_device_info(i) for i in range(count.value)]


class _PinnedBuffer:
    """Page-locked host allocation exposed to NumPy (freed with the last view)."""

    def __init__(self, nbytes: int, dtype: np.dtype, shape: tuple[int, ...]):
        address = ctypes.c_void_p()
        _lib.call("gg_host_alloc_pinned", ctypes.c_size_t(max(int(nbytes), 1)), ctypes.byref(address))
        self.address = int(address.value)
        self.__array_interface__ = {
            "shape": shape,
            "typestr": np.dtype(dtype).str,
            "data": (self.address, False),
            "version": 3,
        }
        weakref.finalize(self, _lib.load().gg_host_free_pinned, ctypes.c_void_p(self.address))


class RawFitsReadQueue:
    """Host threads reading FITS data units into caller buffers
    (native_bindings.cpp:2605-2915, 20417-20429): submit(frame_index, path,
    data_offset, byte_count, output uint8[byte_count]) -> dict;
    wait_completed(timeout_s=-1) -> dict or None; stats(); close()."""

    def __init__(self, worker_count: int = 1):
        handle = ctypes.c_void_p()
        _lib.call("gg_read_queue_create", int(worker_count), ctypes.byref(handle))
        self._handle = handle
        self._buffers: dict[int, np.ndarray] = {}  # keep outputs alive until their completion
        weakref.finalize(self, _lib.load().gg_read_queue_destroy, handle)

    def submit(self, frame_index: int, path: str, data_offset: int, byte_count: int, output: np.ndarray) -> dict:
        if int(byte_count) <= 0:
            raise ValueError("native raw FITS queue byte count must be non-empty")
        if (not isinstance(output, np.ndarray) or output.dtype != np.uint8 or output.ndim != 1
                or output.shape[0] != int(byte_count) or not output.flags.c_contiguous):
            raise ValueError("native raw FITS queue output shape does not match byte count")
        pending = ctypes.c_uint64()
        _lib.call("gg_read_queue_submit", self._handle, int(frame_index), str(path).encode(), int(data_offset),
                  int(byte_count), _lib.ptr(output), ctypes.byref(pending))
        self._buffers[int(frame_index)] = output
        st = self.stats()
        return {"schema_version": 1, "backend": "native_u16be_raw_queue", "frame_index": int(frame_index),
                "pending_count": int(pending.value), "submitted_count": st["submitted_count"],
                "worker_count": st["worker_count"]}

    def wait_completed(self, timeout_s: float = -1.0):
        done = _lib.ReadCompletion()
        has = ctypes.c_int32()
        status = _lib.load().gg_read_queue_wait(self._handle, float(timeout_s), ctypes.byref(done), ctypes.byref(has))
        if has.value:
            self._buffers.pop(int(done.frame_index), None)
        _lib.check(status, "wait_completed")
        if not has.value:
            return None
        st = self.stats()
        return {"schema_version": 1, "backend": "native_u16be_raw_queue", "frame_index": int(done.frame_index),
                "bytes_read": int(done.bytes_read), "file_open_s": float(done.file_open_s),
                "file_read_s": float(done.file_read_s), "decode_s": 0.0, "total_s": float(done.total_s),
                "completed_count": st["completed_count"], "worker_count": st["worker_count"]}

    def stats(self) -> dict:
        s = _lib.ReadQueueStats()
        _lib.call("gg_read_queue_stats", self._handle, ctypes.byref(s))
        out = {name: int(getattr(s, name)) for name, _ in _lib.ReadQueueStats._fields_ if name != "pad"}
        out["closed"] = bool(out["closed"])
        out.update(schema_version=1, backend="native_u16be_raw_queue")
        return out

    def close(self) -> None:
        _lib.call("gg_read_queue_close", self._handle)


def integrate_stacks_batch(stacks: list, rejection: int = _lib.GG_REJECT_WINSORIZED, low_sigma: float = 3.0,
                           high_sigma: float = 3.0, min_samples: int = 3, max_reject_fraction: float = 0.5,
                           count_map_dtype: str = "uint16") -> None:
    """Integrates several resident stacks (each at most 32 frames, uneven
    frame counts and shapes allowed) in one kernel launch, each with its own
    device weights; read each stack's maps with its download_maps()."""
    if count_map_dtype not in {"float32", "uint16"}:
        raise ValueError("count_map_dtype must be float32 or uint16")
    if not stacks:
        return
    params = _lib.IntegrateParams(int(rejection), float(low_sigma), float(high_sigma), int(min_samples),
                                  float(max_reject_fraction),
                                  _lib.GG_COUNT_U16 if count_map_dtype == "uint16" else _lib.GG_COUNT_F32, 5)
    handles = (ctypes.c_void_p * len(stacks))(*[s.handle.value for s in stacks])
    _lib.call("gg_stacks_integrate_batch", handles, len(stacks), ctypes.byref(params))
    for s in stacks:
        s._last_count_dtype = np.dtype(np.uint16 if count_map_dtype == "uint16" else np.float32)


class StacksGraph:
    """Several resident stacks' calibrate -> weights -> warp -> rejection +
    integration captured in one CUDA graph (gg_stacks_graph_capture; no
    counterpart in the reference).  `steps` is a list of dicts with keys
    stack, dev_raw (device pointer of the stack's uint16 frames), matrices
    (frame_count x 3 x 3 forward matrices; identities are not warped),
    interpolation ("bilinear" / "lanczos3"), rejection (GG_REJECT_*), and
    optionally weighting ("simple_snr" / "unit"), low_sigma, high_sigma,
    min_samples, max_reject_fraction, count_map_dtype, linear_fit_iterations,
    calib (a _lib.CalibParams).  Read each stack's maps with download_maps()
    after launch() and a synchronisation of `stream`."""

    def __init__(self, steps: list[dict], cuda_stream: int | None = None):
        if not steps:
            raise ValueError("at least one stack is required")
        interps = {"bilinear": _lib.GG_INTERP_BILINEAR, "lanczos3": _lib.GG_INTERP_LANCZOS3}
        self._keep = []
        arr = (_lib.StackStep * len(steps))()
        for k, st in enumerate(steps):
            stack = st["stack"]
            mats = np.ascontiguousarray(np.asarray(st["matrices"], dtype=np.float64).reshape(-1, 3, 3))
            if mats.shape[0] != stack.frame_count:
                raise ValueError("one matrix per frame is required")
            if st.get("interpolation", "lanczos3") not in interps:
                raise ValueError("interpolation must be bilinear or lanczos3")
            dtype = st.get("count_map_dtype", "uint16")
            if dtype not in ("uint16", "float32"):
                raise ValueError("count_map_dtype must be float32 or uint16")
            self._keep.append(mats)
            arr[k].stack = stack.handle.value
            arr[k].dev_raw = int(st["dev_raw"])
            arr[k].host_matrices = mats.ctypes.data
            arr[k].interpolation = interps[st.get("interpolation", "lanczos3")]
            arr[k].clamping_threshold = float(st.get("clamping_threshold", -1.0))
            arr[k].weighting = 1 if st.get("weighting", "simple_snr") == "simple_snr" else 0
            arr[k].calib = st.get("calib") or _lib.CalibParams(1, 1.0, 1.0e-6, 0.0)
            arr[k].integrate = _lib.IntegrateParams(
                int(st.get("rejection", _lib.GG_REJECT_WINSORIZED)), float(st.get("low_sigma", 3.0)),
                float(st.get("high_sigma", 3.0)), int(st.get("min_samples", 3)),
                float(st.get("max_reject_fraction", 0.5)),
                _lib.GG_COUNT_U16 if dtype == "uint16" else _lib.GG_COUNT_F32,
                int(st.get("linear_fit_iterations", 5)))
            stack._last_count_dtype = np.dtype(np.uint16 if dtype == "uint16" else np.float32)
        self._stacks = [st["stack"] for st in steps]
        self._handle = ctypes.c_void_p()
        _lib.call("gg_stacks_graph_capture", arr, len(steps), ctypes.c_void_p(cuda_stream),
                  ctypes.byref(self._handle))

    def launch(self) -> None:
        _lib.call("gg_stacks_graph_launch", self._handle)

    @property
    def kernel_count(self) -> int:
        out = ctypes.c_int32()
        _lib.call("gg_stacks_graph_kernel_count", self._handle, ctypes.byref(out))
        return int(out.value)

    def close(self) -> None:
        if self._handle and self._handle.value:
            _lib.call("gg_stacks_graph_destroy", self._handle)
            self._handle = ctypes.c_void_p()


class _DeviceView:
    """A resident frame exposed through __cuda_array_interface__ (keeps its stack alive)."""

    def __init__(self, address: int, height: int, width: int, owner: Any):
        self.owner = owner
        self.__cuda_array_interface__ = {
            "shape": (height, width),
            "typestr": "<f4",
            "data": (address, False),
            "version": 2,
            "strides": None,
        }


def host_pinned_empty_f32(height: int, width: int) -> np.ndarray:
    h, w = int(height), int(width)
    if h <= 0 or w <= 0:
        raise ValueError("height and width must be positive")
    return np.asarray(_PinnedBuffer(h * w * 4, np.float32, (h, w)))


def host_pinned_empty_u8(byte_count: int) -> np.ndarray:
    n = int(byte_count)
    if n < 0:
        raise ValueError("byte_count must be non-negative")
    return np.asarray(_PinnedBuffer(n, np.uint8, (n,)))


def _policy_fields(policy: Any | None) -> tuple[bool, bool, float, float]:
    """Fields of CalibrationPolicy the calibration reads (models.py:67-81)."""
    p = policy if isinstance(policy, dict) else ({} if policy is None else dict(policy))
    return (
        bool(p.get("master_dark_includes_bias", True)),
        bool(p.get("dark_scaling_enabled", True)),
        float(p.get("flat_floor", 1.0e-6)),
        float(p.get("pedestal", 0.0)),
    )


def _calib_params(policy: Any | None, has_dark: bool, light_exposure_s: float,
                  dark_exposure_s: float | None) -> _lib.CalibParams:
    """cpu/calibration.py:62-66: scale = t_light / t_dark when scaling applies."""
    includes_bias, scaling, floor, pedestal = _policy_fields(policy)
    scale = 1.0
    if has_dark and scaling and dark_exposure_s not in (None, 0):
        scale = float(light_exposure_s) / float(dark_exposure_s)
    return _lib.CalibParams(int(includes_bias), float(scale), float(floor), float(pedestal))


def _f32(value: Any, name: str) -> np.ndarray:
    array = np.ascontiguousarray(np.asarray(value, dtype=np.float32))
    if array.ndim != 2 and name != "frame":
        raise ValueError(f"{name} must be a 2-D array")
    return array


def calibrate_tile_f32(light: Any, bias: Any | None, dark: Any | None, flat: Any | None,
                       light_exposure_s: float, dark_exposure_s: float | None,
                       policy: Any | None = None) -> np.ndarray:
    """Module `calibrate_tile_f32` (glass_cuda.py:477-508)."""
    light_a = np.ascontiguousarray(np.asarray(light, dtype=np.float32))
    masters = []
    for name, m in (("bias", bias), ("dark", dark), ("flat", flat)):
        if m is None:
            masters.append(None)
            continue
        arr = np.ascontiguousarray(np.asarray(m, dtype=np.float32))
        if arr.shape != light_a.shape:
            raise ValueError(f"{name} shape {arr.shape} does not match light shape {light_a.shape}")
        masters.append(arr)
    params = _calib_params(policy, dark is not None, light_exposure_s, dark_exposure_s)
    out = np.empty_like(light_a)
    _lib.call(
        "gg_calibrate_tile_f32",
        _lib.ptr(light_a), _lib.ptr(masters[0]), _lib.ptr(masters[1]), _lib.ptr(masters[2]),
        ctypes.c_int64(light_a.size), ctypes.byref(params), _lib.ptr(out),
    )
    return out


def _matrix64(matrix: Any) -> np.ndarray:
    """The reference takes float32 matrices (np.asarray(m, np.float32)) and
    inverts them in float64 (native_bindings.cpp:1423-1457)."""
    m = np.asarray(np.asarray(matrix, dtype=np.float32), dtype=np.float64)
    if m.shape != (3, 3):
        raise ValueError(f"warp matrix must be 3x3, got {m.shape}")
    return np.ascontiguousarray(m)


def _warp_image(data: Any, matrix: np.ndarray, interpolation: int, fill: float, clamp: float):
    image = np.ascontiguousarray(np.asarray(data, dtype=np.float32))
    if image.ndim != 2:
        raise ValueError("data must be a 2-D array")
    h, w = image.shape
    out = np.empty_like(image)
    cov = np.empty_like(image)
    _lib.call("gg_warp_matrix_f32", _lib.ptr(image), ctypes.c_int64(h), ctypes.c_int64(w),
              _lib.ptr(np.ascontiguousarray(matrix, dtype=np.float64)), int(interpolation), ctypes.c_float(fill),
              ctypes.c_float(clamp), _lib.ptr(out), _lib.ptr(cov))
    return out, cov


def _translation_matrix(dx: float, dy: float) -> np.ndarray:
    return np.array([[1.0, 0.0, dx], [0.0, 1.0, dy], [0.0, 0.0, 1.0]], dtype=np.float64)


def warp_translation_f32(data: Any, dx: float, dy: float, fill: float = 0.0):
    """Integer translation (cpu/warp.py:6-22): shifts by round(dx), round(dy)."""
    return _warp_image(data, _translation_matrix(float(int(round(dx))), float(int(round(dy)))),
                       _lib.GG_INTERP_NEAREST, fill, -1.0)


def warp_translation_bilinear_f32(data: Any, dx: float, dy: float, fill: float = 0.0):
    """Sub-pixel bilinear translation (glass_cuda.py:564-593)."""
    return _warp_image(data, _translation_matrix(float(dx), float(dy)), _lib.GG_INTERP_BILINEAR, fill, -1.0)


def warp_matrix_bilinear_f32(data: Any, matrix: Any, fill: float = 0.0):
    """glass_cuda.py:595-629 -> (warped, coverage)."""
    return _warp_image(data, _matrix64(matrix), _lib.GG_INTERP_BILINEAR, fill, -1.0)


def warp_matrix_lanczos3_f32(data: Any, matrix: Any, fill: float = 0.0, clamping_threshold: float = -1.0):
    """glass_cuda.py:644-706 -> (warped, coverage)."""
    return _warp_image(data, _matrix64(matrix), _lib.GG_INTERP_LANCZOS3, fill, clamping_threshold)


def detect_stars_f32(data: Any, threshold_sigma: float = 5.0, max_stars: int = 500,
                     background: float | None = None, noise: float | None = None, window_radius: int = 4,
                     min_separation_px: float = 2.0) -> np.ndarray:
    """detect_stars (cpu/star_detect.py:121-168) of one host image on the GPU."""
    image = np.ascontiguousarray(np.asarray(data, dtype=np.float32))
    if image.ndim != 2:
        raise ValueError("data must be a 2-D array")
    stack = ResidentCalibratedStack(1, image.shape[0], image.shape[1])
    try:
        stack.upload_calibrated_frame(0, image)
        return stack.detect_stars([0], threshold_sigma, max_stars, background, noise, window_radius,
                                  min_separation_px)[0]
    finally:
        stack.close()


# ---- registration: triangle asterisms (cpu/registration.py:242-475) ----------------
_REG_MAX_STARS = 80


def _catalog_xy(x: Any, y: Any) -> np.ndarray:
    xa = np.asarray(x, dtype=np.float32).reshape(-1)
    ya = np.asarray(y, dtype=np.float32).reshape(-1)
    if xa.shape != ya.shape:
        raise ValueError("catalog coordinate arrays must have the same shape")
    return np.ascontiguousarray(np.column_stack([xa, ya]).astype(np.float64))


def _points_xy(points: Any) -> np.ndarray:
    """(n, 2) float64 (x, y) from an array or a list of objects with .x/.y."""
    if isinstance(points, np.ndarray) and points.dtype.names and "x" in points.dtype.names:
        xy = np.column_stack([points["x"], points["y"]])
    elif isinstance(points, (list, tuple)) and points and hasattr(points[0], "x"):
        xy = [(p.x, p.y) for p in points]
    else:
        xy = points
    arr = np.asarray(xy, dtype=np.float64).reshape(-1, 2)
    return np.ascontiguousarray(arr)


_REG_MODELS = {"similarity": _lib.GG_TRANSFORM_SIMILARITY, "affine": _lib.GG_TRANSFORM_AFFINE}


def _register_params(transform_model: str, min_inliers: int, tolerance_px: float, max_stars: int, neighbors: int,
                     descriptor_radius: float, max_descriptors: int, max_candidates: int) -> _lib.RegisterParams:
    if transform_model not in _REG_MODELS:
        raise ValueError("triangle asterism registration supports similarity or affine transforms")
    return _lib.RegisterParams(_REG_MODELS[transform_model], int(min_inliers), float(tolerance_px),
                               float(descriptor_radius), int(max_stars), int(neighbors), int(max_descriptors),
                               int(max_candidates))


def _registration_dict(r: _lib.Registration, pairs: np.ndarray | None = None,
                       transform_model: str = "similarity") -> dict[str, Any]:
    out = {
        "transform_model": transform_model,
        "matrix": np.asarray(r.matrix, dtype=np.float64).reshape(3, 3),
        "matched_stars": int(r.inliers),
        "inliers": int(r.inliers),
        "rms_px": float(r.rms_px),
        "status": "ok" if r.status == 1 else "failed",
        "best_candidate_index": int(r.best_candidate),
        "reference_descriptor_count": int(r.descriptors_reference),
        "moving_descriptor_count": int(r.descriptors_moving),
        "descriptor_matches": int(r.matches),
    }
    if pairs is not None:
        p = pairs.reshape(-1, 2)[: int(r.inliers)]
        out["pairs"] = [(int(a), int(b)) for a, b in p]
    return out


def triangle_asterism_descriptors_f32(x: Any, y: Any, max_stars: int = 80, neighbors: int = 5,
                                      max_descriptors: int = 1200) -> dict[str, Any]:
    """Module triangle_asterism_descriptors_f32 (glass_cuda.py:1835-1902): local
    triangle descriptors of one catalog, area-descending."""
    if max_stars < 0:
        raise ValueError("max_stars must be non-negative")
    if max_descriptors < 0:
        raise ValueError("max_descriptors must be non-negative")
    xy = _catalog_xy(x, y)
    limited = min(len(xy), int(max_stars))
    cap = limited * 20
    desc = np.zeros((max(cap, 1), 2), dtype=np.float64)
    idx = np.zeros((max(cap, 1), 3), dtype=np.int32)
    areas = np.zeros(max(cap, 1), dtype=np.float64)
    count = ctypes.c_int64()
    _lib.call("gg_triangle_descriptors", _lib.ptr(xy), ctypes.c_int64(len(xy)), ctypes.c_int32(int(max_stars)),
              ctypes.c_int32(int(neighbors)), ctypes.c_int32(int(max_descriptors)), _lib.ptr(desc), _lib.ptr(idx),
              _lib.ptr(areas), ctypes.c_int64(desc.shape[0]), ctypes.byref(count))
    n = int(count.value)
    k = min(limited, max(3, int(neighbors)))
    raw = limited * k * (k - 1) * (k - 2) // 6 if limited >= 3 else 0
    return {"count": n, "raw_count": int(raw), "max_stars": int(max_stars), "neighbors": int(k),
            "descriptors": desc[:n].astype(np.float32), "indices": idx[:n].copy(),
            "areas": areas[:n].astype(np.float32), "model": "triangle_asterism_descriptors_cuda"}


def triangle_asterism_descriptors_batch_f32(x_list: list[Any], y_list: list[Any], max_stars: int = 80,
                                            neighbors: int = 5, max_descriptors: int = 1200) -> list[dict[str, Any]]:
    """Module triangle_asterism_descriptors_batch_f32 (glass_cuda.py:1935-1990)."""
    if len(x_list) != len(y_list):
        raise ValueError("catalog x/y batch lists must have the same length")
    out = []
    for k, (x, y) in enumerate(zip(x_list, y_list)):
        r = triangle_asterism_descriptors_f32(x, y, max_stars, neighbors, max_descriptors)
        r.update(batch_index=k, batch_count=len(x_list), batch_model="triangle_asterism_descriptors_cuda_batch")
        out.append(r)
    return out


def estimate_similarity_from_triangle_descriptors_f32(reference_x: Any, reference_y: Any, moving_x: Any,
                                                      moving_y: Any, reference_descriptors: Any,
                                                      reference_indices: Any, moving_descriptors: Any,
                                                      moving_indices: Any, tolerance_px: float = 2.0,
                                                      descriptor_radius: float = 0.1) -> dict[str, Any]:
    """Module estimate_similarity_from_triangle_descriptors_f32
    (glass_cuda.py:2054-2140): best similarity over every descriptor pair within
    the radius (reference-major), both orientations, no refit."""
    if tolerance_px < 0.0:
        raise ValueError("tolerance_px must be non-negative")
    if descriptor_radius < 0.0:
        raise ValueError("descriptor_radius must be non-negative")
    ref = _catalog_xy(reference_x, reference_y)
    mov = _catalog_xy(moving_x, moving_y)
    rd = np.ascontiguousarray(np.asarray(reference_descriptors, dtype=np.float32).reshape(-1, 2))
    md = np.ascontiguousarray(np.asarray(moving_descriptors, dtype=np.float32).reshape(-1, 2))
    ri = np.ascontiguousarray(np.asarray(reference_indices, dtype=np.int32).reshape(-1, 3))
    mi = np.ascontiguousarray(np.asarray(moving_indices, dtype=np.int32).reshape(-1, 3))
    if rd.shape[0] != ri.shape[0] or md.shape[0] != mi.shape[0]:
        raise ValueError("descriptor and index row counts must match")
    res = _lib.Registration()
    _lib.call("gg_similarity_from_descriptors", _lib.ptr(ref), ctypes.c_int64(len(ref)), _lib.ptr(mov),
              ctypes.c_int64(len(mov)), _lib.ptr(rd), _lib.ptr(ri), ctypes.c_int64(rd.shape[0]), _lib.ptr(md),
              _lib.ptr(mi), ctypes.c_int64(md.shape[0]), ctypes.c_double(float(tolerance_px)),
              ctypes.c_double(float(descriptor_radius)), ctypes.byref(res), None)
    m = np.asarray(res.matrix, dtype=np.float64).reshape(3, 3)
    a, b = float(m[0, 0]), float(m[1, 0])
    return {"matrix": m.astype(np.float32).tolist(), "scale": float(np.sqrt(a * a + b * b)),
            "rotation_rad": float(np.arctan2(b, a)), "rms_px": float(res.rms_px), "inliers": int(res.inliers),
            "best_candidate_index": int(res.best_candidate), "candidate_count": int(rd.shape[0] * md.shape[0] * 2),
            "reference_count": int(len(ref)), "moving_count": int(len(mov)),
            "reference_descriptor_count": int(rd.shape[0]), "moving_descriptor_count": int(md.shape[0]),
            "tolerance_px": float(tolerance_px), "descriptor_radius": float(descriptor_radius),
            "status": "ok" if res.inliers > 0 else "failed", "model": "triangle_descriptor_similarity_cuda"}


def estimate_similarity_from_triangle_descriptors_batch_f32(reference_x: Any, reference_y: Any,
                                                            reference_descriptors: Any, reference_indices: Any,
                                                            moving_x_list: list[Any], moving_y_list: list[Any],
                                                            moving_descriptors_list: list[Any],
                                                            moving_indices_list: list[Any],
                                                            tolerance_px: float = 2.0,
                                                            descriptor_radius: float = 0.1) -> list[dict[str, Any]]:
    """Module estimate_similarity_from_triangle_descriptors_batch_f32 (glass_cuda.py:2149-2230)."""
    lists = (moving_x_list, moving_y_list, moving_descriptors_list, moving_indices_list)
    if len({len(v) for v in lists}) != 1:
        raise ValueError("moving batch lists must have the same length")
    out = []
    for k, (mx, my, md, mi) in enumerate(zip(*lists)):
        r = estimate_similarity_from_triangle_descriptors_f32(reference_x, reference_y, mx, my,
                                                              reference_descriptors, reference_indices, md, mi,
                                                              tolerance_px, descriptor_radius)
        r.update(batch_index=k, batch_count=len(moving_x_list), batch_model="triangle_descriptor_similarity_cuda")
        out.append(r)
    return out


def estimate_triangle_asterism_transform(reference: Any, moving: Any, transform_model: str = "similarity",
                                         min_inliers: int = 6, tolerance_px: float = 3.0, max_stars: int = 80,
                                         neighbors: int = 5, descriptor_radius: float = 0.1,
                                         max_descriptors: int = 1200, max_candidates: int = 1500) -> dict[str, Any]:
    """estimate_triangle_asterism_transform (cpu/registration.py:361-475) on the
    GPU.  reference / moving: (n, 2) arrays, star records or Star-like objects,
    brightest first.  Returns the StarRegistration fields as a dict."""
    params = _register_params(transform_model, min_inliers, tolerance_px, max_stars, neighbors, descriptor_radius,
                              max_descriptors, max_candidates)
    ref = _points_xy(reference)
    mov = _points_xy(moving)
    res = _lib.Registration()
    pairs = np.full((_REG_MAX_STARS, 2), -1, dtype=np.int32)
    _lib.call("gg_register_star_lists", _lib.ptr(ref), ctypes.c_int64(len(ref)), _lib.ptr(mov),
              ctypes.c_int64(len(mov)), ctypes.byref(params), ctypes.byref(res), _lib.ptr(pairs))
    return _registration_dict(res, pairs, transform_model)


# ---- alignment metrics / sub-pixel refinement (glass_cuda.py:706-1245) -------------
def _metrics_dict(m: _lib.AlignmentMetrics, model: str) -> dict[str, Any]:
    return {"valid_pixels": int(m.valid_pixels), "sampled_pixels": int(m.sampled_pixels),
            "sample_stride": int(m.sample_stride), "rms": float(m.rms), "mean_abs_diff": float(m.mean_abs_diff),
            "ncc": float(m.ncc), "model": model}


def _pair_stack(reference: Any, moving: Any) -> "ResidentCalibratedStack":
    ref = np.ascontiguousarray(np.asarray(reference, dtype=np.float32))
    mov = np.ascontiguousarray(np.asarray(moving, dtype=np.float32))
    if ref.shape != mov.shape:
        raise ValueError(f"shape mismatch for registration: {ref.shape} != {mov.shape}")
    if ref.ndim != 2:
        raise ValueError("reference and moving must be 2-D arrays")
    stack = ResidentCalibratedStack(2, ref.shape[0], ref.shape[1])
    stack.upload_calibrated_frame(0, ref)
    stack.upload_calibrated_frame(1, mov)
    return stack


def star_grid_top_nms_candidates_f32(data: Any, threshold: float, grid_cols: int = 16, grid_rows: int = 12,
                                     candidates_per_cell: int = 4, max_output_candidates: int = 64,
                                     min_separation_px: float = 32.0) -> dict[str, Any]:
    """Module star_grid_top_nms_candidates_f32 (glass_cuda.py:2514-2606) on a
    host image through a one-frame resident stack."""
    image = np.ascontiguousarray(np.asarray(data, dtype=np.float32))
    if image.ndim != 2:
        raise ValueError("data must be a 2-D array")
    stack = ResidentCalibratedStack(1, image.shape[0], image.shape[1])
    try:
        stack.upload_calibrated_frame(0, image)
        return stack.star_grid_top_nms_candidates_deterministic(0, threshold, grid_cols, grid_rows,
                                                                 candidates_per_cell, max_output_candidates,
                                                                 min_separation_px)
    finally:
        stack.close()


def matrix_alignment_metrics_f32(reference: Any, moving: Any, matrix: Any, sample_stride: int = 1) -> dict[str, Any]:
    """Module matrix_alignment_metrics_f32 (glass_cuda.py:706-768)."""
    if sample_stride <= 0:
        raise ValueError("sample_stride must be positive")
    stack = _pair_stack(reference, moving)
    try:
        return stack.matrix_alignment_metrics(0, [1], [matrix], sample_stride)[0]
    finally:
        stack.close()


def refine_matrix_translation_with_metrics_f32(reference: Any, moving: Any, matrix: Any,
                                               search_radius_px: float = 1.0, coarse_step_px: float = 0.25,
                                               fine_radius_px: float = 0.25, fine_step_px: float = 0.0625,
                                               coarse_sample_stride: int = 4,
                                               final_sample_stride: int = 1) -> dict[str, Any]:
    """Module refine_matrix_translation_with_metrics_f32 (glass_cuda.py:771-900)."""
    stack = _pair_stack(reference, moving)
    try:
        res = stack.refine_matrix_translation_candidates_batch_to_reference(
            0, [1], [matrix], search_radius_px, coarse_step_px, fine_radius_px, fine_step_px, coarse_sample_stride,
            final_sample_stride)[0]
    finally:
        stack.close()
    for key in ("reference_index", "moving_index", "batch_index", "batch_count", "batch_model"):
        res.pop(key, None)
    res["model"] = "cuda_matrix_metric_translation_refine_grid"
    return res


def estimate_translation_subpixel_ncc_f32(reference: Any, moving: Any, center_dx: float, center_dy: float,
                                          radius_steps: int, step: float, sample_stride: int = 1) -> dict[str, Any]:
    """Module estimate_translation_subpixel_ncc_f32 (glass_cuda.py:1175-1245)."""
    if sample_stride <= 0:
        raise ValueError("sample_stride must be positive")
    if radius_steps < 0:
        raise ValueError("radius_steps must be non-negative")
    if step <= 0.0:
        raise ValueError("step must be positive")
    stack = _pair_stack(reference, moving)
    out = _lib.TranslationNcc()
    try:
        _lib.call("gg_stack_translation_ncc", stack.handle, ctypes.c_int64(0), ctypes.c_int64(1),
                  ctypes.c_double(float(center_dx)), ctypes.c_double(float(center_dy)),
                  ctypes.c_int32(int(radius_steps)), ctypes.c_double(float(step)), ctypes.c_int32(int(sample_stride)),
                  ctypes.byref(out))
    finally:
        stack.close()
    return {"dx": float(out.dx), "dy": float(out.dy), "score": float(out.score),
            "candidate_count": int(out.candidate_count), "center_dx": float(center_dx),
            "center_dy": float(center_dy), "radius_steps": int(radius_steps), "step": float(step),
            "sample_stride": int(sample_stride), "model": "translation_subpixel_ncc_cuda"}


def resident_dq_map_count_maps_i16(master: Any, weight_map: Any, coverage_map: Any | None = None,
                                   low_rejection_map: Any | None = None,
                                   high_rejection_map: Any | None = None,
                                   geometric_warp_coverage_map: Any | None = None,
                                   active_frame_count: int = 0) -> np.ndarray:
    """Module `resident_dq_map_count_maps_i16` (glass_cuda.py:270-290)."""
    m = np.ascontiguousarray(np.asarray(master, dtype=np.float32))
    w = np.ascontiguousarray(np.asarray(weight_map, dtype=np.float32))
    if w.shape != m.shape:
        raise ValueError("weight_map must have the master shape")

    def opt(x):
        if x is None:
            return None
        a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
        if a.shape != m.shape:
            raise ValueError("count maps must have the master shape")
        return a

    cov, low, high, geo = (opt(x) for x in (coverage_map, low_rejection_map, high_rejection_map,
                                             geometric_warp_coverage_map))
    dq = np.empty(m.shape, dtype=np.int16)
    _lib.call("gg_dq_map_i16", _lib.ptr(m), _lib.ptr(w), _lib.ptr(cov), _lib.ptr(low), _lib.ptr(high),
              _lib.ptr(geo), ctypes.c_int64(m.size), ctypes.c_int64(int(active_frame_count)), _lib.ptr(dq))
    return dq


# ---------------------------------------------------------------------------
# ResidentCalibratedStack
# ---------------------------------------------------------------------------
_DOWNLOAD_MODES = {"full", "master_weight", "master_only"}


class ResidentCalibratedStack:
    """VRAM-resident calibrated stack (native_bindings.cpp:2915-2934).

    Frames live in padded slots of one HBM allocation; the device table
    frame->slot lets warps swap output slots instead of copying frames back.
    """

    def __init__(self, frame_count: int, height: int, width: int):
        handle = ctypes.c_void_p()
        _lib.call("gg_stack_create", ctypes.c_int64(int(frame_count)), ctypes.c_int64(int(height)),
                  ctypes.c_int64(int(width)), ctypes.byref(handle))
        self._handle = handle
        self._finalizer = weakref.finalize(self, _lib.load().gg_stack_destroy, handle)
        self._last_count_dtype: np.dtype | None = None

    # ---- plumbing ----------------------------------------------------------
    @property
    def handle(self) -> ctypes.c_void_p:
        return self._handle

    def _info(self) -> _lib.StackInfo:
        info = _lib.StackInfo()
        _lib.call("gg_stack_info", self._handle, ctypes.byref(info))
        return info

    def close(self) -> None:
        self._finalizer()

    def set_stream(self, cuda_stream: int | None) -> None:
        """Enqueues this stack's work on an external cudaStream_t (None: own stream)."""
        _lib.call("gg_stack_set_stream", self._handle, ctypes.c_void_p(int(cuda_stream) if cuda_stream else 0))

    def synchronize(self) -> None:
        _lib.call("gg_stack_synchronize", self._handle)

    def device_pointers(self) -> dict[str, int]:
        ptrs = _lib.StackDevicePtrs()
        _lib.call("gg_stack_device_ptrs", self._handle, ctypes.byref(ptrs))
        return {name: int(getattr(ptrs, name) or 0) for name, _ in _lib.StackDevicePtrs._fields_}

    def frame_tensor(self, index: int):
        """Zero-copy torch CUDA view (H x W float32) of loaded frame `index`.

        Valid until the frame is warped (warps move frames between slots);
        synchronises the stack's stream."""
        import torch

        addr = ctypes.c_void_p()
        _lib.call("gg_stack_frame_device_ptr", self._handle, ctypes.c_int64(int(index)), ctypes.byref(addr))
        info = self._info()
        return torch.as_tensor(_DeviceView(int(addr.value), int(info.height), int(info.width), self))

    # ---- properties (native_bindings.cpp:20624-20645) -----------------------
    @property
    def frame_count(self) -> int:
        return int(self._info().frame_count)

    @property
    def height(self) -> int:
        return int(self._info().height)

    @property
    def width(self) -> int:
        return int(self._info().width)

    @property
    def pixels_per_frame(self) -> int:
        return int(self._info().pixels_per_frame)

    @property
    def loaded_count(self) -> int:
        return int(self._info().loaded_count)

    @property
    def bytes_allocated(self) -> int:
        return int(self._info().bytes_allocated)

    @property
    def warp_scratch_bytes(self) -> int:
        return int(self._info().warp_scratch_bytes)

    @property
    def warp_copy_mode(self) -> str:
        return "slot_swap_no_copy"

    @property
    def host_pinned_bytes(self) -> int:
        return int(self._info().host_pinned_bytes)

    @property
    def calibration_lane_count(self) -> int:
        return int(self._info().calibration_lane_count)

    @property
    def warp_coverage_frame_count(self) -> int:
        return int(self._info().warp_coverage_frame_count)

    @property
    def frame_stride(self) -> int:
        return int(self._info().frame_stride)

    # ---- masters / upload / download ---------------------------------------
    def _frame_array(self, value: Any, name: str) -> np.ndarray:
        info = self._info()
        array = np.ascontiguousarray(np.asarray(value, dtype=np.float32))
        if array.shape != (info.height, info.width):
            raise ValueError(f"{name} must have shape ({info.height}, {info.width}), got {array.shape}")
        return array

    def set_calibration_masters(self, bias: Any | None = None, dark: Any | None = None,
                                flat: Any | None = None) -> None:
        arrays = [None if m is None else self._frame_array(m, n)
                  for m, n in ((bias, "bias"), (dark, "dark"), (flat, "flat"))]
        _lib.call("gg_stack_set_masters", self._handle, *(_lib.ptr(a) for a in arrays))

    def upload_calibrated_frame(self, index: int, frame: Any) -> None:
        array = self._frame_array(frame, "frame")
        _lib.call("gg_stack_upload_frame", self._handle, ctypes.c_int64(int(index)), _lib.ptr(array))

    def download_frame_tile(self, index: int, x0: int, y0: int, x1: int, y1: int) -> np.ndarray:
        return self.download_frames_tile(np.asarray([index], dtype=np.int64), x0, y0, x1, y1)[0]

    def download_frames_tile(self, indices: Any, x0: int, y0: int, x1: int, y1: int) -> np.ndarray:
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1))
        if idx.size == 0:
            raise ValueError("indices must contain at least one frame index")
        out = np.empty((idx.size, max(int(y1) - int(y0), 0), max(int(x1) - int(x0), 0)), dtype=np.float32)
        _lib.call("gg_stack_download_frames_tile", self._handle, _lib.ptr(idx), ctypes.c_int64(idx.size),
                  ctypes.c_int64(int(x0)), ctypes.c_int64(int(y0)), ctypes.c_int64(int(x1)),
                  ctypes.c_int64(int(y1)), _lib.ptr(out))
        return out

    def download_frame(self, index: int) -> np.ndarray:
        info = self._info()
        return self.download_frame_tile(index, 0, 0, info.width, info.height)

    # ---- calibration ---------------------------------------------------------
    def _params(self, light_exposure_s: float, dark_exposure_s: float | None, policy: Any | None):
        return _calib_params(policy, bool(self._info().has_dark), light_exposure_s, dark_exposure_s)

    def calibrate_frame(self, index: int, light: Any, light_exposure_s: float,
                        dark_exposure_s: float | None, policy: Any | None = None) -> None:
        array = self._frame_array(light, "light")
        params = self._params(light_exposure_s, dark_exposure_s, policy)
        _lib.call("gg_stack_calibrate_f32", self._handle, ctypes.c_int64(int(index)), _lib.ptr(array),
                  ctypes.byref(params))

    def calibrate_frame_timed(self, index: int, light: Any, light_exposure_s: float,
                              dark_exposure_s: float | None, policy: Any | None = None) -> dict[str, Any]:
        start = perf_counter()
        self.calibrate_frame(index, light, light_exposure_s, dark_exposure_s, policy)
        total = perf_counter() - start
        return {"schema_version": 1, "h2d_mode": "pageable", "event_mode": "none", "host_copy_s": 0.0,
                "h2d_s": 0.0, "calibrate_store_s": total, "total_s": total,
                "host_pinned_bytes": self.host_pinned_bytes}

    def calibrate_frames_u16(self, indices: Any, raw_lights: Any, light_exposure_s: float,
                             dark_exposure_s: float | None, policy: Any | None = None,
                             big_endian_bzero: bool = False) -> None:
        """Fused uint16 decode + calibrate of a (n, H, W) uint16 block (one H2D pipeline)."""
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1))
        raw = np.asarray(raw_lights)
        info = self._info()
        if raw.dtype not in (np.dtype(np.uint16), np.dtype(">u2"), np.dtype(np.int16)):
            raise ValueError("raw lights must be uint16")
        raw = np.ascontiguousarray(raw.view(np.uint16) if raw.dtype != np.uint16 else raw)
        if raw.shape != (idx.size, info.height, info.width):
            raise ValueError(f"raw lights must have shape ({idx.size}, {info.height}, {info.width})")
        params = self._params(light_exposure_s, dark_exposure_s, policy)
        _lib.call("gg_stack_calibrate_u16", self._handle, _lib.ptr(idx), ctypes.c_int64(idx.size),
                  _lib.ptr(raw), int(bool(big_endian_bzero)), ctypes.byref(params))
        self.synchronize()

    def calibrate_frames_fits_u16be_bzero_host_async_multistream_callback_release_timed(
        self, indices: Any, raw_lights: Any, light_exposures_s: Any, dark_exposures_s: Any,
        stream_count: int, wave_frames: int, release_callback: Any, policy: Any | None = None,
    ) -> dict[str, Any]:
        """FITS BITPIX=16 big-endian raw bytes (BZERO 32768) per frame (native_bindings.cpp:7422-8094)."""
        idx = np.asarray(indices, dtype=np.int64).reshape(-1)
        raws = list(raw_lights)
        t_l = np.asarray(light_exposures_s, dtype=np.float32).reshape(-1)
        t_d = np.asarray(dark_exposures_s, dtype=np.float32).reshape(-1)
        if not (len(raws) == idx.size == t_l.size == t_d.size):
            raise ValueError("indices, raw_lights and exposures must have the same length")
        info = self._info()
        frame_bytes = info.height * info.width * 2
        start = perf_counter()
        for k in range(idx.size):
            buf = np.ascontiguousarray(np.asarray(raws[k]).view(np.uint8).reshape(-1))
            if buf.size < frame_bytes:
                raise ValueError(f"raw light {k} has {buf.size} bytes, expected {frame_bytes}")
            dark_t = None if not np.isfinite(t_d[k]) or t_d[k] == 0 else float(t_d[k])
            params = self._params(float(t_l[k]), dark_t, policy)
            one = np.asarray([idx[k]], dtype=np.int64)
            _lib.call("gg_stack_calibrate_u16", self._handle, _lib.ptr(one), ctypes.c_int64(1), _lib.ptr(buf),
                      1, ctypes.byref(params))
        self.synchronize()
        if release_callback is not None:
            for k in range(idx.size):
                release_callback(int(k))
        total = perf_counter() - start
        return {"schema_version": 1, "h2d_mode": "pinned_lanes", "frames": int(idx.size),
                "stream_count": int(stream_count), "wave_frames": int(wave_frames), "total_s": total,
                "host_pinned_bytes": self.host_pinned_bytes}

    # ---- grid star catalogs (star_detect_kernels.cu:40-101, 317-742) ----------------
    def _grid_catalog(self, indices: Any, threshold: float, grid_cols: int, grid_rows: int,
                      candidates_per_cell: int, max_output_candidates: int, min_separation_px: float,
                      centroid_radius: int, centroid_global_mean_background: bool,
                      deterministic: bool) -> list[dict[str, Any]]:
        """The reference's batch grid catalog (native_bindings.cpp:12211-12645):
        per-cell top-K local maxima, value-ordered separation scan, optional
        windowed centroid.  Every variant runs the deterministic order; it is
        also a valid result of the reference's lock-based variant."""
        if grid_cols <= 0 or grid_rows <= 0 or candidates_per_cell <= 0 or max_output_candidates <= 0:
            raise ValueError("grid dimensions and candidate counts must be positive")
        if min_separation_px < 0.0:
            raise ValueError("min_separation_px must be non-negative")
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1))
        if idx.size == 0:
            return []
        n, mo = idx.size, int(max_output_candidates)
        params = _lib.GridCatalogParams(float(threshold), int(grid_cols), int(grid_rows), int(candidates_per_cell),
                                        mo, float(min_separation_px), max(0, int(centroid_radius)),
                                        1 if centroid_global_mean_background else 0)
        planes = np.empty((5, n, mo), dtype=np.float32)
        status = np.zeros((n, mo), dtype=np.uint8)
        counts = np.empty((n, 2), dtype=np.int32)
        start = perf_counter()
        _lib.call("gg_stack_star_grid_catalog", self._handle, _lib.ptr(idx), ctypes.c_int64(n), ctypes.byref(params),
                  _lib.ptr(planes), _lib.ptr(status), _lib.ptr(counts))
        elapsed = (perf_counter() - start) / n
        radius = max(0, int(centroid_radius))
        results = []
        for k in range(n):
            stored = int(counts[k, 1])
            x, y, flux = (planes[c, k, :stored].copy() for c in range(3))
            refine = {"enabled": radius > 0, "radius": radius, "stored_count": stored,
                      "refined_count": int(status[k, :stored].sum()) if radius else 0,
                      "failed_count": int(stored - status[k, :stored].sum()) if radius else 0,
                      "max_shift_px": float(np.hypot(x.astype(np.float64) - planes[3, k, :stored],
                                                     y.astype(np.float64) - planes[4, k, :stored])[
                          status[k, :stored] != 0].max(initial=0.0)) if radius else 0.0,
                      "mode": ("off" if not radius else "resident_gpu_global_mean_centroid"
                               if centroid_global_mean_background else "resident_gpu_window_centroid"),
                      "background_mode": ("off" if not radius else "global_mean"
                                          if centroid_global_mean_background else "local_median"),
                      "background": None}
            results.append({
                "frame_index": int(idx[k]), "count": int(counts[k, 0]), "stored_count": stored,
                "grid_cols": int(grid_cols), "grid_rows": int(grid_rows),
                "candidates_per_cell": int(candidates_per_cell), "max_output_candidates": mo,
                "min_separation_px": float(min_separation_px),
                "catalog_sort_mode": "device_bitonic_u64_keys", "catalog_topk_mode": "deterministic_cta_per_cell",
                "catalog_timing_model": "single_stream_one_sync", "catalog_batch_size": n,
                "catalog_stream_limit": 1, "catalog_stream_count": 1, "catalog_batch_sync_count": 1,
                "catalog_sync_phase_count": 1, "catalog_download_mode": "bulk_full_capacity",
                "catalog_workspace_layout": "contiguous_soa", "catalog_grid_workspace_allocation_count": 1,
                "catalog_output_workspace_allocation_count": 1, "catalog_output_download_copy_count": 1,
                "catalog_centroid_before_download_copy_count": 0, "catalog_output_download_bytes": int(planes.nbytes),
                "catalog_centroid_mean_sync_mode": ("fused_with_catalog_sync" if radius and
                                                    centroid_global_mean_background else
                                                    "not_applicable_local_median" if radius else "off"),
                "catalog_centroid_mean_blocks": 128 if radius and centroid_global_mean_background else 0,
                "catalog_enqueue_s": 0.0, "catalog_sync_s": elapsed, "catalog_count_download_s": 0.0,
                "catalog_centroid_refine_s": 0.0, "catalog_output_download_s": 0.0, "catalog_native_s": elapsed,
                "centroid_refine": refine, "x": x, "y": y, "flux": flux})
        return results

    def star_grid_top_nms_candidates_batch(self, indices: Any, threshold: float, grid_cols: int, grid_rows: int,
                                           candidates_per_cell: int, max_output_candidates: int,
                                           min_separation_px: float) -> list[dict[str, Any]]:
        return self._grid_catalog(indices, threshold, grid_cols, grid_rows, candidates_per_cell,
                                  max_output_candidates, min_separation_px, 0, False, False)

    def star_grid_top_nms_candidates_batch_deterministic(self, indices: Any, threshold: float, grid_cols: int,
                                                         grid_rows: int, candidates_per_cell: int,
                                                         max_output_candidates: int,
                                                         min_separation_px: float) -> list[dict[str, Any]]:
        return self._grid_catalog(indices, threshold, grid_cols, grid_rows, candidates_per_cell,
                                  max_output_candidates, min_separation_px, 0, False, True)

    def star_grid_top_nms_candidates_batch_centroid(self, indices: Any, threshold: float, grid_cols: int,
                                                    grid_rows: int, candidates_per_cell: int,
                                                    max_output_candidates: int, min_separation_px: float,
                                                    centroid_radius: int,
                                                    centroid_global_mean_background: bool = False):
        return self._grid_catalog(indices, threshold, grid_cols, grid_rows, candidates_per_cell,
                                  max_output_candidates, min_separation_px, centroid_radius,
                                  centroid_global_mean_background, False)

    def star_grid_top_nms_candidates_batch_deterministic_centroid(
            self, indices: Any, threshold: float, grid_cols: int, grid_rows: int, candidates_per_cell: int,
            max_output_candidates: int, min_separation_px: float, centroid_radius: int,
            centroid_global_mean_background: bool = False) -> list[dict[str, Any]]:
        """native_bindings.cpp:12622-12645: the resident triangle path's batch
        catalog (resident_cuda.py:10914)."""
        return self._grid_catalog(indices, threshold, grid_cols, grid_rows, candidates_per_cell,
                                  max_output_candidates, min_separation_px, centroid_radius,
                                  centroid_global_mean_background, True)

    def _grid_single(self, index: int, *args) -> dict[str, Any]:
        result = self._grid_catalog([int(index)], *args)[0]
        result.pop("frame_index")
        return result

    def star_grid_top_nms_candidates(self, index: int, threshold: float, grid_cols: int, grid_rows: int,
                                     candidates_per_cell: int, max_output_candidates: int,
                                     min_separation_px: float) -> dict[str, Any]:
        return self._grid_single(index, threshold, grid_cols, grid_rows, candidates_per_cell, max_output_candidates,
                                 min_separation_px, 0, False, False)

    def star_grid_top_nms_candidates_deterministic(self, index: int, threshold: float, grid_cols: int,
                                                   grid_rows: int, candidates_per_cell: int,
                                                   max_output_candidates: int,
                                                   min_separation_px: float) -> dict[str, Any]:
        return self._grid_single(index, threshold, grid_cols, grid_rows, candidates_per_cell, max_output_candidates,
                                 min_separation_px, 0, False, True)

    def star_grid_top_nms_candidates_centroid(self, index: int, threshold: float, grid_cols: int, grid_rows: int,
                                              candidates_per_cell: int, max_output_candidates: int,
                                              min_separation_px: float, centroid_radius: int,
                                              centroid_global_mean_background: bool = False) -> dict[str, Any]:
        return self._grid_single(index, threshold, grid_cols, grid_rows, candidates_per_cell, max_output_candidates,
                                 min_separation_px, centroid_radius, centroid_global_mean_background, False)

    def star_grid_top_nms_candidates_deterministic_centroid(self, index: int, threshold: float, grid_cols: int,
                                                            grid_rows: int, candidates_per_cell: int,
                                                            max_output_candidates: int, min_separation_px: float,
                                                            centroid_radius: int,
                                                            centroid_global_mean_background: bool = False):
        return self._grid_single(index, threshold, grid_cols, grid_rows, candidates_per_cell, max_output_candidates,
                                 min_separation_px, centroid_radius, centroid_global_mean_background, True)

    # ---- star catalogs (star_detect.py:121-168) -------------------------------------
    def detect_stars(self, indices: Any, threshold_sigma: float = 5.0, max_stars: int = 500,
                     background: float | None = None, noise: float | None = None, window_radius: int = 4,
                     min_separation_px: float = 2.0, with_info: bool = False, catalog_min_fwhm: float = 0.0,
                     catalog_max_eccentricity: float = 1.0, mesh_cell: int = 0):
        """detect_stars semantics per resident frame -> list of structured arrays
        (x, y, flux, peak, fwhm, eccentricity, snr, sharpness, npix), brightest first.

        The first 80 stars passing the optional catalog shape filter stay on
        the device as each frame's registration catalog.  mesh_cell > 0
        thresholds against a background mesh of that cell size instead of
        the global median / MAD."""
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1))
        if idx.size == 0:
            raise ValueError("indices must contain at least one frame index")
        params = _lib.StarParams(float(threshold_sigma), int(max_stars), int(window_radius), float(min_separation_px),
                                 np.nan if background is None else float(background),
                                 np.nan if noise is None else float(noise), float(catalog_min_fwhm),
                                 float(catalog_max_eccentricity), int(mesh_cell))
        stars = np.zeros((idx.size, int(max_stars)), dtype=_lib.STAR_DTYPE)
        counts = np.zeros(idx.size, dtype=np.int32)
        info = (_lib.StarFrameInfo * idx.size)()
        _lib.call("gg_stack_detect_stars", self._handle, _lib.ptr(idx), ctypes.c_int64(idx.size), ctypes.byref(params),
                  _lib.ptr(stars), _lib.ptr(counts), info)
        catalogs = [stars[k, : counts[k]].copy() for k in range(idx.size)]
        if with_info:
            meta = [{"median": float(i.median), "mad": float(i.mad), "noise": float(i.noise),
                     "threshold": float(i.threshold), "candidates": int(i.candidates),
                     "valid_pixels": int(i.valid_pixels)} for i in info]
            return catalogs, meta
        return catalogs

    def cosmetic_mask_frames(self, indices: Any, hot_sigma: float = 8.0, cold_sigma: float = 8.0,
                             structure_sigma: float = 1.5, min_neighbor_support: int = 2,
                             star_protection: bool = False, star_threshold_sigma: float = 5.0,
                             star_protection_radius_px: float = 3.0, star_min_pixels: int = 3,
                             star_max_sharpness: float = 0.95, apply: bool = True) -> list[dict[str, Any]]:
        """Isolated hot / cold pixels of each frame (cpu/cosmetic.py rules)
        set to NaN on the device (apply=False only counts); returns the
        per-frame counts and statistics."""
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1))
        if idx.size == 0:
            return []
        params = _lib.CosmeticParams(float(hot_sigma), float(cold_sigma), float(structure_sigma),
                                     int(min_neighbor_support), int(bool(star_protection)),
                                     float(star_threshold_sigma), float(star_protection_radius_px),
                                     int(star_min_pixels), float(star_max_sharpness), int(bool(apply)))
        out = (_lib.CosmeticResult * idx.size)()
        _lib.call("gg_stack_cosmetic_mask", self._handle, _lib.ptr(idx), ctypes.c_int64(idx.size),
                  ctypes.byref(params), out)
        model = "star_protected_isolated_cosmetic" if star_protection else "isolated_cosmetic"
        return [{"frame_index": int(idx[k]), "hot_pixels": int(r.hot_pixels), "cold_pixels": int(r.cold_pixels),
                 "candidate_hot_pixels": int(r.candidate_hot_pixels),
                 "candidate_cold_pixels": int(r.candidate_cold_pixels),
                 "star_protected_hot_pixels": int(r.star_protected_hot_pixels),
                 "star_protected_cold_pixels": int(r.star_protected_cold_pixels), "median": float(r.median),
                 "sigma": float(r.sigma), "star_count": int(r.star_count), "applied": bool(apply),
                 "model": model} for k, r in enumerate(out)]

    # ---- source DQ: threshold-only cosmetic mask (native_bindings.cpp:3243-3400, 4307-4620) ----
    def _cosmetic_threshold(self, indices: Any, lows: Any, highs: Any, apply: bool) -> tuple[np.ndarray, np.ndarray,
                                                                                               np.ndarray, np.ndarray,
                                                                                               dict[str, float]]:
        idx = np.ascontiguousarray(np.asarray(list(indices), dtype=np.int64).reshape(-1))
        lo = np.ascontiguousarray(np.asarray(list(lows), dtype=np.float32).reshape(-1))
        hi = np.ascontiguousarray(np.asarray(list(highs), dtype=np.float32).reshape(-1))
        if idx.size != lo.size or idx.size != hi.size:
            raise ValueError("indices, low_thresholds, and high_thresholds must have the same length")
        if idx.size > 65535:
            raise ValueError("batch cosmetic threshold application supports at most 65535 frames per launch")
        counts = np.zeros((idx.size, 3), dtype=np.int64)
        t0 = perf_counter()
        if idx.size:
            _lib.call("gg_stack_cosmetic_threshold", self._handle, _lib.ptr(idx), ctypes.c_int64(idx.size),
                      _lib.ptr(lo), _lib.ptr(hi), ctypes.c_int32(int(bool(apply))), _lib.ptr(counts))
        t1 = perf_counter()
        return idx, lo, hi, counts, {"kernel_enqueue_s": t1 - t0, "sync_s": 0.0, "device_counts_download_s": 0.0,
                                     "mask_upload_s": 0.0}

    def _cosmetic_threshold_frame(self, index: int, low_threshold: float, high_threshold: float, apply: bool):
        t0 = perf_counter()
        _, lo, hi, counts, timing = self._cosmetic_threshold([int(index)], [low_threshold], [high_threshold], apply)
        hot, cold, nonfinite = (int(x) for x in counts[0])
        name = "apply" if apply else "count"
        return {"schema_version": 1, "native_method": f"ResidentCalibratedStack.{name}_cosmetic_threshold_mask_frame",
                "frame_index": int(index), "total_pixels": int(self.height * self.width),
                "low_threshold": float(lo[0]), "high_threshold": float(hi[0]), "hot_samples": hot,
                "cold_samples": cold, "nonfinite_samples": nonfinite, "cosmetic_corrected_samples": hot + cold,
                "invalid_samples": hot + cold + nonfinite, "applied": bool(apply) and hot + cold + nonfinite > 0,
                **timing, "total_s": perf_counter() - t0, "detector_execution": f"cuda_threshold_{name}"}

    def apply_cosmetic_threshold_mask_frame(self, index: int, low_threshold: float,
                                            high_threshold: float) -> dict[str, Any]:
        """Samples of frame `index` above high_threshold (hot), below
        low_threshold (cold) or non-finite become NaN; returns the counts."""
        return self._cosmetic_threshold_frame(index, low_threshold, high_threshold, True)

    def count_cosmetic_threshold_mask_frame(self, index: int, low_threshold: float,
                                            high_threshold: float) -> dict[str, Any]:
        """The counts of apply_cosmetic_threshold_mask_frame; the frame is not changed."""
        return self._cosmetic_threshold_frame(index, low_threshold, high_threshold, False)

    def _cosmetic_threshold_frames(self, indices: Any, low_thresholds: Any, high_thresholds: Any, apply: bool):
        t0 = perf_counter()
        idx, lo, hi, counts, timing = self._cosmetic_threshold(indices, low_thresholds, high_thresholds, apply)
        name = "apply" if apply else "count"
        method = f"ResidentCalibratedStack.{name}_cosmetic_threshold_mask_frames"
        frames = []
        for k in range(idx.size):
            hot, cold, nonfinite = (int(x) for x in counts[k])
            frames.append({"schema_version": 1, "native_method": method,
                           "per_frame_native_method": f"ResidentCalibratedStack.{name}_cosmetic_threshold_mask_frame",
                           "frame_index": int(idx[k]), "batch_position": k,
                           "total_pixels": int(self.height * self.width), "low_threshold": float(lo[k]),
                           "high_threshold": float(hi[k]), "hot_samples": hot, "cold_samples": cold,
                           "nonfinite_samples": nonfinite, "cosmetic_corrected_samples": hot + cold,
                           "invalid_samples": hot + cold + nonfinite,
                           "applied": bool(apply) and hot + cold + nonfinite > 0,
                           "batch_single_kernel_launch": True, "batch_single_sync": True,
                           "batch_frame_count": int(idx.size), **timing,
                           "detector_execution": f"cuda_threshold_{name}_batch"})
        tot = counts.sum(axis=0) if idx.size else np.zeros(3, dtype=np.int64)
        hot, cold, nonfinite = (int(x) for x in tot)
        return {"schema_version": 1, "native_method": method, "frame_count": int(idx.size),
                "total_pixels_per_frame": int(self.height * self.width), "hot_samples": hot, "cold_samples": cold,
                "nonfinite_samples": nonfinite, "cosmetic_corrected_samples": hot + cold,
                "invalid_samples": hot + cold + nonfinite, "applied": bool(apply) and hot + cold + nonfinite > 0,
                **timing, "batch_single_kernel_launch": True, "batch_single_sync": True,
                "detector_execution": f"cuda_threshold_{name}_batch", "total_s": perf_counter() - t0,
                "frames": frames}

    def apply_cosmetic_threshold_mask_frames(self, indices: Any, low_thresholds: Any,
                                             high_thresholds: Any) -> dict[str, Any]:
        """apply_cosmetic_threshold_mask_frame over several frames (one
        threshold pair per frame) in one launch."""
        return self._cosmetic_threshold_frames(indices, low_thresholds, high_thresholds, True)

    def count_cosmetic_threshold_mask_frames(self, indices: Any, low_thresholds: Any,
                                             high_thresholds: Any) -> dict[str, Any]:
        """count_cosmetic_threshold_mask_frame over several frames in one launch."""
        return self._cosmetic_threshold_frames(indices, low_thresholds, high_thresholds, False)

    def apply_invalid_mask_frame(self, index: int, invalid_mask: Any) -> dict[str, Any]:
        """Source-DQ invalid samples (non-zero mask entries) become NaN."""
        mask = np.ascontiguousarray(np.asarray(invalid_mask).astype(np.uint8))
        if mask.shape != (self.height, self.width):
            raise ValueError("invalid_mask must have the frame's shape")
        n = ctypes.c_int64()
        _lib.call("gg_stack_apply_invalid_mask", self._handle, ctypes.c_int64(int(index)), _lib.ptr(mask),
                  ctypes.byref(n))
        return {"frame_index": int(index), "invalid_samples": int(n.value)}

    def register_frames_triangle(self, reference_index: int, indices: Any, transform_model: str = "similarity",
                                 min_inliers: int = 6, tolerance_px: float = 3.0, max_stars: int = 80,
                                 neighbors: int = 5, descriptor_radius: float = 0.1, max_descriptors: int = 1200,
                                 max_candidates: int = 1500) -> list[dict[str, Any]]:
        """estimate_triangle_asterism_transform of each frame's catalog (from its
        last detect_stars) against the reference frame's catalog, all on the
        device; returns one StarRegistration-like dict per index."""
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1))
        if idx.size == 0:
            raise ValueError("indices must contain at least one frame index")
        params = _register_params(transform_model, min_inliers, tolerance_px, max_stars, neighbors,
                                  descriptor_radius, max_descriptors, max_candidates)
        out = (_lib.Registration * idx.size)()
        _lib.call("gg_stack_register_frames", self._handle, ctypes.c_int64(int(reference_index)), _lib.ptr(idx),
                  ctypes.c_int64(idx.size), ctypes.byref(params), out)
        return [_registration_dict(r, None, transform_model) for r in out]

    # ---- alignment metrics / refinement (native_bindings.cpp:10186-10417) ------------
    def _matrices(self, matrices: Any, count: int) -> np.ndarray:
        mats = np.ascontiguousarray(np.asarray(matrices, dtype=np.float64).reshape(-1, 3, 3))
        if mats.shape[0] != count:
            raise ValueError("batch refine requires one seed matrix per moving frame")
        return mats

    def matrix_alignment_metrics(self, reference_index: int, moving_indices: Any, matrices: Any,
                                 sample_stride: int = 1) -> list[dict[str, Any]]:
        """matrix_alignment_metrics_f32 of each moving frame against the reference frame."""
        idx = np.ascontiguousarray(np.asarray(moving_indices, dtype=np.int64).reshape(-1))
        if idx.size == 0:
            return []
        mats = self._matrices(matrices, idx.size)
        out = (_lib.AlignmentMetrics * idx.size)()
        _lib.call("gg_stack_alignment_metrics", self._handle, ctypes.c_int64(int(reference_index)), _lib.ptr(idx),
                  ctypes.c_int64(idx.size), _lib.ptr(mats), ctypes.c_int32(int(sample_stride)), out)
        return [_metrics_dict(m, "matrix_alignment_metrics_cuda") for m in out]

    def refine_matrix_translation_candidates_batch_to_reference(
            self, reference_index: int, moving_indices: Any, matrices: Any, search_radius_px: float = 1.0,
            coarse_step_px: float = 0.25, fine_radius_px: float = 0.25, fine_step_px: float = 0.0625,
            coarse_sample_stride: int = 4, final_sample_stride: int = 1) -> list[dict[str, Any]]:
        """Coarse-to-fine translation refinement of each moving frame's matrix
        against the reference frame (native_bindings.cpp:10186-10417)."""
        if search_radius_px < 0.0 or fine_radius_px < 0.0:
            raise ValueError("search radii must be non-negative")
        if coarse_step_px <= 0.0 or fine_step_px <= 0.0:
            raise ValueError("search steps must be positive")
        if coarse_sample_stride <= 0 or final_sample_stride <= 0:
            raise ValueError("sample strides must be positive")
        idx = np.ascontiguousarray(np.asarray(moving_indices, dtype=np.int64).reshape(-1))
        if idx.size == 0:
            return []
        mats = self._matrices(matrices, idx.size)
        params = _lib.RefineParams(float(search_radius_px), float(coarse_step_px), float(fine_radius_px),
                                   float(fine_step_px), int(coarse_sample_stride), int(final_sample_stride))
        out = (_lib.RefineResult * idx.size)()
        _lib.call("gg_stack_refine_translation", self._handle, ctypes.c_int64(int(reference_index)), _lib.ptr(idx),
                  ctypes.c_int64(idx.size), _lib.ptr(mats), ctypes.byref(params), out)
        results = []
        for k, r in enumerate(out):
            results.append({
                "matrix": np.asarray(r.matrix, dtype=np.float32).reshape(3, 3).tolist(),
                "dx_correction": float(r.dx_correction), "dy_correction": float(r.dy_correction),
                "metrics": _metrics_dict(r.metrics, "matrix_alignment_metrics_cuda_candidate_grid"),
                "coarse_candidates": int(r.coarse_candidates), "fine_candidates": int(r.fine_candidates),
                "search_radius_px": float(search_radius_px), "coarse_step_px": float(coarse_step_px),
                "fine_radius_px": float(fine_radius_px), "fine_step_px": float(fine_step_px),
                "coarse_sample_stride": int(coarse_sample_stride), "final_sample_stride": int(final_sample_stride),
                "reference_index": int(reference_index), "moving_index": int(idx[k]), "batch_index": k,
                "batch_count": int(idx.size), "batch_model": "gb300_candidate_grid_batch_refine"})
        return results

    # ---- gradient refinement (no reference counterpart) -----------------------------
    _MODELS = {"translation": _lib.GG_TRANSFORM_TRANSLATION, "similarity": _lib.GG_TRANSFORM_SIMILARITY,
               "affine": _lib.GG_TRANSFORM_AFFINE}
    _INTERPS = {"bilinear": _lib.GG_INTERP_BILINEAR, "lanczos3": _lib.GG_INTERP_LANCZOS3}

    def _gradient_params(self, model, interpolation, sample_stride, row_stride, stats_passes, iterations,
                         min_samples, clip_sigma, mask_shift_px, tolerance_px, max_step_px) -> _lib.GradientRefineParams:
        if model not in self._MODELS:
            raise ValueError("model must be translation, similarity or affine")
        if interpolation not in self._INTERPS:
            raise ValueError("interpolation must be bilinear or lanczos3")
        return _lib.GradientRefineParams(self._MODELS[model], self._INTERPS[interpolation], int(sample_stride),
                                         int(row_stride), int(stats_passes), int(iterations), int(min_samples), 0,
                                         float(clip_sigma), float(mask_shift_px), float(tolerance_px),
                                         float(max_step_px))

    def refine_matrix_gradient_batch_to_reference(
            self, reference_index: int, moving_indices: Any, matrices: Any, model: str = "similarity",
            interpolation: str = "lanczos3", sample_stride: int = 2, stats_passes: int = 3, iterations: int = 8,
            min_samples: int = 256, clip_sigma: float = 5.0, mask_shift_px: float = 1.0,
            tolerance_px: float = 1.0e-3, max_step_px: float = 2.0, row_stride: int = 0) -> list[dict[str, Any]]:
        """Gauss-Newton refinement of each moving frame's affine matrix against
        the reference frame on the device (masked, photometrically matched
        sum of squares; the warp adjoint's position derivatives).  Samples
        every sample_stride-th column of every row_stride-th row (0: a square
        grid of sample_stride)."""
        idx = np.ascontiguousarray(np.asarray(moving_indices, dtype=np.int64).reshape(-1))
        if idx.size == 0:
            return []
        mats = self._matrices(matrices, idx.size)
        params = self._gradient_params(model, interpolation, sample_stride, row_stride, stats_passes, iterations,
                                       min_samples, clip_sigma, mask_shift_px, tolerance_px, max_step_px)
        out = (_lib.GradientRefineResult * idx.size)()
        _lib.call("gg_stack_refine_gradient", self._handle, ctypes.c_int64(int(reference_index)), _lib.ptr(idx),
                  ctypes.c_int64(idx.size), _lib.ptr(mats), ctypes.byref(params), out)
        status = {1: "converged", 2: "iteration_cap", -1: "too_few_samples", -2: "singular"}
        return [{"matrix": np.asarray(r.matrix, dtype=np.float64).reshape(3, 3), "alpha": float(r.alpha),
                 "beta": float(r.beta), "sigma": float(r.sigma), "rms": float(r.rms),
                 "last_step_px": float(r.last_step_px), "samples": int(r.samples), "iterations": int(r.iterations),
                 "status": status.get(int(r.status), str(int(r.status))), "ok": int(r.status) >= 1,
                 "moving_index": int(idx[k]), "reference_index": int(reference_index)} for k, r in enumerate(out)]

    def gradient_normal_equations(self, reference_index: int, moving_indices: Any, thetas: Any, photometric: Any,
                                  model: str = "similarity", interpolation: str = "lanczos3", sample_stride: int = 2,
                                  clip_sigma: float = 5.0, mask_shift_px: float = 1.0,
                                  row_stride: int = 0) -> np.ndarray:
        """One accumulation pass of the gradient refinement -> (n, 48) sums:
        J^T J upper triangle (36), J^T r (8), sum r^2, kept count, 0, 0."""
        idx = np.ascontiguousarray(np.asarray(moving_indices, dtype=np.int64).reshape(-1))
        th = np.ascontiguousarray(np.asarray(thetas, dtype=np.float64).reshape(idx.size, 6))
        ph = np.ascontiguousarray(np.asarray(photometric, dtype=np.float64).reshape(idx.size, 3))
        params = self._gradient_params(model, interpolation, sample_stride, row_stride, 1, 1, 16, clip_sigma,
                                       mask_shift_px, 0.0, 1.0)
        out = np.zeros((idx.size, 48), dtype=np.float64)
        _lib.call("gg_stack_gradient_normal_equations", self._handle, ctypes.c_int64(int(reference_index)),
                  _lib.ptr(idx), ctypes.c_int64(idx.size), _lib.ptr(th), _lib.ptr(ph), ctypes.byref(params),
                  _lib.ptr(out))
        return out

    # ---- warps (native_bindings.cpp:8900-9924) ------------------------------------
    @property
    def tma_enabled(self) -> bool:
        flag = ctypes.c_int()
        _lib.call("gg_stack_tma_enabled", self._handle, ctypes.byref(flag))
        return bool(flag.value)

    def warp_frames_async(self, indices: Any, matrices: Any, interpolation: int, fill: float = np.nan,
                          clamping_threshold: float = -1.0, track_coverage: bool = False) -> None:
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1))
        mats = np.asarray(matrices)
        if mats.dtype != np.float64:
            mats = np.asarray(np.asarray(mats, dtype=np.float32), dtype=np.float64)
        mats = np.ascontiguousarray(mats.reshape(-1, 3, 3))
        if mats.shape[0] != idx.size:
            raise ValueError("matrices must have shape (len(indices), 3, 3)")
        if idx.size == 0:
            return
        _lib.call("gg_stack_warp_frames", self._handle, _lib.ptr(idx), ctypes.c_int64(idx.size), _lib.ptr(mats),
                  int(interpolation), ctypes.c_float(fill), ctypes.c_float(clamping_threshold),
                  int(bool(track_coverage)))

    def _warp_timed(self, indices, matrices, interpolation, fill, clamp, track_coverage, name) -> dict[str, Any]:
        start = perf_counter()
        self.warp_frames_async(indices, matrices, interpolation, fill, clamp, track_coverage)
        enqueue = perf_counter()
        self.synchronize()
        done = perf_counter()
        n = int(np.asarray(indices).size)
        return {"schema_version": 1, "method": name, "frames": n, "dispatch": "slot_swap_batches",
                "interpolation": {0: "nearest", 1: "bilinear", 3: "lanczos3"}[interpolation],
                "track_coverage": bool(track_coverage), "tma_staged": self.tma_enabled,
                "enqueue_s": enqueue - start, "sync_s": done - enqueue, "total_s": done - start}

    def apply_translation_frame(self, index: int, dx: int, dy: int, fill: float = np.nan) -> None:
        self.warp_frames_async([index], _translation_matrix(float(int(dx)), float(int(dy)))[None],
                               _lib.GG_INTERP_NEAREST, fill)
        self.synchronize()

    def apply_translation_bilinear_frame(self, index: int, dx: float, dy: float, fill: float = np.nan) -> None:
        self.warp_frames_async([index], _translation_matrix(float(dx), float(dy))[None], _lib.GG_INTERP_BILINEAR,
                               fill)
        self.synchronize()

    def apply_matrix_bilinear_frame(self, index: int, matrix: Any, fill: float = np.nan) -> None:
        self.warp_frames_async([index], _matrix64(matrix)[None], _lib.GG_INTERP_BILINEAR, fill)
        self.synchronize()

    def apply_matrix_lanczos3_frame(self, index: int, matrix: Any, fill: float = np.nan,
                                    clamping_threshold: float = -1.0) -> None:
        self.warp_frames_async([index], _matrix64(matrix)[None], _lib.GG_INTERP_LANCZOS3, fill, clamping_threshold)
        self.synchronize()

    def apply_matrix_bilinear_frames(self, indices: Any, matrices: Any, fill: float = np.nan, *rest) -> dict:
        """(indices, matrices, fill, track_coverage) or (..., max_chunk_capacity_frames, track_coverage)."""
        track = bool(rest[-1]) if rest else True
        return self._warp_timed(indices, matrices, _lib.GG_INTERP_BILINEAR, fill, -1.0, track,
                                "apply_matrix_bilinear_frames")

    def apply_matrix_lanczos3_frames(self, indices: Any, matrices: Any, fill: float = np.nan,
                                     clamping_threshold: float = -1.0, *rest) -> dict:
        """(..., clamping_threshold, track_coverage) or (..., max_chunk_capacity_frames, track_coverage)."""
        track = bool(rest[-1]) if rest else True
        return self._warp_timed(indices, matrices, _lib.GG_INTERP_LANCZOS3, fill, clamping_threshold, track,
                                "apply_matrix_lanczos3_frames")

    def reset_warp_coverage(self) -> None:
        _lib.call("gg_stack_reset_warp_coverage", self._handle)

    def accumulate_full_warp_coverage_frame(self) -> None:
        _lib.call("gg_stack_accumulate_full_warp_coverage_frame", self._handle)

    def warp_coverage_map(self) -> np.ndarray:
        info = self._info()
        out = np.empty((info.height, info.width), np.float32)
        _lib.call("gg_stack_download_warp_coverage", self._handle, _lib.ptr(out))
        return out

    # ---- statistics ------------------------------------------------------------
    def frame_global_stats(self, index: int) -> dict[str, Any]:
        return self.frames_global_stats([index])[0]

    def frames_global_stats(self, indices: Any) -> list[dict[str, Any]]:
        idx = np.ascontiguousarray(np.asarray(indices, dtype=np.int64).reshape(-1))
        out = (_lib.FrameStats * idx.size)()
        _lib.call("gg_stack_frame_stats", self._handle, _lib.ptr(idx), ctypes.c_int64(idx.size), out)
        return [
            {"mean": float(s.mean), "std": float(s.std), "valid_pixels": int(s.valid_pixels),
             "total_pixels": int(s.total_pixels), "nonfinite_pixels": int(s.total_pixels - s.valid_pixels),
             "model": "float_float_device_sum"}
            for s in out
        ]

    # ---- local normalisation (native_bindings.cpp:10645-11200) ---------------------
    def _grid_dims(self, tile_height: int, tile_width: int) -> tuple[int, int]:
        if int(tile_height) <= 0 or int(tile_width) <= 0:
            raise ValueError("tile dimensions must be positive")
        info = self._info()
        return (-(-int(info.height) // int(tile_height)), -(-int(info.width) // int(tile_width)))

    def frame_pair_grid_stats_batch(self, reference_index: int, source_indices: Any, tile_height: int,
                                    tile_width: int) -> dict[str, Any]:
        """Per-tile float32 mean / std of each source frame and of the
        reference over the pixels finite in both, and the pixel counts."""
        idx = np.ascontiguousarray(np.asarray(source_indices, dtype=np.int64).reshape(-1))
        rows, cols = self._grid_dims(tile_height, tile_width)
        start = perf_counter()
        shape = (idx.size, rows, cols)
        sm, ss, rm, rs = (np.zeros(shape, np.float32) for _ in range(4))
        valid = np.zeros(shape, np.uint64)
        if idx.size:
            _lib.call("gg_stack_pair_grid_stats", self._handle, ctypes.c_int64(int(reference_index)), _lib.ptr(idx),
                      ctypes.c_int64(idx.size), int(tile_height), int(tile_width), _lib.ptr(sm), _lib.ptr(ss),
                      _lib.ptr(rm), _lib.ptr(rs), _lib.ptr(valid))
        frames = []
        for k in range(idx.size):
            frames.append({"source_mean": sm[k], "source_std": ss[k], "reference_mean": rm[k], "reference_std": rs[k],
                           "valid_pixels": valid[k], "grid_rows": rows, "grid_cols": cols,
                           "tile_height": int(tile_height), "tile_width": int(tile_width),
                           "valid_pixel_total": int(valid[k].sum(dtype=np.uint64)),
                           "model": "resident_grid_pair_mean_std", "source_index": int(idx[k]),
                           "reference_index": int(reference_index), "batch_position": k})
        return {"schema_version": 1, "model": "resident_grid_pair_mean_std_batch",
                "batch_model": "gb300_tile_pair_float_float_sums", "reference_index": int(reference_index),
                "source_count": int(idx.size), "grid_rows": rows, "grid_cols": cols, "grid_count": rows * cols,
                "tile_height": int(tile_height), "tile_width": int(tile_width),
                "source_indices": idx.astype(np.int32), "total_s": perf_counter() - start, "frames": frames}

    def frame_pair_grid_stats(self, reference_index: int, source_index: int, tile_height: int,
                              tile_width: int) -> dict[str, Any]:
        frame = self.frame_pair_grid_stats_batch(reference_index, [source_index], tile_height, tile_width)["frames"][0]
        for key in ("source_index", "reference_index", "batch_position"):
            frame.pop(key)
        return frame

    def apply_grid_normalization_frames(self, frame_indices: Any, scales: Any, offsets: Any, tile_height: int,
                                        tile_width: int) -> dict[str, Any]:
        """In place v * scale + offset per tile for each frame (coefficients
        of shape (frame_count, grid_rows, grid_cols))."""
        idx = np.ascontiguousarray(np.asarray(frame_indices, dtype=np.int64).reshape(-1))
        sc = np.ascontiguousarray(np.asarray(scales, dtype=np.float32))
        of = np.ascontiguousarray(np.asarray(offsets, dtype=np.float32))
        if sc.ndim != 3 or of.ndim != 3:
            raise ValueError("scales and offsets must have shape (frame_count, grid_rows, grid_cols)")
        if sc.shape[0] != idx.size or of.shape[0] != idx.size:
            raise ValueError("coefficient frame count must match frame_indices length")
        if sc.shape != of.shape:
            raise ValueError("scales and offsets grid shapes must match")
        if int(tile_height) <= 0 or int(tile_width) <= 0:
            raise ValueError("tile dimensions must be positive")
        start = perf_counter()
        if idx.size:
            _lib.call("gg_stack_apply_grid_normalization", self._handle, _lib.ptr(idx), ctypes.c_int64(idx.size),
                      _lib.ptr(sc), _lib.ptr(of), int(sc.shape[1]), int(sc.shape[2]), int(tile_height),
                      int(tile_width))
        return {"schema_version": 1, "mode": "in_place_device_update_batch",
                "model": "resident_grid_mean_std_batch_apply", "frame_count": int(idx.size),
                "grid_rows": int(sc.shape[1]), "grid_cols": int(sc.shape[2]),
                "grid_count": int(sc.shape[1] * sc.shape[2]), "coefficient_count": int(sc.size),
                "coefficient_bytes": int(sc.nbytes + of.nbytes), "total_s": perf_counter() - start}

    def apply_grid_normalization_frame(self, index: int, scales: Any, offsets: Any, tile_height: int,
                                       tile_width: int) -> dict[str, Any]:
        sc = np.asarray(scales, dtype=np.float32)
        of = np.asarray(offsets, dtype=np.float32)
        if sc.ndim != 2 or of.ndim != 2:
            raise ValueError("scales and offsets must have shape (grid_rows, grid_cols)")
        if sc.shape != of.shape:
            raise ValueError("scales and offsets shapes must match")
        out = self.apply_grid_normalization_frames([index], sc[None], of[None], tile_height, tile_width)
        out.update(mode="in_place_device_update", model="resident_grid_mean_std", frame_index=int(index))
        return out

    def apply_global_normalization_frame(self, index: int, scale: float, offset: float) -> dict[str, Any]:
        start = perf_counter()
        _lib.call("gg_stack_apply_global_normalization", self._handle, ctypes.c_int64(int(index)),
                  ctypes.c_float(scale), ctypes.c_float(offset))
        return {"schema_version": 1, "mode": "in_place_device_update", "model": "resident_global_mean_std",
                "frame_index": int(index), "total_s": perf_counter() - start}

    def device_frame_weights(self) -> np.ndarray:
        """The frame weights currently on the device (synchronises)."""
        out = np.empty(self.frame_count, np.float32)
        _lib.call("gg_stack_download_weights", self._handle, _lib.ptr(out))
        return out

    def local_normalize_grid(self, reference_index: int, source_indices: Any, tile: int = 256, eps: float = 1.0e-6,
                             update_weights: bool = True, download: bool = False):
        """Statistics, coefficients and the in-place apply on the device (no
        host round trip unless download=True, which returns (scales, offsets))."""
        idx = np.ascontiguousarray(np.asarray(source_indices, dtype=np.int64).reshape(-1))
        if idx.size == 0:
            return None
        rows, cols = self._grid_dims(tile, tile)
        sc = np.empty((idx.size, rows, cols), np.float32) if download else None
        of = np.empty((idx.size, rows, cols), np.float32) if download else None
        _lib.call("gg_stack_local_normalize_grid", self._handle, ctypes.c_int64(int(reference_index)), _lib.ptr(idx),
                  ctypes.c_int64(idx.size), int(tile), int(tile), ctypes.c_double(eps), int(bool(update_weights)),
                  _lib.ptr(sc), _lib.ptr(of))
        return (sc, of) if download else None

    # ---- integration -------------------------------------------------------------
    def _weights(self, weights: Any | None) -> np.ndarray | None:
        if weights is None:
            return None
        w = np.ascontiguousarray(np.asarray(weights, dtype=np.float32).reshape(-1))
        if w.shape != (self.frame_count,):
            raise ValueError("weights must have shape (frame_count,)")
        return w

    def compute_frame_weights(self, mode: str = "simple_snr", prior: Any | None = None, eps: float = 1.0e-6,
                              download: bool = True) -> np.ndarray | None:
        """Frame weights on the device (simple_snr: resident_cuda.py:1948-1956).

        The weights stay in the stack for ``integrate_async(weights="device")``;
        with download=True they are also returned (one sync).
        """
        modes = {"unit": 0, "prior": 0, "simple_snr": 1}
        if mode not in modes:
            raise ValueError("weighting mode must be unit, prior or simple_snr")
        p = self._weights(prior)
        out = np.empty(self.frame_count, np.float32) if download else None
        _lib.call("gg_stack_compute_weights", self._handle, modes[mode], _lib.ptr(p), ctypes.c_float(eps),
                  _lib.ptr(out))
        return out

    def integrate_async(self, weights: Any | None = None, rejection: int = _lib.GG_REJECT_WINSORIZED,
                        low_sigma: float = 3.0, high_sigma: float = 3.0, min_samples: int = 3,
                        max_reject_fraction: float = 0.5, count_map_dtype: str = "uint16",
                        linear_fit_iterations: int = 5) -> None:
        """Enqueues the integration; maps stay on the device (see download_maps).

        ``weights="device"`` uses the weights of the last compute_frame_weights
        without a host round trip.
        """
        if count_map_dtype not in {"float32", "uint16"}:
            raise ValueError("count_map_dtype must be float32 or uint16")
        params = _lib.IntegrateParams(
            int(rejection), float(low_sigma), float(high_sigma), int(min_samples), float(max_reject_fraction),
            _lib.GG_COUNT_U16 if count_map_dtype == "uint16" else _lib.GG_COUNT_F32, int(linear_fit_iterations),
        )
        if isinstance(weights, str):
            if weights != "device":
                raise ValueError("weights must be an array, None or 'device'")
            _lib.call("gg_stack_integrate_device_weights", self._handle, None, ctypes.byref(params))
        else:
            w = self._weights(weights)
            _lib.call("gg_stack_integrate", self._handle, _lib.ptr(w), ctypes.byref(params))
        self._last_count_dtype = np.dtype(np.uint16 if count_map_dtype == "uint16" else np.float32)

    def download_maps(self, download_mode: str = "full", include_dq: bool = True, out: tuple | None = None):
        """(master, weight, coverage, low, high, dq) of the last integration.

        ``out`` may supply the six destination arrays (e.g. reused pinned
        buffers from host_pinned_empty_f32); entries the mode does not
        download may be None.
        """
        if download_mode not in _DOWNLOAD_MODES:
            raise ValueError("download_mode must be full, master_weight, or master_only")
        if self._last_count_dtype is None:
            raise RuntimeError("no integration has been run")
        info = self._info()
        shape = (info.height, info.width)
        full = download_mode == "full"
        want = (True, download_mode != "master_only", full, full, full, full and include_dq)
        dtypes = (np.float32, np.float32, self._last_count_dtype, self._last_count_dtype, self._last_count_dtype,
                  np.int16)
        bufs = []
        for k in range(6):
            if not want[k]:
                bufs.append(None)
                continue
            given = None if out is None else out[k]
            if given is None:
                bufs.append(np.empty(shape, dtypes[k]))
                continue
            if (not isinstance(given, np.ndarray) or given.shape != shape or given.dtype != np.dtype(dtypes[k])
                    or not given.flags.c_contiguous or not given.flags.writeable):
                raise ValueError(f"out[{k}] must be a writable C-contiguous {np.dtype(dtypes[k])} array of shape "
                                 f"{shape}")
            bufs.append(given)
        master, weight, cov, low, high, dq = bufs
        _lib.call("gg_stack_download_maps", self._handle, _lib.ptr(master), _lib.ptr(weight), _lib.ptr(cov),
                  _lib.ptr(low), _lib.ptr(high), _lib.ptr(dq))
        return master, weight, cov, low, high, dq

    def integrate_mean(self, weights: Any | None = None) -> tuple[np.ndarray, np.ndarray]:
        """Weighted mean (cpu/integration.py:106-118; reference kernel integration_kernels.cu:1610)."""
        self.integrate_async(weights, _lib.GG_REJECT_NONE, count_map_dtype="float32")
        master, weight, *_ = self.download_maps("master_weight")
        return master, weight

    def integrate_sigma_clip(self, weights: Any | None = None, low_sigma: float = 3.0, high_sigma: float = 3.0,
                             winsorize: bool = True, download_mode: str = "full"):
        """integrate_sigma_clip (native_bindings.cpp:13227) with the CPU semantics.

        winsorize=False is the CPU "sigma_clip" (median centre, std scale);
        winsorize=True is the CPU "winsorized_sigma" estimator.
        """
        if low_sigma <= 0.0 or high_sigma <= 0.0:
            raise ValueError("sigma thresholds must be positive")
        if download_mode not in _DOWNLOAD_MODES:
            raise ValueError("download_mode must be full, master_weight, or master_only")
        mode = _lib.GG_REJECT_WINSORIZED if winsorize else _lib.GG_REJECT_SIGMA_CLIP
        self.integrate_async(weights, mode, low_sigma, high_sigma, count_map_dtype="float32")
        master, weight, cov, low, high, _ = self.download_maps(download_mode, include_dq=False)
        return master, weight, cov, low, high

    # ---- fused warp + integration (glass_cuda.py:5142-5287) ----------------------
    def _integrate_warped(self, matrices, weights, interpolation, clamping_threshold, rejection, low_sigma,
                          high_sigma) -> dict[str, Any]:
        if interpolation not in {"bilinear", "lanczos3"}:
            raise ValueError("fused matrix-warped interpolation must be bilinear or lanczos3")
        mats = np.ascontiguousarray(np.asarray(matrices, dtype=np.float32).astype(np.float64))
        if mats.shape != (self.frame_count, 3, 3):
            raise ValueError("matrices must have shape (frame_count, 3, 3)")
        w = self._weights(weights)
        params = _lib.IntegrateParams(int(rejection), float(low_sigma), float(high_sigma), 3, 0.5, _lib.GG_COUNT_F32,
                                      5)
        interp = _lib.GG_INTERP_BILINEAR if interpolation == "bilinear" else _lib.GG_INTERP_LANCZOS3
        start = perf_counter()
        _lib.call("gg_stack_integrate_warped", self._handle, _lib.ptr(mats), interp,
                  ctypes.c_float(float(clamping_threshold)), _lib.ptr(w), ctypes.byref(params))
        self._last_count_dtype = np.dtype(np.float32)
        return {"schema_version": 1, "interpolation": interpolation, "clamping_threshold": float(clamping_threshold),
                "frame_count": self.frame_count, "enqueue_s": perf_counter() - start, "avoids_stack_scatter": True,
                "modifies_resident_stack": False}

    def fused_geometric_coverage(self) -> np.ndarray:
        out = np.empty((self.height, self.width), np.float32)
        _lib.call("gg_stack_download_fused_coverage", self._handle, _lib.ptr(out))
        return out

    def _tile_local(self, mode: int, target_mask, tile_extents, tile_multipliers, weights, low_sigma, high_sigma):
        tm = np.ascontiguousarray(np.asarray(target_mask).astype(np.uint8).reshape(-1))
        if tm.shape != (self.frame_count,):
            raise ValueError("target_mask must have shape (frame_count,)")
        ext = np.ascontiguousarray(np.asarray(tile_extents, dtype=np.int32))
        if ext.ndim != 2 or ext.shape[1] != 4:
            raise ValueError("tile_extents must have shape (tile_count, 4)")
        mult = np.ascontiguousarray(np.asarray(tile_multipliers, dtype=np.float32).reshape(-1))
        if mult.shape != (ext.shape[0],):
            raise ValueError("tile_multipliers must have shape (tile_count,)")
        w = self._weights(weights)
        start = perf_counter()
        _lib.call("gg_stack_integrate_tile_local", self._handle, int(mode), _lib.ptr(w), _lib.ptr(tm), _lib.ptr(ext),
                  _lib.ptr(mult), int(ext.shape[0]), ctypes.c_float(low_sigma), ctypes.c_float(high_sigma))
        self._last_count_dtype = np.dtype(np.float32)
        maps = self.download_maps("full" if mode else "master_weight", include_dq=False)
        timing = {"schema_version": 1, "tile_count": int(ext.shape[0]), "target_frame_count": int(tm.sum()),
                  "total_s": perf_counter() - start, "timing_model": "gb300_tile_local_column_in_shared_memory"}
        return maps, timing

    def integrate_tile_local_mean(self, target_mask: Any, tile_extents: Any, tile_multipliers: Any,
                                  weights: Any | None = None):
        """Weighted mean with per-tile multipliers on the target frames'
        weights -> (master, weight_map, timing)."""
        maps, timing = self._tile_local(0, target_mask, tile_extents, tile_multipliers, weights, 3.0, 3.0)
        return maps[0], maps[1], timing

    def integrate_tile_local_sigma_clip(self, target_mask: Any, tile_extents: Any, tile_multipliers: Any,
                                        weights: Any | None = None, low_sigma: float = 3.0, high_sigma: float = 3.0,
                                        winsorize: bool = True):
        """Sigma clip (winsorized when winsorize) with per-tile multipliers ->
        (master, weight, coverage, low, high, timing), float32 maps."""
        if low_sigma <= 0.0 or high_sigma <= 0.0:
            raise ValueError("sigma thresholds must be positive")
        maps, timing = self._tile_local(2 if winsorize else 1, target_mask, tile_extents, tile_multipliers, weights,
                                        low_sigma, high_sigma)
        return maps[0], maps[1], maps[2], maps[3], maps[4], timing

    def integrate_warped_device_weights(self, matrices: Any, interpolation: str = "lanczos3",
                                        clamping_threshold: float = -1.0,
                                        rejection: int = _lib.GG_REJECT_WINSORIZED, low_sigma: float = 3.0,
                                        high_sigma: float = 3.0, min_samples: int = 3,
                                        max_reject_fraction: float = 0.5, count_map_dtype: str = "uint16") -> None:
        """Fused warp + rejection + integration with the weights of the last
        compute_frame_weights (device, no host round trip); asynchronous."""
        interps = {"bilinear": _lib.GG_INTERP_BILINEAR, "lanczos3": _lib.GG_INTERP_LANCZOS3}
        if interpolation not in interps:
            raise ValueError("interpolation must be bilinear or lanczos3")
        if count_map_dtype not in {"float32", "uint16"}:
            raise ValueError("count_map_dtype must be float32 or uint16")
        mats = self._matrices(matrices, self.frame_count)
        params = _lib.IntegrateParams(int(rejection), float(low_sigma), float(high_sigma), int(min_samples),
                                      float(max_reject_fraction),
                                      _lib.GG_COUNT_U16 if count_map_dtype == "uint16" else _lib.GG_COUNT_F32, 5)
        _lib.call("gg_stack_integrate_warped_device_weights", self._handle, _lib.ptr(mats), interps[interpolation],
                  ctypes.c_float(clamping_threshold), ctypes.byref(params))
        self._last_count_dtype = np.dtype(np.uint16 if count_map_dtype == "uint16" else np.float32)

    # ---- CUDA graph of the resident step (no reference counterpart) ----------------
    def capture_step_graph(self, dev_raw_ptr: int, matrices: Any, calib_params: Any,
                           interpolation: str = "lanczos3", clamping_threshold: float = -1.0,
                           weighting: str = "simple_snr", rejection: int = _lib.GG_REJECT_WINSORIZED,
                           low_sigma: float = 3.0, high_sigma: float = 3.0, min_samples: int = 3,
                           max_reject_fraction: float = 0.5, count_map_dtype: str = "uint16") -> int:
        """Captures calibrate (uint16 frames at dev_raw_ptr) -> weights ->
        fused warp + rejection + integration into a CUDA graph owned by the
        stack; returns the number of kernels it replays."""
        interps = {"bilinear": _lib.GG_INTERP_BILINEAR, "lanczos3": _lib.GG_INTERP_LANCZOS3}
        if interpolation not in interps:
            raise ValueError("interpolation must be bilinear or lanczos3")
        modes = {"unit": 0, "simple_snr": 1}
        if weighting not in modes:
            raise ValueError("weighting must be unit or simple_snr")
        if count_map_dtype not in {"float32", "uint16"}:
            raise ValueError("count_map_dtype must be float32 or uint16")
        mats = self._matrices(matrices, self.frame_count)
        params = _lib.IntegrateParams(int(rejection), float(low_sigma), float(high_sigma), int(min_samples),
                                      float(max_reject_fraction),
                                      _lib.GG_COUNT_U16 if count_map_dtype == "uint16" else _lib.GG_COUNT_F32, 5)
        _lib.call("gg_stack_graph_capture_step", self._handle, ctypes.c_void_p(int(dev_raw_ptr)), _lib.ptr(mats),
                  interps[interpolation], ctypes.c_float(clamping_threshold), modes[weighting],
                  ctypes.byref(calib_params), ctypes.byref(params))
        self._last_count_dtype = np.dtype(np.uint16 if count_map_dtype == "uint16" else np.float32)
        return self.step_graph_kernels

    @property
    def step_graph_kernels(self) -> int:
        count = ctypes.c_int()
        _lib.call("gg_stack_graph_kernel_count", self._handle, ctypes.byref(count))
        return int(count.value)

    def launch_step_graph(self) -> None:
        """Replays the captured step on the stack's stream (asynchronous)."""
        _lib.call("gg_stack_graph_launch", self._handle)

    def destroy_step_graph(self) -> None:
        _lib.call("gg_stack_graph_destroy", self._handle)

    def integrate_matrix_warped_mean(self, matrices: Any, weights: Any | None = None, interpolation: str = "bilinear",
                                     clamping_threshold: float = -1.0, download_mode: str = "full"):
        """Fused warp + weighted mean -> (master, weight, coverage, geometric
        coverage, timing); the resident frames are not modified."""
        if download_mode not in _DOWNLOAD_MODES:
            raise ValueError("download_mode must be full, master_weight, or master_only")
        timing = self._integrate_warped(matrices, weights, interpolation, clamping_threshold, _lib.GG_REJECT_NONE,
                                        3.0, 3.0)
        master, weight, cov, _low, _high, _dq = self.download_maps(download_mode, include_dq=False)
        geo = self.fused_geometric_coverage() if download_mode == "full" else None
        timing.update(rejection="none", download_mode=download_mode)
        return master, weight, cov, geo, timing

    def integrate_matrix_warped_sigma_clip(self, matrices: Any, weights: Any | None = None,
                                           interpolation: str = "bilinear", clamping_threshold: float = -1.0,
                                           low_sigma: float = 3.0, high_sigma: float = 3.0, winsorize: bool = True,
                                           download_mode: str = "full"):
        """Fused warp + sigma clip (winsorized when winsorize) -> (master,
        weight, coverage, low, high, geometric coverage, timing)."""
        if low_sigma <= 0.0 or high_sigma <= 0.0:
            raise ValueError("sigma thresholds must be positive")
        if download_mode not in _DOWNLOAD_MODES:
            raise ValueError("download_mode must be full, master_weight, or master_only")
        mode = _lib.GG_REJECT_WINSORIZED if winsorize else _lib.GG_REJECT_SIGMA_CLIP
        timing = self._integrate_warped(matrices, weights, interpolation, clamping_threshold, mode, low_sigma,
                                        high_sigma)
        master, weight, cov, low, high, _dq = self.download_maps(download_mode, include_dq=False)
        geo = self.fused_geometric_coverage() if download_mode == "full" else None
        timing.update(rejection="winsorized_sigma" if winsorize else "sigma_clip", winsorize=bool(winsorize),
                      low_sigma=float(low_sigma), high_sigma=float(high_sigma), download_mode=download_mode)
        return master, weight, cov, low, high, geo, timing

    def integrate_hardened_winsorized_sigma(self, weights: Any | None = None, low_sigma: float = 3.0,
                                            high_sigma: float = 3.0, min_samples: int = 3,
                                            max_reject_fraction: float = 0.5, count_map_dtype: str = "float32",
                                            profile: bool = False, download_mode: str = "full"):
        """native_bindings.cpp:13395 (integration_kernels.cu:2292) with CPU parity."""
        if low_sigma <= 0.0 or high_sigma <= 0.0:
            raise ValueError("sigma thresholds must be positive")
        if int(min_samples) < 1:
            raise ValueError("min_samples must be at least 1")
        if not 0.0 <= float(max_reject_fraction) <= 1.0:
            raise ValueError("max_reject_fraction must be between 0 and 1")
        if download_mode not in _DOWNLOAD_MODES:
            raise ValueError("download_mode must be full, master_weight, or master_only")
        start = perf_counter()
        self.integrate_async(weights, _lib.GG_REJECT_WINSORIZED, low_sigma, high_sigma, min_samples,
                             max_reject_fraction, count_map_dtype)
        enqueue = perf_counter()
        master, weight, cov, low, high, _ = self.download_maps(download_mode, include_dq=False)
        done = perf_counter()
        if profile:
            info = {"native_kernel_frame_capacity": 64 if self.frame_count <= 64 else 512,
                    "native_kernel_capacity_selector": "register_column" if self.frame_count <= 64
                    else "shared_memory_column",
                    "enqueue_s": enqueue - start, "sync_download_s": done - enqueue}
            return master, weight, cov, low, high, info
        return master, weight, cov, low, high

    def integrate_linear_fit_clip(self, weights: Any | None = None, low_sigma: float = 3.0,
                                  high_sigma: float = 3.0, min_samples: int = 3,
                                  max_reject_fraction: float = 0.5, iterations: int = 5,
                                  count_map_dtype: str = "float32", download_mode: str = "full"):
        """Linear-fit clipping (no counterpart in the reference)."""
        if low_sigma <= 0.0 or high_sigma <= 0.0:
            raise ValueError("sigma thresholds must be positive")
        self.integrate_async(weights, _lib.GG_REJECT_LINEAR_FIT, low_sigma, high_sigma, min_samples,
                             max_reject_fraction, count_map_dtype, iterations)
        master, weight, cov, low, high, _ = self.download_maps(download_mode, include_dq=False)
        return master, weight, cov, low, high

    def dq_map(self) -> np.ndarray:
        """DQ int16 map fused into the last integration (resident_cuda.py:3110-3297 rules)."""
        return self.download_maps("full", include_dq=True)[5]
