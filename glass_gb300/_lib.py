"""ctypes binding of libglass_gb300.so (the C ABI in include/glass_gb300.h).

This module only loads the library and declares its prototypes; the
reference-facing Python surface lives in ``_glass_cuda_native``.  Loading
fails loudly: there is no CPU fallback behind these names.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PACKAGE_DIR = Path(__file__).resolve().parent
LIBRARY_PATH = PACKAGE_DIR / "libglass_gb300.so"

GG_OK = 0
GG_ERR_INVALID_ARGUMENT = -1
GG_ERR_OUT_OF_RANGE = -2
GG_ERR_RUNTIME = -3
GG_ERR_CUDA = -4
GG_ERR_NO_DEVICE = -5
GG_ERR_OUT_OF_MEMORY = -6
GG_ERR_TIMEOUT = -7

GG_REJECT_NONE = 0
GG_REJECT_SIGMA_CLIP = 1
GG_REJECT_WINSORIZED = 2
GG_REJECT_LINEAR_FIT = 3

GG_COUNT_F32 = 0
GG_COUNT_U16 = 1

GG_INTERP_NEAREST = 0
GG_INTERP_BILINEAR = 1
GG_INTERP_LANCZOS3 = 3

c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_int16_p = ctypes.POINTER(ctypes.c_int16)


class DeviceInfo(ctypes.Structure):
    _fields_ = [
        ("name", ctypes.c_char * 256),
        ("major", ctypes.c_int),
        ("minor", ctypes.c_int),
        ("multiprocessor_count", ctypes.c_int),
        ("total_global_mem", ctypes.c_int64),
        ("l2_cache_bytes", ctypes.c_int64),
        ("shared_mem_per_block_optin", ctypes.c_int64),
    ]


class CalibParams(ctypes.Structure):
    _fields_ = [
        ("master_dark_includes_bias", ctypes.c_int),
        ("dark_scale", ctypes.c_float),
        ("flat_floor", ctypes.c_float),
        ("pedestal", ctypes.c_float),
    ]


class StackInfo(ctypes.Structure):
    _fields_ = [
        ("frame_count", ctypes.c_int64),
        ("height", ctypes.c_int64),
        ("width", ctypes.c_int64),
        ("pixels_per_frame", ctypes.c_int64),
        ("frame_stride", ctypes.c_int64),
        ("slot_count", ctypes.c_int64),
        ("loaded_count", ctypes.c_int64),
        ("bytes_allocated", ctypes.c_int64),
        ("warp_scratch_bytes", ctypes.c_int64),
        ("host_pinned_bytes", ctypes.c_int64),
        ("calibration_lane_count", ctypes.c_int64),
        ("warp_coverage_frame_count", ctypes.c_int64),
        ("has_bias", ctypes.c_int),
        ("has_dark", ctypes.c_int),
        ("has_flat", ctypes.c_int),
    ]


class FrameStats(ctypes.Structure):
    _fields_ = [
        ("mean", ctypes.c_double),
        ("std", ctypes.c_double),
        ("valid_pixels", ctypes.c_int64),
        ("total_pixels", ctypes.c_int64),
    ]


class StarParams(ctypes.Structure):
    _fields_ = [
        ("threshold_sigma", ctypes.c_float),
        ("max_stars", ctypes.c_int),
        ("window_radius", ctypes.c_int),
        ("min_separation_px", ctypes.c_float),
        ("background", ctypes.c_float),
        ("noise", ctypes.c_float),
        ("catalog_min_fwhm", ctypes.c_float),
        ("catalog_max_eccentricity", ctypes.c_float),
        ("mesh_cell", ctypes.c_int32),
    ]


class GridCatalogParams(ctypes.Structure):
    _fields_ = [
        ("threshold", ctypes.c_float),
        ("grid_cols", ctypes.c_int32),
        ("grid_rows", ctypes.c_int32),
        ("candidates_per_cell", ctypes.c_int32),
        ("max_output_candidates", ctypes.c_int32),
        ("min_separation_px", ctypes.c_float),
        ("centroid_radius", ctypes.c_int32),
        ("centroid_background", ctypes.c_int32),
    ]


class Star(ctypes.Structure):
    _fields_ = [
        ("x", ctypes.c_double),
        ("y", ctypes.c_double),
        ("flux", ctypes.c_double),
        ("peak", ctypes.c_double),
        ("fwhm", ctypes.c_double),
        ("eccentricity", ctypes.c_double),
        ("snr", ctypes.c_double),
        ("sharpness", ctypes.c_double),
        ("npix", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


STAR_DTYPE = np.dtype([("x", "f8"), ("y", "f8"), ("flux", "f8"), ("peak", "f8"), ("fwhm", "f8"),
                       ("eccentricity", "f8"), ("snr", "f8"), ("sharpness", "f8"), ("npix", "i4"), ("pad", "i4")])


class StarFrameInfo(ctypes.Structure):
    _fields_ = [
        ("median", ctypes.c_float),
        ("mad", ctypes.c_float),
        ("noise", ctypes.c_double),
        ("threshold", ctypes.c_double),
        ("candidates", ctypes.c_int64),
        ("valid_pixels", ctypes.c_int64),
    ]


class IntegrateParams(ctypes.Structure):
    _fields_ = [
        ("rejection", ctypes.c_int),
        ("low_sigma", ctypes.c_float),
        ("high_sigma", ctypes.c_float),
        ("min_samples", ctypes.c_int),
        ("max_reject_fraction", ctypes.c_float),
        ("count_dtype", ctypes.c_int),
        ("linear_fit_iterations", ctypes.c_int),
    ]


class StackStep(ctypes.Structure):
    _fields_ = [
        ("stack", ctypes.c_void_p),
        ("dev_raw", ctypes.c_void_p),
        ("host_matrices", ctypes.c_void_p),
        ("interpolation", ctypes.c_int32),
        ("clamping_threshold", ctypes.c_float),
        ("weighting", ctypes.c_int32),
        ("calib", CalibParams),
        ("integrate", IntegrateParams),
    ]


GG_TRANSFORM_TRANSLATION = 0
GG_TRANSFORM_SIMILARITY = 1
GG_TRANSFORM_AFFINE = 2


class RegisterParams(ctypes.Structure):
    _fields_ = [
        ("transform_model", ctypes.c_int32),
        ("min_inliers", ctypes.c_int32),
        ("tolerance_px", ctypes.c_double),
        ("descriptor_radius", ctypes.c_double),
        ("max_stars", ctypes.c_int32),
        ("neighbors", ctypes.c_int32),
        ("max_descriptors", ctypes.c_int32),
        ("max_candidates", ctypes.c_int32),
    ]


class Registration(ctypes.Structure):
    _fields_ = [
        ("matrix", ctypes.c_double * 9),
        ("rms_px", ctypes.c_double),
        ("best_candidate", ctypes.c_int64),
        ("inliers", ctypes.c_int32),
        ("status", ctypes.c_int32),
        ("descriptors_reference", ctypes.c_int32),
        ("descriptors_moving", ctypes.c_int32),
        ("matches", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


class AlignmentMetrics(ctypes.Structure):
    _fields_ = [
        ("valid_pixels", ctypes.c_int64),
        ("sampled_pixels", ctypes.c_int64),
        ("sample_stride", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("rms", ctypes.c_double),
        ("mean_abs_diff", ctypes.c_double),
        ("ncc", ctypes.c_double),
    ]


class RefineParams(ctypes.Structure):
    _fields_ = [
        ("search_radius_px", ctypes.c_double),
        ("coarse_step_px", ctypes.c_double),
        ("fine_radius_px", ctypes.c_double),
        ("fine_step_px", ctypes.c_double),
        ("coarse_sample_stride", ctypes.c_int32),
        ("final_sample_stride", ctypes.c_int32),
    ]


class RefineResult(ctypes.Structure):
    _fields_ = [
        ("matrix", ctypes.c_double * 9),
        ("dx_correction", ctypes.c_double),
        ("dy_correction", ctypes.c_double),
        ("metrics", AlignmentMetrics),
        ("coarse_candidates", ctypes.c_int32),
        ("fine_candidates", ctypes.c_int32),
    ]


class TranslationNcc(ctypes.Structure):
    _fields_ = [
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("score", ctypes.c_double),
        ("candidate_count", ctypes.c_int64),
    ]


class ReadCompletion(ctypes.Structure):
    _fields_ = [
        ("frame_index", ctypes.c_uint64),
        ("bytes_read", ctypes.c_uint64),
        ("file_open_s", ctypes.c_double),
        ("file_read_s", ctypes.c_double),
        ("total_s", ctypes.c_double),
    ]


class ReadQueueStats(ctypes.Structure):
    _fields_ = [
        ("worker_count", ctypes.c_uint64),
        ("submitted_count", ctypes.c_uint64),
        ("completed_count", ctypes.c_uint64),
        ("queued_count", ctypes.c_uint64),
        ("active_count", ctypes.c_uint64),
        ("ready_count", ctypes.c_uint64),
        ("requested_bytes", ctypes.c_uint64),
        ("closed", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


class CosmeticParams(ctypes.Structure):
    _fields_ = [
        ("hot_sigma", ctypes.c_float),
        ("cold_sigma", ctypes.c_float),
        ("structure_sigma", ctypes.c_float),
        ("min_neighbor_support", ctypes.c_int32),
        ("star_protection", ctypes.c_int32),
        ("star_threshold_sigma", ctypes.c_float),
        ("star_protection_radius_px", ctypes.c_float),
        ("star_min_pixels", ctypes.c_int32),
        ("star_max_sharpness", ctypes.c_float),
        ("apply", ctypes.c_int32),
    ]


class CosmeticResult(ctypes.Structure):
    _fields_ = [
        ("hot_pixels", ctypes.c_int64),
        ("cold_pixels", ctypes.c_int64),
        ("candidate_hot_pixels", ctypes.c_int64),
        ("candidate_cold_pixels", ctypes.c_int64),
        ("star_protected_hot_pixels", ctypes.c_int64),
        ("star_protected_cold_pixels", ctypes.c_int64),
        ("median", ctypes.c_double),
        ("sigma", ctypes.c_double),
        ("star_count", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


class GradientRefineParams(ctypes.Structure):
    _fields_ = [
        ("transform_model", ctypes.c_int32),
        ("interpolation", ctypes.c_int32),
        ("sample_stride", ctypes.c_int32),
        ("row_stride", ctypes.c_int32),
        ("stats_passes", ctypes.c_int32),
        ("iterations", ctypes.c_int32),
        ("min_samples", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("clip_sigma", ctypes.c_float),
        ("mask_shift_px", ctypes.c_float),
        ("tolerance_px", ctypes.c_double),
        ("max_step_px", ctypes.c_double),
    ]


class GradientRefineResult(ctypes.Structure):
    _fields_ = [
        ("matrix", ctypes.c_double * 9),
        ("alpha", ctypes.c_double),
        ("beta", ctypes.c_double),
        ("sigma", ctypes.c_double),
        ("rms", ctypes.c_double),
        ("last_step_px", ctypes.c_double),
        ("samples", ctypes.c_int64),
        ("iterations", ctypes.c_int32),
        ("status", ctypes.c_int32),
    ]


class StackDevicePtrs(ctypes.Structure):
    _fields_ = [
        ("slots", ctypes.c_void_p),
        ("slot_of_frame", ctypes.c_void_p),
        ("master", ctypes.c_void_p),
        ("weight", ctypes.c_void_p),
        ("coverage", ctypes.c_void_p),
        ("low", ctypes.c_void_p),
        ("high", ctypes.c_void_p),
        ("dq", ctypes.c_void_p),
        ("warp_coverage", ctypes.c_void_p),
    ]


# name -> (argtypes); every function returns int status.
_P = ctypes.c_void_p
PROTOTYPES: dict[str, list] = {
    "gg_version": [ctypes.POINTER(ctypes.c_int)],
    "gg_last_error": [ctypes.c_char_p, ctypes.c_size_t],
    "gg_kernel_launches": [c_int64_p],
    "gg_cuda_available": [ctypes.POINTER(ctypes.c_int)],
    "gg_device_count": [ctypes.POINTER(ctypes.c_int)],
    "gg_device_info": [ctypes.c_int, ctypes.POINTER(DeviceInfo)],
    "gg_host_alloc_pinned": [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)],
    "gg_host_free_pinned": [_P],
    "gg_calibrate_tile_f32": [_P, _P, _P, _P, ctypes.c_int64, ctypes.POINTER(CalibParams), _P],
    "gg_stack_create": [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)],
    "gg_stack_destroy": [_P],
    "gg_stack_info": [_P, ctypes.POINTER(StackInfo)],
    "gg_stack_set_stream": [_P, _P],
    "gg_stack_synchronize": [_P],
    "gg_stack_set_masters": [_P, _P, _P, _P],
    "gg_stack_upload_frame": [_P, ctypes.c_int64, _P],
    "gg_stack_download_frame_tile": [_P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                     ctypes.c_int64, _P],
    "gg_stack_download_frames_tile": [_P, _P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                      ctypes.c_int64, _P],
    "gg_stack_calibrate_u16": [_P, _P, ctypes.c_int64, _P, ctypes.c_int, ctypes.POINTER(CalibParams)],
    "gg_stack_calibrate_u16_device": [_P, _P, ctypes.c_int64, _P, ctypes.c_int, ctypes.POINTER(CalibParams)],
    "gg_stack_upload_raw_u16": [_P, _P, ctypes.c_int64, _P],
    "gg_stack_calibrate_u16_staged": [_P, _P, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(CalibParams)],
    "gg_stack_calibrate_f32": [_P, ctypes.c_int64, _P, ctypes.POINTER(CalibParams)],
    "gg_stack_frame_stats": [_P, _P, ctypes.c_int64, _P],
    "gg_stack_compute_weights": [_P, ctypes.c_int, _P, ctypes.c_float, _P],
    "gg_frames_stats_f32_noalloc": [_P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _P, _P],
    "gg_stack_integrate": [_P, _P, ctypes.POINTER(IntegrateParams)],
    "gg_stack_integrate_device_weights": [_P, _P, ctypes.POINTER(IntegrateParams)],
    "gg_stack_download_maps": [_P, _P, _P, _P, _P, _P, _P],
    "gg_stack_integrate_warped": [_P, _P, ctypes.c_int, ctypes.c_float, _P, ctypes.POINTER(IntegrateParams)],
    "gg_stack_download_fused_coverage": [_P, _P],
    "gg_stack_graph_capture_step": [_P, _P, _P, ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                    ctypes.POINTER(CalibParams), ctypes.POINTER(IntegrateParams)],
    "gg_stacks_integrate_batch": [_P, ctypes.c_int32, ctypes.POINTER(IntegrateParams)],
    "gg_read_queue_create": [ctypes.c_int32, _P],
    "gg_read_queue_submit": [_P, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_uint64, _P, _P],
    "gg_read_queue_wait": [_P, ctypes.c_double, ctypes.POINTER(ReadCompletion), ctypes.POINTER(ctypes.c_int32)],
    "gg_read_queue_stats": [_P, ctypes.POINTER(ReadQueueStats)],
    "gg_read_queue_close": [_P],
    "gg_read_queue_destroy": [_P],
    "gg_stack_cosmetic_mask": [_P, _P, ctypes.c_int64, ctypes.POINTER(CosmeticParams), _P],
    "gg_stack_apply_invalid_mask": [_P, ctypes.c_int64, _P, _P],
    "gg_stack_cosmetic_threshold": [_P, _P, ctypes.c_int64, _P, _P, ctypes.c_int32, _P],
    "gg_stack_integrate_tile_local": [_P, ctypes.c_int, _P, _P, _P, _P, ctypes.c_int32, ctypes.c_float,
                                      ctypes.c_float],
    "gg_stack_integrate_warped_device_weights": [_P, _P, ctypes.c_int, ctypes.c_float,
                                                 ctypes.POINTER(IntegrateParams)],
    "gg_stack_graph_launch": [_P],
    "gg_stack_pair_grid_stats": [_P, ctypes.c_int64, _P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, _P, _P, _P,
                                 _P, _P],
    "gg_stack_apply_grid_normalization": [_P, _P, ctypes.c_int64, _P, _P, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_int32, ctypes.c_int32],
    "gg_stack_local_normalize_grid": [_P, ctypes.c_int64, _P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_double, ctypes.c_int, _P, _P],
    "gg_stack_apply_global_normalization": [_P, ctypes.c_int64, ctypes.c_float, ctypes.c_float],
    "gg_autotune_set_enabled": [ctypes.c_int],
    "gg_autotune_clear": [],
    "gg_autotune_count": [ctypes.POINTER(ctypes.c_int32)],
    "gg_autotune_entry": [ctypes.c_int32, ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t,
                          ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_float),
                          ctypes.POINTER(ctypes.c_int32)],
    "gg_stack_graph_kernel_count": [_P, ctypes.POINTER(ctypes.c_int)],
    "gg_stack_graph_destroy": [_P],
    "gg_stacks_graph_capture": [_P, ctypes.c_int32, _P, _P],
    "gg_stacks_graph_launch": [_P],
    "gg_stacks_graph_kernel_count": [_P, _P],
    "gg_stacks_graph_destroy": [_P],
    "gg_stack_device_ptrs": [_P, ctypes.POINTER(StackDevicePtrs)],
    "gg_stack_frame_device_ptr": [_P, ctypes.c_int64, _P],
    "gg_stack_download_weights": [_P, _P],
    "gg_dq_map_i16": [_P, _P, _P, _P, _P, _P, ctypes.c_int64, ctypes.c_int64, _P],
    "gg_stack_detect_stars": [_P, _P, ctypes.c_int64, ctypes.POINTER(StarParams), _P, _P, _P],
    "gg_stack_star_grid_catalog": [_P, _P, ctypes.c_int64, ctypes.POINTER(GridCatalogParams), _P, _P, _P],
    "gg_triangle_descriptors": [_P, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P, _P, _P,
                                ctypes.c_int64, c_int64_p],
    "gg_register_star_lists": [_P, ctypes.c_int64, _P, ctypes.c_int64, ctypes.POINTER(RegisterParams),
                               ctypes.POINTER(Registration), _P],
    "gg_similarity_from_descriptors": [_P, ctypes.c_int64, _P, ctypes.c_int64, _P, _P, ctypes.c_int64, _P, _P,
                                       ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                       ctypes.POINTER(Registration), _P],
    "gg_stack_register_frames": [_P, ctypes.c_int64, _P, ctypes.c_int64, ctypes.POINTER(RegisterParams), _P],
    "gg_stack_alignment_metrics": [_P, ctypes.c_int64, _P, ctypes.c_int64, _P, ctypes.c_int32, _P],
    "gg_stack_refine_translation": [_P, ctypes.c_int64, _P, ctypes.c_int64, _P, ctypes.POINTER(RefineParams), _P],
    "gg_stack_translation_ncc": [_P, ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_int32, ctypes.c_double, ctypes.c_int32, ctypes.POINTER(TranslationNcc)],
    "gg_stack_warp_frames": [_P, _P, ctypes.c_int64, _P, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_int],
    "gg_stack_reset_warp_coverage": [_P],
    "gg_stack_accumulate_full_warp_coverage_frame": [_P],
    "gg_stack_download_warp_coverage": [_P, _P],
    "gg_stack_tma_enabled": [_P, ctypes.POINTER(ctypes.c_int)],
    "gg_warp_matrix_f32": [_P, ctypes.c_int64, ctypes.c_int64, _P, ctypes.c_int, ctypes.c_float, ctypes.c_float, _P,
                           _P],
    "gg_warp_affine_f32_device": [_P, ctypes.c_int64, ctypes.c_int64, _P, ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                  _P, _P],
    "gg_warp_affine_backward_f32_device": [_P, ctypes.c_int64, ctypes.c_int64, _P, ctypes.c_int, _P, _P, _P, _P],
    "gg_stack_refine_gradient": [_P, ctypes.c_int64, _P, ctypes.c_int64, _P, ctypes.POINTER(GradientRefineParams),
                                 _P],
    "gg_stack_gradient_normal_equations": [_P, ctypes.c_int64, _P, ctypes.c_int64, _P, _P,
                                           ctypes.POINTER(GradientRefineParams), _P],
}

_LIB: ctypes.CDLL | None = None


class NativeLibraryError(ImportError):
    """The CUDA library is missing or incomplete; there is no fallback."""


def library_path() -> Path:
    override = os.environ.get("GLASS_GB300_LIBRARY")
    return Path(override) if override else LIBRARY_PATH


def load(required: bool = True) -> ctypes.CDLL | None:
    """Loads libglass_gb300.so and declares every prototype."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        if not required:
            return None
        raise NativeLibraryError(
            f"{path} is missing: build it with `python -m glass_gb300.build` (needs nvcc, sm_103a)"
        )
    lib = ctypes.CDLL(str(path))
    for name, argtypes in PROTOTYPES.items():
        try:
            fn = getattr(lib, name)
        except AttributeError as exc:  # pragma: no cover - only on a stale build
            raise NativeLibraryError(f"{path} does not export {name}; rebuild it") from exc
        fn.argtypes = argtypes
        fn.restype = ctypes.c_int
    _LIB = lib
    return lib


def last_error() -> str:
    lib = load()
    buf = ctypes.create_string_buffer(4096)
    lib.gg_last_error(buf, len(buf))
    return buf.value.decode("utf-8", "replace")


def check(status: int, what: str = "") -> None:
    """Raises the Python exception that the reference module would raise."""
    if status == GG_OK:
        return
    message = last_error() or f"status {status}"
    if what:
        message = f"{what}: {message}"
    if status == GG_ERR_INVALID_ARGUMENT:
        raise ValueError(message)
    if status == GG_ERR_OUT_OF_RANGE:
        raise IndexError(message)
    if status == GG_ERR_OUT_OF_MEMORY:
        raise MemoryError(message)
    raise RuntimeError(message)


def call(name: str, *args) -> None:
    lib = load()
    check(getattr(lib, name)(*args), name)


def kernel_launches() -> int:
    """Kernels this library has launched in this process."""
    count = ctypes.c_int64()
    call("gg_kernel_launches", ctypes.byref(count))
    return int(count.value)


def autotune_set_enabled(enabled: bool) -> None:
    call("gg_autotune_set_enabled", int(bool(enabled)))


def autotune_clear() -> None:
    call("gg_autotune_clear")


def autotune_entries() -> list[dict]:
    """The launch shapes the autotuner has chosen in this process."""
    count = ctypes.c_int32()
    call("gg_autotune_count", ctypes.byref(count))
    out = []
    for i in range(count.value):
        kernel, shape, choice = (ctypes.create_string_buffer(256) for _ in range(3))
        ms, cands = ctypes.c_float(), ctypes.c_int32()
        call("gg_autotune_entry", i, kernel, 256, shape, 256, choice, 256, ctypes.byref(ms), ctypes.byref(cands))
        out.append({"kernel": kernel.value.decode(), "shape": shape.value.decode(), "choice": choice.value.decode(),
                    "ms": float(ms.value), "candidates": int(cands.value)})
    return out


def ptr(array: np.ndarray | None) -> int | None:
    """Data pointer of a C-contiguous array (None passes NULL)."""
    if array is None:
        return None
    if not array.flags.c_contiguous:
        raise ValueError("array must be C-contiguous")
    return array.ctypes.data
