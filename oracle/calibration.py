"""Oracle: light calibration and uint16 decoding.

Restates src/glass/cpu/calibration.py:51-76 (calibrate_light) with the
policy defaults of src/glass/models.py:67-81, and the FITS BITPIX=16 decode
of cpu/cuda/calibration_kernels.cu:126-130 (big-endian bytes, BZERO 32768).
"""

from __future__ import annotations

import numpy as np

_F32 = np.float32


def calibrate_light(light, bias=None, dark=None, flat=None, light_exposure_s=1.0, dark_exposure_s=None,
                    master_dark_includes_bias=True, dark_scaling_enabled=True, flat_floor=1.0e-6,
                    pedestal=0.0) -> np.ndarray:
    """cpu/calibration.py:51-76, float32 with one rounding per operation."""
    out = np.asarray(light).astype(_F32, copy=True)
    if dark is not None:
        scale = 1.0
        if dark_scaling_enabled and dark_exposure_s not in (None, 0):
            scale = float(light_exposure_s) / float(dark_exposure_s)
        out = out - np.asarray(dark).astype(_F32) * scale
        if not master_dark_includes_bias and bias is not None:
            out = out - np.asarray(bias).astype(_F32)
    elif bias is not None:
        out = out - np.asarray(bias).astype(_F32)
    if flat is not None:
        out = out / np.maximum(np.asarray(flat).astype(_F32), flat_floor)
    if pedestal:
        out = out + float(pedestal)
    return out.astype(_F32)


def decode_fits_u16be(raw_bytes: np.ndarray, shape) -> np.ndarray:
    """Big-endian int16 with BZERO 32768 -> unsigned value (calibration_kernels.cu:126-130)."""
    be = np.frombuffer(np.ascontiguousarray(raw_bytes).tobytes(), dtype=">u2").reshape(shape)
    return (be.astype(np.uint32) ^ 0x8000).astype(np.uint16)


def encode_fits_u16be(values: np.ndarray) -> np.ndarray:
    """Inverse of decode_fits_u16be: unsigned values -> FITS big-endian bytes."""
    v = (np.asarray(values, dtype=np.uint16).astype(np.uint32) ^ 0x8000).astype(">u2")
    return np.frombuffer(v.tobytes(), dtype=np.uint8).copy()
