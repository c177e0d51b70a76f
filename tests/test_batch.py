"""Several uneven stacks integrated in one launch: each stack's maps must be
bit-identical to its own integration (same kernel body, same per-stack
frame table and weights; only the CTA assignment differs)."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(8, 96, 128), (13, 160, 100), (32, 64, 64)]


def _stack_data(rng, n, h, w):
    data = rng.normal(1000.0, 25.0, (n, h, w)).astype(np.float32)
    data[rng.integers(0, n, 40), rng.integers(0, h, 40), rng.integers(0, w, 40)] = np.float32(9.0e4)
    data[0, :3, :] = np.nan
    return data


@pytest.mark.parametrize("rejection", ["winsorized", "sigma_clip", "none"])
def test_batch_matches_single_stacks(native, rejection):
    from glass_gb300 import _lib

    mode = {"winsorized": _lib.GG_REJECT_WINSORIZED, "sigma_clip": _lib.GG_REJECT_SIGMA_CLIP,
            "none": _lib.GG_REJECT_NONE}[rejection]
    rng = np.random.default_rng(5)
    stacks, singles = [], []
    try:
        for n, h, w in SHAPES:
            s = native.ResidentCalibratedStack(n, h, w)
            stacks.append(s)
            for k, frame in enumerate(_stack_data(rng, n, h, w)):
                s.upload_calibrated_frame(k, frame)
            s.compute_frame_weights("simple_snr", None, 1.0e-6, download=False)
            s.integrate_async("device", mode, 3.0, 3.0, 3, 0.5, "uint16")
            singles.append(s.download_maps("full", include_dq=False))
        native.integrate_stacks_batch(stacks, mode, 3.0, 3.0, 3, 0.5, "uint16")
        for s, single in zip(stacks, singles):
            got = s.download_maps("full", include_dq=False)
            for k in range(5):
                np.testing.assert_array_equal(got[k], single[k], err_msg=f"{s.frame_count} frames, map {k}")
    finally:
        for s in stacks:
            s.close()


def test_batch_arguments(native):
    from glass_gb300 import _lib

    big = native.ResidentCalibratedStack(33, 16, 16)
    try:
        for k in range(33):
            big.upload_calibrated_frame(k, np.ones((16, 16), np.float32))
        params = _lib.IntegrateParams(_lib.GG_REJECT_NONE, 3.0, 3.0, 3, 0.5, _lib.GG_COUNT_U16, 5)
        handles = (ctypes.c_void_p * 1)(big.handle.value if hasattr(big.handle, "value") else big.handle)
        with pytest.raises(ValueError):
            _lib.call("gg_stacks_integrate_batch", handles, 1, ctypes.byref(params))
        handles2 = (ctypes.c_void_p * 2)(handles[0], handles[0])
        with pytest.raises(ValueError):
            _lib.call("gg_stacks_integrate_batch", handles2, 2, ctypes.byref(params))
    finally:
        big.close()
