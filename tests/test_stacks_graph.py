"""Several uneven stacks in one CUDA graph (gg_stacks_graph_capture): each
stack's calibrate -> weights -> warp -> rejection + integration recorded once
and replayed.  The replayed maps must equal, bit for bit, the same sequence
run eagerly stack by stack through the public entry points, for a bilinear
winsorized stack of 40 frames, a Lanczos3 winsorized stack of 70 frames and a
linear-fit stack of 25 frames (the three kinds of the batched-stacks
workload), on two replays in a row."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from glass_gb300 import _lib

pytestmark = pytest.mark.gpu


def _raw(rng, n, h, w):
    base = rng.normal(1000.0, 25.0, (h, w))
    frames = np.stack([base + rng.normal(0.0, 8.0, (h, w)) for _ in range(n)])
    frames[rng.random(frames.shape) < 0.002] += 20000.0
    return np.clip(np.rint(frames), 0, 65535).astype(np.uint16)


def _matrices(rng, n):
    mats = np.tile(np.eye(3), (n, 1, 1))
    for k in range(1, n):
        t = np.deg2rad(rng.uniform(-0.3, 0.3))
        mats[k] = [[np.cos(t), -np.sin(t), rng.uniform(-3, 3)], [np.sin(t), np.cos(t), rng.uniform(-3, 3)], [0, 0, 1]]
    return mats


SPECS = [  # frames, height, width, interpolation, rejection
    (40, 96, 128, "bilinear", _lib.GG_REJECT_WINSORIZED),
    (70, 80, 64, "lanczos3", _lib.GG_REJECT_WINSORIZED),
    (25, 64, 64, "lanczos3", _lib.GG_REJECT_LINEAR_FIT),
]


def _eager(native, stream, raw_dev, mats, spec):
    n, h, w, interp, rejection = spec
    s = native.ResidentCalibratedStack(n, h, w)
    s.set_stream(stream.cuda_stream)
    idx = np.arange(n, dtype=np.int64)
    params = _lib.CalibParams(1, 1.0, 1.0e-6, 0.0)
    _lib.call("gg_stack_calibrate_u16_device", s.handle, _lib.ptr(idx), ctypes.c_int64(n),
              ctypes.c_void_p(raw_dev.data_ptr()), 0, ctypes.byref(params))
    s.compute_frame_weights("simple_snr", None, 1.0e-6, download=False)
    moving = np.arange(1, n, dtype=np.int64)
    code = _lib.GG_INTERP_LANCZOS3 if interp == "lanczos3" else _lib.GG_INTERP_BILINEAR
    s.warp_frames_async(moving, mats[1:], code, np.nan, -1.0, False)
    s.integrate_async("device", rejection, 3.0, 3.0, 3, 0.5, "uint16")
    maps = s.download_maps("full", include_dq=True)
    s.close()
    return maps


def test_stacks_graph_replay_equals_eager_sequence(native):
    rng = np.random.default_rng(44)
    stream = torch.cuda.Stream()
    raws = [torch.from_numpy(_raw(rng, n, h, w).view(np.int16)).cuda() for n, h, w, _, _ in SPECS]
    mats = [_matrices(rng, spec[0]) for spec in SPECS]
    torch.cuda.synchronize()
    expected = [_eager(native, stream, raws[k], mats[k], SPECS[k]) for k in range(len(SPECS))]
    stacks = [native.ResidentCalibratedStack(n, h, w) for n, h, w, _, _ in SPECS]
    try:
        for s in stacks:
            s.set_stream(stream.cuda_stream)
        steps = [{"stack": stacks[k], "dev_raw": raws[k].data_ptr(), "matrices": mats[k],
                  "interpolation": SPECS[k][3], "rejection": SPECS[k][4]} for k in range(len(SPECS))]
        graph = native.StacksGraph(steps, stream.cuda_stream)
        try:
            assert graph.kernel_count > 3 * len(SPECS)
            for _ in range(2):
                graph.launch()
                stream.synchronize()
                for k, s in enumerate(stacks):
                    got = s.download_maps("full", include_dq=True)
                    for g, e in zip(got, expected[k]):
                        np.testing.assert_array_equal(g, e, err_msg=f"stack {k}")
        finally:
            graph.close()
    finally:
        for s in stacks:
            s.close()


def test_stacks_graph_rejects_bad_steps(native):
    s = native.ResidentCalibratedStack(3, 16, 16)
    raw = torch.zeros((3, 16, 16), dtype=torch.int16, device="cuda")
    try:
        with pytest.raises(ValueError):
            native.StacksGraph([{"stack": s, "dev_raw": raw.data_ptr(), "matrices": np.tile(np.eye(3), (2, 1, 1))}])
        with pytest.raises(ValueError):
            native.StacksGraph([{"stack": s, "dev_raw": raw.data_ptr(), "matrices": np.tile(np.eye(3), (3, 1, 1)),
                                 "interpolation": "nearest"}])
        with pytest.raises(ValueError):
            native.StacksGraph([{"stack": s, "dev_raw": raw.data_ptr(), "matrices": np.tile(np.eye(3), (3, 1, 1))},
                                {"stack": s, "dev_raw": raw.data_ptr(), "matrices": np.tile(np.eye(3), (3, 1, 1))}])
    finally:
        s.close()
