"""Raw FITS read queue (the reference's RawFitsReadQueue): host threads
only, so the CPU tests exercise it fully; the GPU test feeds its output to the
big-endian decode + calibration and checks the frames against the oracle."""

from __future__ import annotations

import numpy as np
import pytest

from oracle.calibration import calibrate_light, decode_fits_u16be, encode_fits_u16be


def _write_fits_like(path, values: np.ndarray) -> int:
    """A FITS-shaped file: one 2880-byte header block, then the big-endian
    BZERO-shifted uint16 data unit.  Returns the data offset."""
    header = b"SIMPLE  =                    T".ljust(80) + b"END".ljust(80)
    header = header.ljust(2880, b" ")
    path.write_bytes(header + encode_fits_u16be(values).tobytes())
    return 2880


def _queue():
    from glass_gb300._glass_cuda_native import RawFitsReadQueue

    return RawFitsReadQueue(3)


def test_queue_reads_ranges(tmp_path):
    rng = np.random.default_rng(1)
    frames = [rng.integers(0, 65535, (37, 53), dtype=np.uint16) for _ in range(6)]
    q = _queue()
    outs = []
    try:
        for k, f in enumerate(frames):
            p = tmp_path / f"light_{k}.fits"
            off = _write_fits_like(p, f)
            out = np.empty(f.size * 2, np.uint8)
            outs.append(out)
            info = q.submit(k, str(p), off, out.size, out)
            assert info["frame_index"] == k
        seen = set()
        for _ in frames:
            done = q.wait_completed(10.0)
            assert done is not None and done["bytes_read"] == frames[done["frame_index"]].size * 2
            seen.add(done["frame_index"])
        assert seen == set(range(6))
        for k, f in enumerate(frames):
            np.testing.assert_array_equal(decode_fits_u16be(outs[k], f.shape), f)
        st = q.stats()
        assert st["submitted_count"] == 6 and st["completed_count"] == 6 and st["worker_count"] == 3
        assert q.wait_completed(0.01) is None  # nothing pending: time-out
    finally:
        q.close()
    assert q.stats()["closed"]


def test_queue_errors(tmp_path):
    q = _queue()
    try:
        out = np.empty(100, np.uint8)
        with pytest.raises(ValueError):
            q.submit(0, str(tmp_path / "x"), 0, 0, out)
        with pytest.raises(ValueError):
            q.submit(0, str(tmp_path / "x"), 0, 50, out)
        q.submit(1, str(tmp_path / "missing.fits"), 0, 100, out)
        with pytest.raises(RuntimeError, match="missing.fits"):
            q.wait_completed(10.0)
        short = tmp_path / "short.fits"
        short.write_bytes(b"\0" * 40)
        q.submit(2, str(short), 0, 100, out)
        with pytest.raises(RuntimeError, match="ended"):
            q.wait_completed(10.0)
    finally:
        q.close()
    with pytest.raises(RuntimeError, match="closed"):
        q.submit(3, str(tmp_path / "x"), 0, 100, np.empty(100, np.uint8))


@pytest.mark.gpu
def test_queue_feeds_calibration(native, tmp_path):
    rng = np.random.default_rng(2)
    n, h, w = 4, 64, 80
    lights = rng.integers(900, 1400, (n, h, w), dtype=np.uint16)
    bias = rng.normal(500, 3, (h, w)).astype(np.float32)
    dark = rng.normal(20, 1, (h, w)).astype(np.float32)
    flat = rng.uniform(0.9, 1.1, (h, w)).astype(np.float32)
    q = native.RawFitsReadQueue(2)
    raw = native.host_pinned_empty_u8(n * h * w * 2)
    try:
        for k in range(n):
            p = tmp_path / f"l{k}.fits"
            off = _write_fits_like(p, lights[k])
            q.submit(k, str(p), off, h * w * 2, raw[k * h * w * 2:(k + 1) * h * w * 2])
        for _ in range(n):
            assert q.wait_completed(10.0) is not None
    finally:
        q.close()
    s = native.ResidentCalibratedStack(n, h, w)
    try:
        s.set_calibration_masters(bias, dark, flat)
        fb = h * w * 2
        s.calibrate_frames_fits_u16be_bzero_host_async_multistream_callback_release_timed(
            list(range(n)), [raw[k * fb:(k + 1) * fb] for k in range(n)], [1.0] * n, [1.0] * n, 2, 2, None,
            {"master_dark_includes_bias": False})
        got = np.stack([s.download_frame(k) for k in range(n)])
    finally:
        s.close()
    for k in range(n):
        exp = calibrate_light(lights[k], bias, dark, flat, 1.0, 1.0, master_dark_includes_bias=False)
        np.testing.assert_array_equal(got[k], exp)
