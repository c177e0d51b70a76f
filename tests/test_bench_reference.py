"""The reference arm of bench.py (`--impl reference`): the oracle port of the
reference's CPU path on the host cores, no CUDA.  Its one JSON line carries
the same metric, unit and direction as the GPU arm, "impl": "reference", a
cpu_baseline that describes this run (its value is the line's) and an e2e
record with no host-device traffic.  Run on the c2 sample (32 frames of
384 x 384), one step, a few seconds of CPU work.
"""

from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    proc = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", "c2", "--steps", "1",
                           "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [ln for ln in proc.stdout.splitlines() if ln.strip()]
    line = json.loads(lines[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "stacked Mpix-frames/s" and line["unit"] == "Mpix-frames/s"
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 0
    assert line["value"] > 0.0 and line["ms_per_step"] > 0.0
    assert line["config"]["workload"].startswith("c2:32x2048x2048")
    cpu = line["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["sample"]
    assert cpu["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
