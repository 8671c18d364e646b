"""The benchmark's reference arm (`bench.py --impl reference`) runs on the host alone: its JSON
line carries the fields the benchmark contract asks of it (the oracle timed on all host threads,
no host-device bytes), on a small scan."""

from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2", "--warmup", "1",
                          "--points", "48"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "trajectories/s" and line["higher_is_better"] is True
    assert line["value"] > 0.0 and line["steps"] == 2 and line["warmup"] == 1
    assert line["config"]["points"] == 48 and line["config"]["workload"] == "q1_16state_gaussian_scan_48pt_tsit5"
    cpu = line["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "trajectories/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # the time per step is the time of the 48-point scan it ran
    assert abs(line["ms_per_step"] - 1e3 * 48 / line["value"]) <= 1e-6 * line["ms_per_step"]
