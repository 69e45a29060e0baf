"""The benchmark's reference arm (`bench.py --impl reference`) on the CPU: it
times the FP32 OpenMP transcription of the reference's FP on the host cores
and prints one JSON line with the keys the benchmark contract names (the
metric and unit of the GPU arm, `impl`, `cpu_baseline`, `e2e`).  CPU only;
the GPU arm needs a device and runs on the GPU machines."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    res = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                         timeout=600, cwd=REPO)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "Grays/s"
    # (the benchmark raises a warm-up below 3 to 3)
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] >= 3
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == bench.WORKLOAD
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1
    assert cb["bp_gpix_views_per_s"] > 0 and cb["fbp_ms_per_slice"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": "Grays/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
