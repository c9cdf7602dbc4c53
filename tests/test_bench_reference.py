"""The benchmark's reference arm (`bench.py --impl reference`): the
reference's algorithm (the oracle port of Render::render_line and the
resolve) on the host cores, on the same workload as the GPU arm.  It needs no
GPU, so its JSON line is checked here: the keys the benchmark contract asks
for, a CPU baseline describing the run, and an end-to-end entry with no
host-device copies."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["steps"] == 1 and line["warmup"] == 3
    assert line["unit"] == "Mrays/s" and line["higher_is_better"] is True and line["value"] > 0
    assert line["config"]["workload"].startswith("config 2: 2048x2048x256")
    assert line["config"]["samples_per_ray"] == 2048
    # the GPU arm prints the same workload description (bench.bench_config), key for key
    assert set(line["config"]) == {"workload", "samples_per_ray", "column_rays_per_frame", "runs_per_column", "l2",
                                   "parallelism"}
    assert 5.0 < line["config"]["runs_per_column"] < 12.0 and line["config"]["column_rays_per_frame"] > 1000
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
