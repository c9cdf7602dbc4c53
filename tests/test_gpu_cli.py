"""The command-line renderer (rle-based-voxel-raycasting_gb300/render_frames.py):
JSON-lines metrics for single frames and batches, and PNG output."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CLI = ROOT / "rle-based-voxel-raycasting_gb300" / "render_frames.py"
SMALL = ["--size", "256", "--height", "256", "--width", "320", "--screen-height", "240"]


def _run(args):
    r = subprocess.run([sys.executable, str(CLI), *SMALL, *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_json_lines_per_frame(torch_cuda):
    lines = [json.loads(ln) for ln in _run(["--frames", "3", "--json"]).splitlines()]
    assert [d["index"] for d in lines] == [0, 1, 2]
    for d in lines:
        assert d["frames"] == 1 and d["pixels"] == 320 * 240 and d["samples_per_ray"] == 512
        assert d["ms"] > 0 and d["mrays_per_s"] > 0 and d["column_rays"] > 0


def test_json_lines_per_batch(torch_cuda):
    lines = [json.loads(ln) for ln in _run(["--frames", "5", "--batch", "2", "--batch-lanes", "16", "--json"])
             .splitlines()]
    assert [d["frames"] for d in lines] == [2, 2, 1]
    assert all(d["pixels"] == 320 * 240 * d["frames"] and d["mrays_per_s"] > 0 for d in lines)


def test_png_frames(torch_cuda, tmp_path):
    _run(["--frames", "2", "--png-dir", str(tmp_path)])
    pngs = sorted(tmp_path.glob("frame_*.png"))
    assert [p.name for p in pngs] == ["frame_0000.png", "frame_0001.png"]
    for p in pngs:
        data = p.read_bytes()
        assert data[:8] == b"\x89PNG\r\n\x1a\n"
        assert int.from_bytes(data[16:20], "big") == 320 and int.from_bytes(data[20:24], "big") == 240
