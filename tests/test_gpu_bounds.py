"""The range-checked debug build (build.py --bounds-check):

- on valid scenes no check fires and the ray buffers still equal the
  oracle's (plain frames, ray buffers with hit records, a batch);
- on a resident scene corrupted on purpose (every level-0 column pointed
  past the level's words; the reads stay inside the build's 64 KB zero
  padding either way) the colour-word check fires and the frame completes.
The regular build reports the mode as unsupported.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "rle-based-voxel-raycasting_gb300"

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked_lib(rle, torch_cuda):
    sys.path.insert(0, str(PKG))
    import build as b
    return b.build(checked=True)


def _probe(lib, mode):
    env = dict(os.environ, RLE_GB300_LIB=str(lib))
    r = subprocess.run([sys.executable, str(ROOT / "tests" / "bounds_probe.py"), mode], capture_output=True,
                       text=True, timeout=600, env=env, cwd=str(ROOT))
    assert r.returncode == 0, r.stdout + r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("RESULT ")][-1]
    _, flags, first = line.split()
    return int(flags), int(first)


def test_checked_build_is_silent_on_valid_scenes(checked_lib):
    flags, _ = _probe(checked_lib, "clean")
    assert flags == 0


def test_checked_build_catches_a_corrupted_scene(checked_lib):
    flags, first = _probe(checked_lib, "corrupt")
    assert flags & 4, flags  # colour word past the level's words
    assert first > 0


def test_regular_build_reports_unsupported(rle, torch_cuda):
    with pytest.raises(rle.RLEError) as e:
        rle.bounds_check_read(0)
    assert e.value.name == "RLE_ERR_UNSUPPORTED"
