"""Generates the golden fixtures in this folder from the reference itself.

    python tests/golden/make_golden.py

Needs oracle/_ref/libref.so, the reference's own sources compiled for the
host by oracle/ref/Makefile (only possible where the reference checkout is
present).  Writes golden_v1.npz:

  scene_rle4       .rle4 bytes of a 64x64x64 scene, 4 levels, encoded by the
                   reference's RLE4::compress with Tree::get_mipmap mips
                   (normal-derived colour words, as the reference writes them)
  table_<m>        the reference RLE4::load column table of level m
  cam_<i>          pos[3], rot[3] of camera i
  raymap_<i>       the reference's RayMap_GPU bytes for camera i (LP64)
  raybuf_<i>       the reference's Render::render_line output for all rays of
                   camera i into a zeroed buffer (rays x S words)
  params           S, maxres, border, mip_distance, z_far

The scene volume and cameras are seeded, so re-running reproduces the file.
"""
from __future__ import annotations

import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import pyoracle as po  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden_v1.npz"
N = 64
S = 128
MAXRES = 128
BORDER = 0.125
MIP_DISTANCE = 48
Z_FAR = 1500


def volume(seed: int) -> np.ndarray:
    """[z, y, x] boolean volume: a rolling heightfield (column index 0 at the
    top, as the renderer's column axis points down), tunnels and a floating
    slab, so runs, skips, overhangs and empty columns all occur."""
    rng = np.random.default_rng(seed)
    x = np.arange(N)[None, :]
    z = np.arange(N)[:, None]
    h = 22 + 9 * np.sin(x * 2 * np.pi / N * 2 + 0.7) * np.cos(z * 2 * np.pi / N) + rng.integers(0, 3, (N, N))
    j = np.arange(N)[None, :, None]
    vol = j >= (N - h[:, None, :])  # solid below the surface
    tunnels = rng.random((N // 4, N // 4, N // 4)) < 0.15
    tunnels = tunnels.repeat(4, 0).repeat(4, 1).repeat(4, 2)
    vol &= ~(tunnels & (j < N - 3))
    vol[10:20, 8:12, 30:50] = True   # a floating slab
    vol[:, :, 5] = False             # an empty row of columns
    return vol


def main() -> int:
    if not po.ref_available():
        print("oracle/_ref/libref.so missing: build it with make -C oracle/ref", file=sys.stderr)
        return 1
    vol = volume(11)
    bits = [po.pack_bits(vol)]
    dims = [(N, N, N)]
    for _ in range(3):
        sx, sy, sz = dims[-1]
        bits.append(po.ref_mipmap(bits[-1], sx, sy, sz))
        dims.append((sx // 2, sy // 2, sz // 2))
    levels = []
    for m in range(4):
        _, words = po.ref_compress(bits[m], *dims[m], m)
        levels.append((*dims[m], words))
    data = po.write_rle4(levels)
    out = {"scene_rle4": np.frombuffer(data, np.uint8)}
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "golden.rle4"
        path.write_bytes(data)
        for m in range(4):
            out[f"table_{m}"] = po.ref_load_table(str(path), m, dims[m][0], dims[m][2])
    scene = po.OracleScene(levels)
    rng = np.random.default_rng(5)
    cams = []
    for i in range(6):
        pos = (float(rng.uniform(0, N)), float(-rng.uniform(N - 50, N - 30)), float(rng.uniform(0, N)))
        rot = (float([0.35, -0.3, 1.1, -1.2, 0.6, 1.45][i]), float(rng.uniform(0, 2 * np.pi)), 0.0)
        cams.append((pos, rot))
    for i, (pos, rot) in enumerate(cams):
        rb = po.ref_raymap(pos, rot, BORDER, MAXRES)
        f = po.ref_raymap_fields(rb)
        nrays = min(f["map_line_count"], 4 * MAXRES)
        buf = po.ref_render_rays(rb, scene, S, nrays, MIP_DISTANCE, Z_FAR)
        out[f"cam_{i}"] = np.array([*pos, *rot], np.float32)
        out[f"raymap_{i}"] = np.frombuffer(rb, np.uint8)
        out[f"raybuf_{i}"] = buf
    out["params"] = np.array([S, MAXRES, MIP_DISTANCE, Z_FAR], np.int64)
    out["border"] = np.array([BORDER], np.float32)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
