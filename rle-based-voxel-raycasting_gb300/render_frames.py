"""Render frames of a seeded scene from the command line.

    python rle-based-voxel-raycasting_gb300/render_frames.py [--size 2048] [--height 256] [--seed 2]
        [--width 1920] [--screen-height 1080] [--frames 6] [--fov 90] [--png-dir DIR] [--batch N] [--json]

Builds the scene on the GPU (rle_scenegen_device), walks a seeded camera
path (poses 10-80 voxels above the ground, yaw uniform, pitch up to 30
degrees) and renders each frame with rle_render_frame, printing the time per
frame; with --png-dir it also writes every frame as a PNG; with --json it
prints one JSON object per line instead (frame or batch index, frames,
milliseconds, screen pixels, Mrays/s, column rays, samples per ray).  This is the
headless counterpart of the reference's interactive viewer
(src/main.cpp:446-669): the frame ends in device buffers, not in a window.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import struct
import sys
import time
import zlib
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent


def _package():
    if "rle_gb300" in sys.modules:
        return sys.modules["rle_gb300"]
    spec = importlib.util.spec_from_file_location("rle_gb300", PKG / "__init__.py",
                                                  submodule_search_locations=[str(PKG)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["rle_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def write_png(path: Path, rgb: np.ndarray) -> None:
    """8-bit RGB image (h x w x 3) as a PNG (zlib-compressed scanlines)."""
    h, w, _ = rgb.shape
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    path.write_bytes(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)) +
                     chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def _metrics(index: int, frames: int, ms: float, pixels: int, rays: int, samples: int) -> dict:
    return {"index": index, "frames": frames, "ms": round(ms, 4), "pixels": pixels,
            "mrays_per_s": round(pixels / ms / 1e3, 1) if ms > 0 else None, "column_rays": rays,
            "samples_per_ray": samples}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--size", type=int, default=2048, help="scene columns along x and z (power of two)")
    ap.add_argument("--height", type=int, default=256, help="scene height in voxels (multiple of 64)")
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--no-caves", action="store_true")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--screen-height", type=int, default=1080)
    ap.add_argument("--fov", type=float, default=90.0)
    ap.add_argument("--samples", type=int, default=0,
                    help="samples per column ray (default: the smallest power of two >= width)")
    ap.add_argument("--frames", type=int, default=6)
    ap.add_argument("--path-seed", type=int, default=20261203)
    ap.add_argument("--png-dir", type=str, default=None)
    ap.add_argument("--batch", type=int, default=0,
                    help="render the path in batches of this many frames (rle_batch, autotuned) instead")
    ap.add_argument("--batch-lanes", type=int, default=0,
                    help="with --batch: skip the autotuner, one-ray claims with this many lanes per ray")
    ap.add_argument("--json", action="store_true", help="one JSON object per frame (or batch) on stdout")
    args = ap.parse_args(argv)

    import torch

    rle = _package()
    if not torch.cuda.is_available():
        print("render_frames: no CUDA device", file=sys.stderr)
        return 2
    p = rle.scenegen_default(args.size, args.height, args.size, args.seed, caves=not args.no_caves)
    scene = rle.Scene.generate_on_device(p)
    info = scene.info()
    table, words = scene.copy_level(0)
    rng = np.random.default_rng(args.path_seed)
    W, H = args.width, args.screen_height
    samples = args.samples
    if samples <= 0:
        samples = 1
        while samples < W:
            samples <<= 1
    view = rle.view_params(W, H, samples=samples)
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    colour = torch.empty(W * H, dtype=torch.int32, device="cuda")
    depth = torch.empty(W * H, dtype=torch.float32, device="cuda")
    out_dir = Path(args.png_dir) if args.png_dir else None
    if out_dir:
        out_dir.mkdir(parents=True, exist_ok=True)
    if args.batch > 0:
        return _batched(rle, torch, scene, info, table, words, rng, view, args)
    for i in range(args.frames):
        x, z = rng.uniform(0, info.sx[0]), rng.uniform(0, info.sz[0])
        g = rle.ground_height(table, words, info.sx[0], info.sy[0], int(x), int(z))
        pitch = float(rng.uniform(1.0, 30.0) * rng.choice([-1.0, 1.0]))
        cam = rle.camera(float(x), float(z), g + float(rng.uniform(10, 80)), float(rng.uniform(0, 360)), pitch,
                         args.fov, scene_height=info.sy[0])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rle.render_frame(scene, cam, view, ws, ws_bytes, colour, depth)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if args.json:
            rm = rle.raymap_build(cam, view)
            print(json.dumps(_metrics(i, 1, ms, W * H, rm.rays, rm.samples)), flush=True)
        else:
            print(f"frame {i}: {ms:.3f} ms", flush=True)
        if out_dir:
            rgba = colour.cpu().numpy().view(np.uint8).reshape(H, W, 4)
            write_png(out_dir / f"frame_{i:04d}.png", np.ascontiguousarray(rgba[:, :, :3]))
    scene.free()
    return 0


def _batched(rle, torch, scene, info, table, words, rng, view, args) -> int:
    W, H = view.width, view.height
    cams = []
    for _ in range(args.frames):
        x, z = rng.uniform(0, info.sx[0]), rng.uniform(0, info.sz[0])
        g = rle.ground_height(table, words, info.sx[0], info.sy[0], int(x), int(z))
        pitch = float(rng.uniform(1.0, 30.0) * rng.choice([-1.0, 1.0]))
        cams.append(rle.camera(float(x), float(z), g + float(rng.uniform(10, 80)), float(rng.uniform(0, 360)),
                               pitch, args.fov, scene_height=info.sy[0]))
    outs = [(torch.empty(W * H, dtype=torch.int32, device="cuda"), torch.empty(W * H, dtype=torch.float32,
                                                                                device="cuda"))
            for _ in range(args.batch)]
    groups = [[rle.frame_request(c, view, *outs[k]) for k, c in enumerate(cams[i:i + args.batch])]
              for i in range(0, len(cams), args.batch)]
    b = rle.Batch(args.batch, max(rle.batch_words_needed(g) for g in groups), view.samples)
    if args.batch_lanes:
        b.set_tuning(1, args.batch_lanes, 1, 128)
    else:
        best, ms = b.autotune(scene, groups[0], repeats=1)
        msg = (f"autotuned: tile {best.tile_rays} lanes {best.lanes_per_ray} staging {best.staging} "
               f"per_frame {best.per_frame} ({ms:.3f} ms)")
        print(msg, file=sys.stderr if args.json else sys.stdout, flush=True)
    for i, g in enumerate(groups):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.render(scene, g)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if args.json:
            rays = sum(rle.raymap_build(r.cam, r.view).rays for r in g)
            print(json.dumps(_metrics(i, len(g), ms, W * H * len(g), rays, view.samples)), flush=True)
        else:
            print(f"batch {i}: {len(g)} frames, {ms:.3f} ms", flush=True)
    b.free()
    scene.free()
    return 0


if __name__ == "__main__":
    sys.exit(main())
