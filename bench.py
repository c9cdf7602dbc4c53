"""Benchmark: primary rays per second of the plain per-frame render at 1080p.

Workload (one step = one frame through the public render call): the
2048 x 2048 x 256 cave scene (seed 2, fBm heightfield + 3D simplex caves,
4 mip levels, ~8 runs per column), a seeded camera path of 1920x1080 frames
at 90 degrees, positions uniform over the grid 10-80 voxels above the local
ground, yaw uniform in [0, 360), pitch uniform in [-30, 30] degrees
(|pitch| >= 1, a horizontal view puts the ray map's vanishing point at
infinity).  Primary rays = screen pixels; the column rays and ray-buffer
samples behind them are reported beside the metric.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is device-timed (CUDA events on the render
stream, L2 flushed between steps); `e2e` adds, per step, the camera from
host memory and the copy of the colour + depth result to pinned host memory.
`--impl reference` times the reference's CPU algorithm (the oracle port of
Render::render_line + the resolve, all host threads) on the same frames.
"""
from __future__ import annotations

import argparse
import atexit
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG_DIR = ROOT / "rle-based-voxel-raycasting_gb300"
METRIC = "primary Mrays/s @1080p (plain per-frame launch, 2048^2 cave scene)"
WORKLOAD = ("config 2: 2048x2048x256 cave scene seed 2, 1920x1080 frames, 90 deg FOV, "
            "poses 10-80 above ground, yaw U[0,360), pitch U[-30,30]")
W, H = 1920, 1080
SCENE = dict(n=2048, sy=256, seed=2, caves=True)


def load_rle():
    import importlib.util
    if "rle_gb300" in sys.modules:
        return sys.modules["rle_gb300"]
    spec = importlib.util.spec_from_file_location("rle_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["rle_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per raycast
# launch on this workload: the mean over the first five timed frames of the
# default run, captured with ncu (profiles/raycast_traffic_1080p_cave2048.md
# gives the command and the per-frame figures).  A profiler run cannot be part
# of the timed benchmark; the capture is repeated when the kernel changes.
RAYCAST_DRAM_BYTES_PER_LAUNCH = 33_878_784
RAYCAST_DRAM_FRAMES = "frames 0-4 of the timed camera path (seed 20261203, after 5 warm-up frames)"
# The end-to-end loop renders like a throughput-oriented renderer: several frames in flight (one
# stream, workspace and output set each) and 16 lanes per column ray (two rays per warp, twice the
# rays in flight per SM), which wins once frames overlap; isolated frames (`value`) keep 32.
# Measured on GB300, 60 frames: 32 lanes x 3 / 4 / 6 in flight -> 7891 / 8204 / 8225 Mrays/s;
# 16 lanes x 4 / 6 / 8 -> 7818 / 8790 / 8845.
E2E_FRAMES_IN_FLIGHT = 6
E2E_LANES_PER_RAY = 16


def bench_config(rays_per_frame, runs_per_column: float, world: int) -> dict:
    """The workload description both arms print (the GPU arm and
    `--impl reference`), key for key and value for value, so that their lines
    describe the same run: the same frames of the same scene, their mean
    column rays, the scene's runs per column, and how each arm treats the
    L2 and the ranks."""
    return {
        "workload": WORKLOAD,
        "samples_per_ray": pow2_ceil(W),
        "column_rays_per_frame": round(sum(rays_per_frame) / len(rays_per_frame), 1),
        "runs_per_column": round(runs_per_column, 2),
        "l2": "GPU arm: flushed before every step (256 MiB write); the host arm has no GPU cache to flush",
        "parallelism": f"replicas x{world}: every rank renders its own camera path; the host arm runs on rank 0's cores",
    }


def pow2_ceil(v: int) -> int:
    p = 1
    while p < v:
        p <<= 1
    return p


def frame_view(rle, w: int, h: int, **kw):
    """A frame of w x h pixels mapped onto the reference's geometry as the
    configs define it: maxres = w (RAYS_CASTED_RES = 4w), samples per column
    ray = the smallest power of two >= w (RENDER_SIZE), border (w-h)/(2w)."""
    return rle.view_params(w, h, samples=pow2_ceil(w), **kw)


def scene_bytes(rle):
    p = rle.scenegen_default(SCENE["n"], SCENE["sy"], SCENE["n"], SCENE["seed"], caves=SCENE["caves"])
    return rle.scenegen_rle4(p)


def poses(rle, level0, count, seed=20261203):
    """Seeded camera path; level0 = (sx, sy, sz, uint2 table as u32 pairs, words)."""
    sx, sy, sz, table, words = level0
    rng = np.random.default_rng(seed)
    cams = []
    for _ in range(count):
        x, z = rng.uniform(0, sx), rng.uniform(0, sz)
        g = rle.ground_height(table, words, sx, sy, int(x), int(z))
        pitch = float(rng.uniform(1.0, 30.0) * rng.choice([-1.0, 1.0]))
        cams.append(rle.camera(float(x), float(z), g + float(rng.uniform(10, 80)), float(rng.uniform(0, 360)),
                               pitch, 90.0, scene_height=sy))
    return cams


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            atexit.register(self.__exit__, None, None, None)  # never leave the sampler running
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def clock_summary(primary: ClockSampler, whole: ClockSampler) -> dict:
    """Median SM clock and throttle reasons over the whole GPU run, with the
    samples that fell inside the plain-frame timed region beside them."""
    a, b = primary.summary(), whole.summary()
    out = dict(b) if b["samples"] else dict(a)
    out["reasons"] = sorted(set(a["reasons"]) | set(b["reasons"]))
    out["window"] = "warm-up to the last config-5 frame, nvidia-smi every 200 ms"
    out["timed_region"] = a
    return out


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (ValueError, KeyError):
            pass
    return 6800.0, "fallback"


def replica_throughput(local_ms: float, local_units: float, dist=None, device: str = "cuda"):
    """Replicas (no exchange step): every rank renders its own frames.  The
    job's time is the slowest rank's, its work the sum over ranks; returns
    (mega-units per second, job milliseconds)."""
    ms, units = float(local_ms), float(local_units)
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        import torch
        t_max = torch.tensor([ms], dtype=torch.float64, device=device)
        t_sum = torch.tensor([units], dtype=torch.float64, device=device)
        dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
        dist.all_reduce(t_sum, op=dist.ReduceOp.SUM)
        ms, units = float(t_max.item()), float(t_sum.item())
    return units / (ms / 1e3) / 1e6, ms


def max_overlap(starts: np.ndarray, ends: np.ndarray) -> int:
    """Largest number of [start, end) intervals open at one time."""
    ev = np.concatenate([np.stack([starts, np.ones_like(starts)], 1), np.stack([ends, -np.ones_like(ends)], 1)])
    ev = ev[np.lexsort((ev[:, 1], ev[:, 0]))]  # ends before starts at equal times
    return int(np.cumsum(ev[:, 1]).max()) if len(ev) else 0


def critical_path(rle, torch, scene, rms, raybuf, raydepth, flush, stream, raycast_ms):
    """Per-ray times of the timed frames, taken outside the timed region with
    rle_render_rays_timed (the same production kernel plus two timestamps
    per ray).  Two lower bounds on a frame's raycast:
      critical_path_ms: its slowest column ray, end_clock - start_clock at
        the SM clock (read from the records: cycles / globaltimer ns of the
        rays longer than 50 us);
      work_bound_ms: the sum of all rays' times spread perfectly over every
        ray slot (SMs used x the most rays seen running at once on one SM).
    tail_frac = critical_path_ms / the raycast's time in the timed frames:
    near 1, the frame waits on its slowest ray, and only shortening that
    ray's own chain of work speeds it up."""
    sp = stream.cuda_stream
    size = rle.RAY_TIME_DTYPE.itemsize
    buf = torch.zeros(max(rm.rays for rm in rms) * size, dtype=torch.uint8, device="cuda")
    rows = []
    for k, rm in enumerate(rms):
        flush.zero_()
        with torch.cuda.stream(stream):
            rle.render_rays_timed(scene, rm, raybuf, raydepth, buf, stream=sp)
        torch.cuda.synchronize()
        t = buf[: rm.rays * size].cpu().numpy().view(rle.RAY_TIME_DTYPE)
        cyc = (t["end_clock"] - t["start_clock"]).astype(np.float64)
        ns = (t["end_ns"] - t["start_ns"]).astype(np.float64)
        long = ns > 50_000
        ghz = float(np.median(cyc[long] / ns[long])) if long.any() else float("nan")
        t0 = int(t["start_ns"].min())
        per_sm = [max_overlap(t["start_ns"][t["sm"] == m], t["end_ns"][t["sm"] == m]) for m in np.unique(t["sm"])]
        slots = len(per_sm) * max(per_sm)
        crit_ms = float(cyc.max() / ghz / 1e6) if ghz == ghz else float(ns.max() / 1e6)
        rows.append({
            "critical_path_ms": crit_ms,
            "work_bound_ms": float(ns.sum() / slots / 1e6),
            "span_ms": float((int(t["end_ns"].max()) - t0) / 1e6),
            "last_ray_start_ms": float((int(t["start_ns"].max()) - t0) / 1e6),
            "median_ray_ms": float(np.median(ns) / 1e6),
            "sm_ghz": ghz,
            "slots": slots,
            "kernel_ms": float(raycast_ms[k]),
        })
    mean = lambda key: float(np.mean([r[key] for r in rows]))  # noqa: E731
    worst = max(rows, key=lambda r: r["critical_path_ms"] / r["kernel_ms"])
    crit, kern = mean("critical_path_ms"), mean("kernel_ms")
    return {
        "critical_path_ms": round(crit, 4),
        "tail_frac": round(crit / kern, 3),
        "work_bound_ms": round(mean("work_bound_ms"), 4),
        "span_ms": round(mean("span_ms"), 4),
        "last_ray_start_ms": round(mean("last_ray_start_ms"), 4),
        "median_ray_ms": round(mean("median_ray_ms"), 4),
        "kernel_ms": round(kern, 4),
        "sm_clock_mhz_from_rays": round(mean("sm_ghz") * 1e3, 1),
        "ray_slots": int(np.median([r["slots"] for r in rows])),
        "frames": len(rows),
        "frame_tail_frac_min_max": [round(min(r["critical_path_ms"] / r["kernel_ms"] for r in rows), 3),
                                    round(worst["critical_path_ms"] / worst["kernel_ms"], 3)],
        "source": "rle_render_rays_timed on the timed frames, outside the timed region (L2 flushed before each); "
                  "critical_path_ms = slowest ray's SM cycles / SM clock, mean over frames; "
                  "tail_frac = critical_path_ms / kernel_ms",
    }


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_ours(args):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(args.backend, device_id=torch.device("cuda", local))
    rle = load_rle()
    data = scene_bytes(rle)
    scene = rle.Scene.from_bytes(data, device=local)
    info = scene.info()
    table, words = scene.copy_level(0)
    lv0 = (info.sx[0], info.sy[0], info.sz[0], table, words)
    cams = poses(rle, lv0, args.warmup + args.steps, seed=20261203 + rank)
    view = frame_view(rle, W, H)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    colour = torch.empty(W * H, dtype=torch.int32, device="cuda")
    depth = torch.empty(W * H, dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    rms = [rle.raymap_build(c, view) for c in cams]
    words = rle.raybuf_words(rms[0])
    raybuf = ws[: words * 4].view(torch.int32)
    raydepth = ws[((words * 4 + 255) // 256) * 256:][: words * 4].view(torch.float32)

    def step(i, marks=None):
        """One frame: the raycast (rle_render_rays, the drop-in for
        cuda_main_render2) and the resolve (rle_resolve) through the C ABI,
        the launches rle_render_frame makes; `marks` = three events around
        and between them."""
        rm = rms[i]
        if marks:
            marks[0].record(stream)
        rle.render_rays(scene, rm, raybuf, raydepth, None, None, stream=sp)
        if marks:
            marks[1].record(stream)
        rle.resolve(rm, raybuf, raydepth, colour, depth, stream=sp)
        if marks:
            marks[2].record(stream)

    # clocks over every GPU section of the run (warm-up to the config-5 frames):
    # the plain-frame region alone is shorter than nvidia-smi's sampling period
    clk_all = ClockSampler(local).__enter__()
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            flush.zero_()
            step(i)
    torch.cuda.synchronize()

    # ---- device-timed plain frames (value); the raycast's share of the same
    # frames from the event between its launch and the resolve's ----
    ev = [tuple(torch.cuda.Event(enable_timing=True) for _ in range(3)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                step(args.warmup + k, ev[k])
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    frame_ms = [a.elapsed_time(c) for a, _, c in ev]
    raycast_ms = [a.elapsed_time(b) for a, b, _ in ev]
    value, total_ms = replica_throughput(sum(frame_ms), W * H * args.steps, dist, device="cuda")

    # ---- outside the timed region, the same frames again: work counters
    # (algorithmic bytes) and per-ray times (critical path) ----
    algo_bytes = []
    cnt = torch.zeros(6, dtype=torch.int64, device="cuda")
    for k in range(args.steps):
        rm = rms[args.warmup + k]
        cnt.zero_()
        rle.render_rays(scene, rm, raybuf, raydepth, None, cnt, stream=sp)
        torch.cuda.synchronize()
        c = [int(v) for v in cnt.cpu()]
        # algorithmic bytes: 8 B per column-table entry, 2 B per run header
        # and per colour word read, 8 B (packed word + depth) per ray sample
        algo_bytes.append(8 * c[1] + 2 * c[2] + 2 * c[5] + 8 * rm.rays * rm.samples)
    critical = critical_path(rle, torch, scene, [rms[args.warmup + k] for k in range(args.steps)], raybuf, raydepth,
                             flush, stream, raycast_ms)
    k_ms = sum(raycast_ms) / len(raycast_ms)
    achieved = (sum(algo_bytes) / len(algo_bytes)) / (k_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()

    # ---- end to end: camera from host through the C ABI, colour + depth of
    # every frame back to pinned host memory; a multi-buffered frame loop:
    # frames rotate over E2E_FRAMES_IN_FLIGHT streams (own workspace and
    # outputs each), so a frame's read-back and its last rays overlap the
    # next frames' renders; the launch shape is set through rle_tuning_set ----
    sets = [(stream, ws, colour, depth)]
    for _ in range(E2E_FRAMES_IN_FLIGHT - 1):
        sets.append((torch.cuda.Stream(), torch.empty_like(ws), torch.empty_like(colour), torch.empty_like(depth)))
    hosts = [(torch.empty(W * H, dtype=torch.int32, pin_memory=True),
              torch.empty(W * H, dtype=torch.float32, pin_memory=True)) for _ in sets]
    rle.tuning_set(E2E_LANES_PER_RAY, 0, 0, 0)
    for i, (s_, w_, c_, d_) in enumerate(sets):  # warm-up: every stream, this launch shape
        with torch.cuda.stream(s_):
            rle.render_frame(scene, cams[i % args.warmup], view, w_, ws_bytes, c_, d_, None, stream=s_.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s_ in sets[1:]:
        s_[0].wait_event(e0)
    for k in range(args.steps):
        s_, w_, c_, d_ = sets[k % len(sets)]
        hc, hd = hosts[k % len(sets)]
        with torch.cuda.stream(s_):
            rle.render_frame(scene, cams[args.warmup + k], view, w_, ws_bytes, c_, d_, None, stream=s_.cuda_stream)
            hc.copy_(c_, non_blocking=True)
            hd.copy_(d_, non_blocking=True)
    for s_ in sets[1:]:
        ej = torch.cuda.Event()
        ej.record(s_[0])
        stream.wait_event(ej)
    e1.record(stream)
    torch.cuda.synchronize()
    rle.tuning_set(0, 0, 0, 0)
    e2e_ms = e0.elapsed_time(e1)
    e2e = W * H * args.steps / (e2e_ms / 1e3) / 1e6

    config1 = None
    if not args.no_config1:
        config1 = run_config1(rle, torch, flush, with_cpu=rank == 0 and world == 1 and not args.no_cpu_baseline)
    batched = None
    if not args.no_batch:
        batched = run_batched(rle, torch, scene, lv0)
    serving = None
    if args.serve_seconds > 0:
        serving = run_serving(rle, torch, seconds=args.serve_seconds)
    config5 = None
    if args.config5_frames > 0:
        config5 = run_config5(rle, torch, frames=args.config5_frames)
    clk_all.__exit__(None, None, None)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(rle, data, cams[args.warmup:args.warmup + max(1, min(args.cpu_frames, args.steps))])

    rays = [rms[args.warmup + k].rays for k in range(args.steps)]
    line = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "Mrays/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded scene and camera path)",
        "config": bench_config(rays, info.run_headers / (SCENE["n"] ** 2), world),
        "scene": {"device_bytes": int(info.device_bytes)},
        "e2e": {"value": round(e2e, 2), "unit": "Mrays/s", "h2d_bytes_per_step": 28,
                "d2h_bytes_per_step": W * H * 8,
                "pipeline": f"multi-buffered frame loop: frames rotate over {E2E_FRAMES_IN_FLIGHT} streams; a frame's read-back and last rays overlap the next frames' renders",
                "frames_in_flight": E2E_FRAMES_IN_FLIGHT, "lanes_per_ray": E2E_LANES_PER_RAY,
                "l2": "not flushed: the scene (294 MB) exceeds L2 and every frame has its own camera"},
        "gpu_launches": 2 * args.steps,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": RAYCAST_DRAM_BYTES_PER_LAUNCH,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, mean per launch over "
                                       + RAYCAST_DRAM_FRAMES + " (profiles/raycast_traffic_1080p_cave2048.md)",
                     "kernel": "raycast_kernel", "kernel_ms": round(k_ms, 4), "peak_kind": peak_kind,
                     "kernel_ms_source": "CUDA events between the raycast and the resolve launches of the timed "
                                         "frames themselves (mean over the steps)",
                     "limiter": "per-ray dependency chains, not DRAM: the slowest column ray of a frame bounds "
                                "its raycast from below (critical_path)",
                     "algorithmic_bytes_per_launch": int(sum(algo_bytes) / len(algo_bytes))},
        "critical_path": critical,
        "clocks": clock_summary(clk, clk_all),
        "wall_s_timed": round(t_wall, 3),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if config1:
        line["config1"] = config1
    if batched:
        line["batched_vs_plain"] = batched
    if serving:
        line["serving"] = serving
    if config5:
        line["config5_8192"] = config5
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))
    return 0


def run_config1(rle, torch, flush, reps=20, cpu_reps=5, with_cpu=True):
    """Config 1: the 512^2 x 256 fBm heightfield (seed 1, no caves), one
    640x480 view at 90 deg, 40 voxels above the terrain at the centre of the
    grid, yaw 30, pitch -15 (1024 samples per column ray, 640 rays per fan
    unit), rendered plain: GPU ms per frame (CUDA events, L2 flushed before
    each) and, beside it, the reference's algorithm on the host cores (the
    oracle port of the ray map, Render::render_line and the resolve, all
    threads)."""
    data = rle.scenegen_rle4(rle.scenegen_default(512, 256, 512, 1, caves=False))
    scene = rle.Scene.from_bytes(data)
    table, words = scene.copy_level(0)
    g = rle.ground_height(table, words, 512, 256, 256, 256)
    cam = rle.camera(256.0, 256.0, g + 40.0, 30.0, -15.0, 90.0, scene_height=256)
    view = frame_view(rle, 640, 480)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    col = torch.empty(640 * 480, dtype=torch.int32, device="cuda")
    dep = torch.empty(640 * 480, dtype=torch.float32, device="cuda")
    ms = []
    with torch.cuda.stream(stream):
        for r in range(reps + 3):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            rle.render_frame(scene, cam, view, ws, ws_bytes, col, dep, None, stream=sp)
            b.record(stream)
            b.synchronize()
            if r >= 3:
                ms.append(a.elapsed_time(b))
    gpu_ms = float(np.median(ms))
    rm = rle.raymap_build(cam, view)
    out = {"workload": "config 1: 512x512x256 fBm heightfield seed 1, one 640x480 view at 90 deg, 40 above the "
                       "terrain centre, yaw 30, pitch -15",
           "column_rays": rm.rays, "samples_per_ray": rm.samples,
           "gpu": {"ms_per_frame": round(gpu_ms, 4), "value": round(640 * 480 / gpu_ms / 1e3, 1), "unit": "Mrays/s",
                   "timing": f"CUDA events around rle_render_frame, L2 flushed, median of {reps}"}}
    scene.free()
    if with_cpu:
        sys.path.insert(0, str(ROOT))
        from oracle import pyoracle as po
        po.build_oracle()
        oscene = po.OracleScene.from_rle4(data)
        threads = os.cpu_count() or 1
        cms = []
        for _ in range(cpu_reps):
            t0 = time.perf_counter()
            om = po.raymap_build(list(cam.pos), list(cam.rot), rm.border, rm.maxres, rm.fov_scale, rm.samples,
                                 rm.mip_distance, rm.z_far)
            o, d, _, _ = po.render_rays(om, oscene, nthreads=threads)
            po.resolve(om, 640, 480, o, d)
            cms.append((time.perf_counter() - t0) * 1e3)
        cpu_ms = float(np.median(cms))
        out["cpu"] = {"ms_per_frame": round(cpu_ms, 3), "value": round(640 * 480 / cpu_ms / 1e3, 2),
                      "unit": "Mrays/s", "cores": threads, "kind": "port",
                      "timing": f"oracle port (ray map + raycast + resolve, OpenMP over column rays), median of "
                                f"{cpu_reps}"}
        out["gpu_over_cpu"] = round(cpu_ms / gpu_ms, 1)
    return out


BATCH_RES = [(320, 240), (640, 480), (1280, 720), (1920, 1080)]


def run_batched(rle, torch, scene, lv0, n_cams=64, repeats=5, seed=20261204):
    """Config 3: 64 cameras with resolutions drawn from BATCH_RES and poses
    as config 2, rendered (a) as 64 plain per-frame launches in sequence and
    (b) as one batched launch (tuning picked by the autotuner).  Both timed
    with CUDA events on one stream; primary rays = pixels of all 64 frames."""
    rng = np.random.default_rng(seed)
    cams = poses(rle, lv0, n_cams, seed=seed)
    views = [frame_view(rle, *BATCH_RES[int(rng.integers(0, len(BATCH_RES)))]) for _ in range(n_cams)]
    pixels = sum(v.width * v.height for v in views)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    outs = []
    reqs = []
    for c, v in zip(cams, views):
        col = torch.empty(v.width * v.height, dtype=torch.int32, device="cuda")
        dep = torch.empty(v.width * v.height, dtype=torch.float32, device="cuda")
        outs.append((col, dep))
        reqs.append(rle.frame_request(c, v, col, dep))
    ws_bytes = max(rle.frame_workspace_bytes(v) for v in views)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")

    def plain():
        for c, v, (col, dep) in zip(cams, views, outs):
            rle.render_frame(scene, c, v, ws, ws_bytes, col, dep, None, stream=sp)

    batch = rle.Batch(max_frames=n_cams, raybuf_words=rle.batch_words_needed(reqs),
                      max_samples=max(v.samples for v in views))
    t_tune = time.perf_counter()
    best, best_ms = batch.autotune(scene, reqs, repeats=2)
    t_tune = time.perf_counter() - t_tune

    def batched():
        batch.render(scene, reqs, stream=sp)

    def timed(fn):
        with torch.cuda.stream(stream):
            for _ in range(2):
                fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(repeats):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                a.record(stream)
                fn()
                b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return float(np.median(ms))

    plain_ms = timed(plain)
    batch_ms = timed(batched)
    batch.free()
    return {
        "workload": f"config 3: {n_cams} cameras, resolutions U{{320x240,640x480,1280x720,1920x1080}}, "
                    f"config-2 poses, {pixels} pixels per batch",
        "plain_sequential": {"value": round(pixels / plain_ms / 1e3, 1), "unit": "Mrays/s", "ms": round(plain_ms, 3)},
        "batched": {"value": round(pixels / batch_ms / 1e3, 1), "unit": "Mrays/s", "ms": round(batch_ms, 3),
                    "mode": ("per-frame launch pairs forked over the batch's 8 worker streams" if best.per_frame
                             else "one persistent raycast + resolve pair replayed from a CUDA graph"),
                    "launches_per_batch": 2 * n_cams if best.per_frame else 2,
                    "cuda_graph": not best.per_frame},
        "speedup": round(plain_ms / batch_ms, 3),
        "autotuned": {"tile_rays": best.tile_rays, "lanes_per_ray": best.lanes_per_ray, "staging": best.staging,
                      "threads_per_block": best.threads_per_block, "per_frame": best.per_frame,
                      "tune_s": round(t_tune, 2)},
    }


def dense_caves_8192(rle, seed=7):
    """Generator settings of the 8192^2 x 512 large-scene workload: fBm
    terrain with cave noise of period 66 voxels carved where its density
    exceeds 0.25 in the band 128-400, for a mean of about 12 runs per column
    and about 6 GB of slab words over 4 levels (the default cave settings
    give about 9.7 runs per column at this size)."""
    p = rle.scenegen_default(8192, 512, 8192, seed, caves=True)
    p.cave_threshold = 0.25
    p.cave_period = 66.0
    return p


def run_config5(rle, torch, frames=120, views_per_batch=8, seed=7, repeats=3):
    """Config 5: the 8192^2 x 512 cave scene (seed 7) built on the GPU
    (generator, mips, encoder and column tables as kernels), then 3840x2160
    frames at 75 deg FOV with LOD switches at 256/512/1024 (mip_distance 256),
    poses 20-200 voxels above the ground, rendered plain (one launch pair per
    frame) and batched (8 views per launch)."""
    p = dense_caves_8192(rle, seed)
    builds = []
    scene = None
    for _ in range(repeats):
        if scene is not None:
            scene.free()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        scene = rle.Scene.generate_on_device(p)
        builds.append(time.perf_counter() - t0)
    info = scene.info()
    table, words = scene.copy_level(0)
    rng = np.random.default_rng(seed)
    cams = []
    for _ in range(frames):
        x, z = rng.uniform(0, 8192, 2)
        g = rle.ground_height(table, words, 8192, 512, int(x), int(z))
        cams.append(rle.camera(float(x), float(z), g + float(rng.uniform(20, 200)), float(rng.uniform(0, 360)),
                               float(rng.uniform(1, 30) * rng.choice([-1, 1])), 75.0, scene_height=512))
    W4, H4 = 3840, 2160
    view = frame_view(rle, W4, H4, mip_distance=256)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    outs = [(torch.empty(W4 * H4, dtype=torch.int32, device="cuda"),
             torch.empty(W4 * H4, dtype=torch.float32, device="cuda")) for _ in range(views_per_batch)]
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")

    def plain():
        for i, cam in enumerate(cams):
            c, d = outs[i % views_per_batch]
            rle.render_frame(scene, cam, view, ws, ws_bytes, c, d, None, stream=sp)

    groups = [[rle.frame_request(cam, view, *outs[k]) for k, cam in enumerate(cams[i:i + views_per_batch])]
              for i in range(0, frames, views_per_batch)]
    batch = rle.Batch(max_frames=views_per_batch, raybuf_words=max(rle.batch_words_needed(g) for g in groups),
                      max_samples=4096)
    best, _ = batch.autotune(scene, groups[0], repeats=1)

    def batched():
        for g in groups:
            batch.render(scene, g, stream=sp)

    def timed(fn):
        with torch.cuda.stream(stream):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    plain_ms = timed(plain)
    batch_ms = timed(batched)
    batch.free()
    del ws
    pixels = W4 * H4 * frames
    slab_bytes = sum(int(info.slab_words[m]) * 2 for m in range(info.nummaps))
    out = {
        "workload": f"config 5: 8192x8192x512 cave scene seed 7 (cave period 66, threshold 0.25) built on the GPU; "
                    f"{frames} frames 3840x2160, 75 deg FOV, mip switches 256/512/1024, poses 20-200 above ground",
        "scene_build_s": round(float(np.median(builds)), 4),
        "scene_device_bytes": int(info.device_bytes),
        "slab_bytes": slab_bytes,
        "runs_per_column": round(info.run_headers / (8192 * 8192), 2),
        "plain": {"value": round(pixels / plain_ms / 1e3, 1), "unit": "Mrays/s", "ms_per_frame": round(plain_ms / frames, 4)},
        "batched": {"value": round(pixels / batch_ms / 1e3, 1), "unit": "Mrays/s",
                    "ms_per_frame": round(batch_ms / frames, 4), "views_per_call": views_per_batch,
                    "mode": ("per-frame launch pairs forked over the batch's 8 worker streams" if best.per_frame
                             else "one persistent raycast + resolve pair per call"),
                    "autotuned": {"tile_rays": best.tile_rays, "lanes_per_ray": best.lanes_per_ray,
                                  "staging": best.staging, "per_frame": best.per_frame}},
    }
    scene.free()
    return out


SERVE_RES = [((256, 256), 0.4), ((640, 480), 0.3), ((1280, 720), 0.2), ((1920, 1080), 0.1)]
SERVE_SCENES = [(1024, 3), (2048, 4), (2048, 5), (4096, 6)]


def run_serving(rle, torch, seconds=60.0, lam=2000.0, seed=20261205, scenes=None, short_seconds=5.0):
    """Config 4: 4 resident scenes (1024^2, 2048^2, 2048^2, 4096^2 x 256,
    seeds 3-6), Poisson arrivals at `lam` requests/s for `seconds`, each
    request a uniform scene and a resolution from SERVE_RES, seeded poses
    (config-2 law), HBM budget 120 GB.  Served twice -- continuous batching
    and one launch per request -- at the offered load for the whole
    `seconds`; then, on the first `short_seconds` of the same arrivals, at
    twice that load (arrival times halved) and at saturation (every request
    queued at once).  Every pass also records where the slowest requests'
    time went: the load generator's lateness against the planned arrival,
    the wait in the server's queue, the device time of the launch that
    carried them (events) and the rest (waiting on the device behind other
    launches, completion polling)."""
    if scenes is None:
        scenes = []
        for n, s in SERVE_SCENES:
            scenes.append(rle.Scene.generate_on_device(rle.scenegen_default(n, 256, n, s, caves=True)))
    rng = np.random.default_rng(seed)
    levels = []
    for sc in scenes:
        info = sc.info()
        t, w = sc.copy_level(0)
        levels.append((info.sx[0], info.sy[0], info.sz[0], t, w))
    n_req = int(lam * seconds)
    n_short = min(n_req, int(lam * short_seconds))
    arrivals = np.cumsum(rng.exponential(1.0 / lam, n_req))
    probs = np.array([p for _, p in SERVE_RES])
    reqs = []
    for i in range(n_req):
        sid = int(rng.integers(0, len(scenes)))
        (w, h) = SERVE_RES[int(rng.choice(len(SERVE_RES), p=probs))][0]
        cam = poses(rle, levels[sid], 1, seed=seed + 7 * i + 1)[0]
        reqs.append((sid, cam, frame_view(rle, w, h)))
    ring = 64  # output buffers reused round-robin
    outs = [(torch.empty(1920 * 1080, dtype=torch.int32, device="cuda"),
             torch.empty(1920 * 1080, dtype=torch.float32, device="cuda")) for _ in range(ring)]
    pixels = sum(v.width * v.height for _, _, v in reqs)
    result = {"workload": f"config 4: 4 resident scenes (1024^2, 2048^2 x2, 4096^2 x 256), Poisson "
                          f"{lam:g} req/s for {seconds:g} s ({n_req} requests, {pixels / n_req / 1e3:.0f} kpx mean), "
                          f"resolution mix 256^2:.4 640x480:.3 1280x720:.2 1920x1080:.1, HBM budget 120 GB",
              "passes": f"offered: all {n_req} requests at {lam:g}/s; offered_2x and saturated: the first "
                        f"{n_short} requests ({short_seconds:g} s of arrivals) at twice the rate and all at once"}
    for mode in ("batched", "plain"):
        srv = rle.Server(hbm_budget_bytes=120 << 30, raybuf_words=32 << 20, max_frames_per_batch=64,
                         max_inflight=3, max_samples=2048, plain=(mode == "plain"))
        for sc in scenes:
            srv.add_scene(sc)
        # warm-up: one of each resolution
        for k in range(8):
            sid, cam, v = reqs[k]
            srv.wait(srv.submit(sid, cam, v, outs[k][0], outs[k][1]))
        srv.reset_stats()
        entry = {}
        for load in ("offered", "offered_2x", "saturated"):
            srv.reset_stats()
            poll_all(srv)
            count = n_req if load == "offered" else n_short
            late = np.zeros(count)
            # the submitting thread is the load generator: a full collection
            # of the interpreter's objects (tens of ms) would hold back the
            # arrivals behind it and release them as one burst
            gc.collect()
            gc.disable()
            t0 = time.perf_counter()
            rate = {"offered": 1.0, "offered_2x": 2.0}.get(load)
            try:
                for i in range(count):
                    sid, cam, v = reqs[i]
                    if rate:
                        due = t0 + arrivals[i] / rate
                        delay = due - time.perf_counter()
                        if delay > 0:
                            time.sleep(delay)
                        late[i] = time.perf_counter() - due
                    c, d = outs[i % ring]
                    srv.submit(sid, cam, v, c, d)
            finally:
                gc.enable()
            srv.drain(600000)
            done = poll_all(srv)
            st = srv.stats()
            entry[load] = {"mrays_per_s": round(st.mrays_per_s, 1), "p50_ms": round(st.p50_ms, 3),
                           "p99_ms": round(st.p99_ms, 3), "max_ms": round(st.max_ms, 3),
                           "completed": int(st.completed), "batches": int(st.batches),
                           "requests": count, "arrival_s": round(float(arrivals[count - 1]) / (rate or 1.0), 2)
                           if rate else 0.0,
                           "wall_s": round(time.perf_counter() - t0, 3)}
            if rate:
                entry[load]["where_the_slowest_1pct_went"] = latency_breakdown(done, late)
        result[mode] = entry
        srv.destroy()
    result["throughput_ratio_saturated"] = round(
        result["batched"]["saturated"]["mrays_per_s"] / max(result["plain"]["saturated"]["mrays_per_s"], 1e-9), 2)
    return result


def poll_all(srv, chunk=65536):
    """Every completion the server holds, oldest first."""
    out = []
    while True:
        got = srv.poll(chunk)
        out.extend(got)
        if len(got) < chunk:
            return out


def latency_breakdown(done, late_s):
    """Where the slowest 1% of a pass's requests spent their time (means, ms):
    the load generator's lateness against the planned arrival (host, Python),
    the wait in the server's queue (submit -> launch), the device time from
    the start of the batch that carried the request to the end of its frame,
    and the rest of launch -> done (waiting on the device behind the other
    in-flight launches, completion polling).
    Also the generator's worst lateness over the whole pass."""
    ok = [c for c in done if c.status == 0]
    if not ok:
        return None
    lat = np.array([(c.done_s - c.submit_s) * 1e3 for c in ok])
    queue = np.array([(c.launch_s - c.submit_s) * 1e3 for c in ok])
    gpu = np.array([c.gpu_ms for c in ok])
    run = np.array([(c.done_s - c.launch_s) * 1e3 for c in ok])
    k = max(1, len(ok) // 100)
    idx = np.argsort(lat)[-k:]
    return {"latency_ms": round(float(lat[idx].mean()), 3),
            "queue_ms": round(float(queue[idx].mean()), 3),
            "launch_gpu_ms": round(float(gpu[idx].mean()), 3),
            "device_wait_and_poll_ms": round(float((run[idx] - gpu[idx]).mean()), 3),
            "requests": int(k),
            "generator_late_ms_p99_max": [round(float(np.percentile(late_s, 99) * 1e3), 3),
                                          round(float(late_s.max() * 1e3), 3)],
            "largest_launch_gpu_ms": round(float(gpu.max()), 3)}


def oracle_raymap(po, cam, w, h):
    """The oracle's RayMap::get_ray_map for a camera and a w x h frame mapped
    as frame_view maps it (maxres w, samples the power of two at or above w,
    border (w-h)/(2w), first LOD switch at w, far distance 80000, fov 90)."""
    return po.raymap_build(list(cam.pos), list(cam.rot), (w - h) / (2 * w), w, 1.0, pow2_ceil(w), w, 80000)


def cpu_baseline(rle, data, cams):
    """The reference's algorithm on the host cores: the oracle port of
    Render::render_line + resolve, OpenMP over column rays, all threads."""
    sys.path.insert(0, str(ROOT))
    from oracle import pyoracle as po
    po.build_oracle()
    oscene = po.OracleScene.from_rle4(data)
    threads = os.cpu_count() or 1
    t = 0.0
    for c in cams:
        t0 = time.perf_counter()
        om = oracle_raymap(po, c, W, H)
        out, dep, _, _ = po.render_rays(om, oscene, nthreads=threads)
        po.resolve(om, W, H, out, dep)
        t += time.perf_counter() - t0
    value = W * H * len(cams) / t / 1e6
    return {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{len(cams)} frame(s) of the same camera path, ray map + raycast + resolve, "
                      f"{t / len(cams) * 1e3:.1f} ms/frame"}


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    rle = load_rle()
    data = scene_bytes(rle)
    sys.path.insert(0, str(ROOT))
    from oracle import pyoracle as po
    po.build_oracle()
    oscene = po.OracleScene.from_rle4(data)
    sx, sy, sz, table, words = oscene.levels[0]
    run_headers = int((table[1::2] & 0xFFFF).astype(np.int64).sum())
    cams = poses(rle, (sx, sy, sz, table, words), args.warmup + args.steps)
    threads = os.cpu_count() or 1

    rays = []

    def frame(c):
        om = oracle_raymap(po, c, W, H)
        rays.append(po.rays_to_render(om))
        out, dep, _, _ = po.render_rays(om, oscene, nthreads=threads)
        po.resolve(om, W, H, out, dep)

    for c in cams[:args.warmup]:
        frame(c)
    rays.clear()  # the timed frames' rays only
    t0 = time.perf_counter()
    for c in cams[args.warmup:]:
        frame(c)
    t = time.perf_counter() - t0
    value = W * H * args.steps / t / 1e6
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene and camera path)",
        "config": bench_config(rays, run_headers / (SCENE["n"] ** 2), world),
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} frame(s): ray map + Render::render_line port + resolve, "
                                   f"OpenMP over column rays, {threads} threads"},
        "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def free_port() -> int:
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def spawn_replicas(n: int, argv: list[str]) -> int:
    """`--gpus N` started without a launcher: N copies of this command, one
    per GPU, with RANK / LOCAL_RANK / WORLD_SIZE and a rendezvous on
    127.0.0.1 set as torch.distributed.run sets them.  Rank 0 prints the JSON
    line; the exit code is the worst of the ranks'."""
    port = str(free_port())
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=port)
        procs.append(subprocess.Popen([sys.executable, str(Path(__file__).resolve()), *argv], env=env))
    rcs = [pr.wait() for pr in procs]
    return max(rcs, key=abs)


def run_plan(args):
    """Host-only check of the replica layout (no GPU): every rank builds its
    own camera path (seed + rank) and ray maps on a small scene of the same
    generator, the ranks reduce their work over the process group (gloo on
    a CPU host) as the GPU run does, and rank 0 prints one JSON line with
    each rank's camera-path digest."""
    import hashlib
    import torch.distributed as dist
    world, rank, _ = dist_setup()
    if world > 1:
        dist.init_process_group(args.backend)
    rle = load_rle()
    n = args.plan_scene
    data = rle.scenegen_rle4(rle.scenegen_default(n, 256, n, SCENE["seed"], caves=True))
    sys.path.insert(0, str(ROOT))
    from oracle import pyoracle as po
    po.build_oracle()
    osc = po.OracleScene.from_rle4(data)
    sx, sy, sz, table, words = osc.levels[0]
    cams = poses(rle, (sx, sy, sz, table, words), args.warmup + args.steps, seed=20261203 + rank)
    view = frame_view(rle, W, H)
    h = hashlib.sha256()
    rays = 0
    for c in cams[args.warmup:]:
        rm = rle.raymap_build(c, view)
        rays += rm.rays
        h.update(bytes(c))
    digest = h.hexdigest()[:16]
    digests = [digest]
    if world > 1:
        digests = [None] * world
        dist.all_gather_object(digests, digest)
    value, ms = replica_throughput(1.0, W * H * args.steps, dist if world > 1 else None, device="cpu")
    if world > 1:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps({"plan": "replicas", "n_gpus": world, "steps": args.steps, "camera_paths": digests,
                          "pixels_all_ranks": round(value * ms / 1e3 * 1e6), "scene": f"{n}^2 x 256"}))
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-frames", type=int, default=3, help="frames in the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the config-3 batched-vs-plain comparison")
    ap.add_argument("--config5-frames", type=int, default=120,
                    help="4K frames of the config-5 run on the 8192^2 x 512 scene (0: skip)")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="seconds of Poisson arrivals of the config-4 offered-load passes (0: skip); the 2x and "
                         "saturated passes use the first 5 s of them")
    ap.add_argument("--no-config1", action="store_true", help="skip the config-1 (512^2, 640x480) frame")
    ap.add_argument("--plan-only", action="store_true",
                    help="host-only check of the replica layout: camera paths per rank, no GPU work")
    ap.add_argument("--plan-scene", type=int, default=256, help="grid of the scene --plan-only uses")
    ap.add_argument("--backend", default="nccl", help="process-group backend of the replicas (gloo on a CPU host)")
    argv = sys.argv[1:] if argv is None else list(argv)
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.gpus < 1:
        ap.error("--gpus must be >= 1")
    world_env = os.environ.get("WORLD_SIZE")
    if world_env is None and args.gpus > 1:
        return spawn_replicas(args.gpus, argv)  # one process per GPU, started here
    if world_env is not None and int(world_env) != args.gpus:
        ap.error(f"--gpus {args.gpus} but WORLD_SIZE={world_env}: start one rank per GPU")
    if args.plan_only:
        return run_plan(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
