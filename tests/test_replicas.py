"""The multi-GPU path of the benchmark is replicas only (column rays,
cameras and frames are independent; no exchange step): each rank renders
its own camera path and the job's throughput is the work of all ranks over
the slowest rank's time.  The reduction runs here as world_size-2 gloo
ranks on the CPU."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank 1 is the slow one and renders fewer pixels
        local_ms = [100.0, 250.0][rank]
        units = [2_000_000, 1_000_000][rank]
        value, ms = bench.replica_throughput(local_ms, units, dist, device="cpu")
        q.put((rank, value, ms))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, ms in res:
        assert ms == 250.0                       # the slowest rank's time
        assert value == pytest.approx(3_000_000 / 0.25 / 1e6)  # all ranks' pixels


def test_replica_throughput_single_process():
    sys.path.insert(0, str(ROOT))
    import bench
    value, ms = bench.replica_throughput(200.0, 4_000_000, None)
    assert ms == 200.0 and value == pytest.approx(20.0)


def test_ranks_render_distinct_camera_paths(rle):
    """bench seeds each rank's camera path with its rank: replicas render
    different frames, not copies of one."""
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import bench
    from oracle import pyoracle as po
    p = rle.scenegen_default(64, 64, 64, 3)
    sx, sy, sz, words = po.parse_rle4(rle.scenegen_rle4(p))[0]
    table = po.build_table(words, sx, sz)
    a = bench.poses(rle, (sx, sy, sz, table, words), 4, seed=20261203 + 0)
    b = bench.poses(rle, (sx, sy, sz, table, words), 4, seed=20261203 + 1)
    assert not np.allclose([c.pos[0] for c in a], [c.pos[0] for c in b])


def test_gpus_flag_starts_that_many_ranks():
    """`bench.py --gpus 2` started without a launcher starts two ranks
    itself (RANK / WORLD_SIZE set as torch.distributed.run sets them); here
    in its host-only plan mode over gloo: both ranks join, their camera
    paths differ, and the reduced work is both ranks' pixels.  A --gpus
    that disagrees with an outer launcher's WORLD_SIZE is refused."""
    import json
    import subprocess
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--plan-only", "--backend", "gloo",
                        "--steps", "4", "--warmup", "3", "--plan-scene", "128"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["n_gpus"] == 2
    assert len(line["camera_paths"]) == 2 and line["camera_paths"][0] != line["camera_paths"][1]
    assert line["pixels_all_ranks"] == 2 * 4 * 1920 * 1080
    bad = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--plan-only"],
                         capture_output=True, text=True, timeout=120, cwd=ROOT, env=dict(env, WORLD_SIZE="3"))
    assert bad.returncode != 0 and "WORLD_SIZE" in bad.stderr
