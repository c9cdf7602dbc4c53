"""Randomised parity: seeded random scenes (grid and height, caves or not,
number of mip levels), views (screen shape, samples per ray, ray count, mip
switch distance, far distance, field of view) and cameras (inside and
outside the map -- the grid wraps --, above the scene's top, under the
ground, any yaw, pitch up to +-89 degrees), rendered on the GPU through the
C ABI and compared with the oracle: ray-buffer words, depths, hit records,
the per-ray work counters of the counting launch, and the resolved screen,
bit for bit (NaN depths, which degenerate spans make on every platform, must
meet NaN at the same sample; their bit patterns are the platform's).
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from gpu_util import (Frame, assert_rays_equal, assert_screen_equal, counters_dict, float_bits, oracle_counters,
                      oracle_screen)

pytestmark = pytest.mark.gpu

# RLE_FUZZ_CASES widens the sweep (the default keeps the suite quick)
CASES = int(os.environ.get("RLE_FUZZ_CASES", "64"))


def _scene(rle, po, rng):
    n = int(rng.choice([32, 64, 128, 256]))
    sy = int(rng.choice([64, 128, 256, 512]))
    p = rle.scenegen_default(n, sy, n, int(rng.integers(1, 1 << 30)), caves=bool(rng.integers(0, 2)))
    p.nummaps = int(rng.integers(1, 5))
    data = rle.scenegen_rle4(p)
    return rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data), n, sy


def _view(rle, rng):
    W = int(rng.integers(64, 481))
    H = int(rng.integers(48, W + 1))
    samples = int(rng.choice([0, int(rng.integers(8, 1025)), 1 << int(rng.integers(6, 11))]))
    maxres = int(rng.choice([0, int(rng.integers(16, W + 1))]))
    mipd = int(rng.choice([0, int(rng.integers(16, 513))]))
    zfar = int(rng.choice([0, int(rng.integers(64, 4001))]))
    return rle.view_params(W, H, samples=samples, maxres=maxres, mip_distance=mipd, z_far=zfar)


def _camera(rle, rng, oscene, n, sy):
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    x, z = rng.uniform(-0.5 * n, 1.5 * n, 2)
    ground = rle.ground_height(t0, s0, n, sy, int(x) % n, int(z) % n)
    kind = int(rng.integers(0, 4))
    if kind == 0:
        eye = ground - float(rng.uniform(1, 20))            # under the ground
    elif kind == 1:
        eye = sy + float(rng.uniform(1, 2 * sy))            # above the scene's top
    else:
        eye = ground + float(rng.uniform(2, 0.6 * sy))
    return rle.camera(float(x), float(z), eye, float(rng.uniform(0, 360)), float(rng.uniform(-89, 89)),
                      fov_deg=float(rng.uniform(30, 120)), scene_height=sy)


@pytest.mark.parametrize("case", range(CASES))
def test_random_scene_view_camera(rle, po, torch_cuda, case):
    rng = np.random.default_rng(9000 + case)
    scene, oscene, n, sy = _scene(rle, po, rng)
    view = _view(rle, rng)
    cam = _camera(rle, rng, oscene, n, sy)
    rm = rle.raymap_build(cam, view)
    label = (f"case {case}: {n}x{sy}x{n}, {view.width}x{view.height} S={rm.samples} rays={rm.rays} "
             f"mipd={rm.mip_distance} zfar={rm.z_far}")
    om = po.raymap_from_product(rm)
    orc = po.render_rays(om, oscene, want_hits=True, want_counters=True)
    fr = Frame(torch_cuda, rle, scene, rm)  # the counting launch: every valid cell walked exactly
    gpu = fr.rays_host()
    assert_rays_equal(gpu, orc, label)
    assert counters_dict(gpu[3]) == oracle_counters(orc[3]), label
    fast = Frame(torch_cuda, rle, scene, rm, hits=True, counters=False).rays_host()
    assert_rays_equal(fast, orc, label + " (fast path)")
    col, dep, hit = fr.resolve_host()
    ocol, odep, ohit, _ = po.resolve(om, view.width, view.height, orc[0], orc[1], orc[2])
    assert np.array_equal(col, ocol), f"{label}: {int((col != ocol).sum())} pixels differ"
    assert np.array_equal(float_bits(dep), float_bits(odep)), label
    assert np.array_equal(hit, ohit), label
    scene.free()


@pytest.mark.parametrize("case", range(max(12, CASES // 5)))
def test_random_batches(rle, po, torch_cuda, case):
    """Batches of 2-6 random views and cameras of one random scene, under a
    random launch shape (claim tile, lanes per ray, staging, graph or not,
    one launch pair per frame or not), equal the frames rendered one by one
    and the oracle's screens: colour, depth (NaN meeting NaN) and hit
    records."""
    torch = torch_cuda
    rng = np.random.default_rng(7000 + case)
    scene, oscene, n, sy = _scene(rle, po, rng)
    frames = []
    for _ in range(int(rng.integers(2, 7))):
        view = _view(rle, rng)
        frames.append((_camera(rle, rng, oscene, n, sy), view))
    outs = []
    for cam, view in frames:
        px = view.width * view.height
        outs.append((torch.full((px,), 7, dtype=torch.int32, device="cuda"),
                     torch.full((px,), 7.0, dtype=torch.float32, device="cuda"),
                     torch.zeros(px * 8, dtype=torch.uint8, device="cuda")))
    reqs = [rle.frame_request(c, v, *o) for (c, v), o in zip(frames, outs)]
    max_s = max(rle.raymap_build(c, v).samples for c, v in frames)
    b = rle.Batch(len(frames), rle.batch_words_needed(reqs), max_s, with_hits=True)
    shape = (int(rng.choice([1, 2, 4, 16])), int(rng.choice([8, 16, 32])), int(rng.integers(1, 4)),
             int(rng.choice([32, 64, 128])), int(rng.integers(0, 2)), int(rng.integers(0, 2)))
    b.set_tuning(*shape)
    b.render(scene, reqs)
    torch.cuda.synchronize()
    for k, (cam, view) in enumerate(frames):
        ws_bytes = rle.frame_workspace_bytes(view)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
        px = view.width * view.height
        c = torch.empty(px, dtype=torch.int32, device="cuda")
        d = torch.empty(px, dtype=torch.float32, device="cuda")
        h = torch.empty(px * 8, dtype=torch.uint8, device="cuda")
        rle.render_frame(scene, cam, view, ws, ws_bytes, c, d, h)
        torch.cuda.synchronize()
        label = f"case {case} frame {k} shape {shape}"
        assert torch.equal(outs[k][0], c), label
        assert np.array_equal(float_bits(outs[k][1].cpu().numpy()), float_bits(d.cpu().numpy())), label
        assert torch.equal(outs[k][2], h), label
        got = (outs[k][0].cpu().numpy().view(np.uint32), outs[k][1].cpu().numpy(),
               outs[k][2].cpu().numpy().view(rle.HIT_DTYPE))
        assert_screen_equal(got, oracle_screen(po, rle, oscene, cam, view), label + " vs oracle")
    b.free()
    scene.free()
