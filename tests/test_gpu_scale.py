"""Parity at the benchmark's full sizes.

- config 2: 1920x1080 frames of the 2048^2 x 256 cave scene, ray buffers and
  the resolved screen against the oracle;
- config 5: the 8192^2 x 512 scene built on the GPU, copied level by level
  to the host for the oracle, and a 3840x2160, 75 degree frame with mip
  switches at 256/512/1024 compared ray by ray (words, depths, hit records);
- the batched launch at config-5 size equals the plain launches and the
  oracle's screens.
"""
from __future__ import annotations

import numpy as np
import pytest

from gpu_util import Frame, assert_rays_equal, assert_screen_equal, float_bits, oracle_screen

pytestmark = pytest.mark.gpu


def _bench():
    import sys
    from pathlib import Path
    root = str(Path(__file__).resolve().parents[1])
    if root not in sys.path:
        sys.path.insert(0, root)
    import bench
    return bench


def _poses(rle, table, words, sx, sy, sz, n, seed, lo, hi, fov):
    rng = np.random.default_rng(seed)
    cams = []
    for _ in range(n):
        x, z = rng.uniform(0, sx), rng.uniform(0, sz)
        g = rle.ground_height(table, words, sx, sy, int(x), int(z))
        pitch = float(rng.uniform(1, 30) * rng.choice([-1, 1]))
        cams.append(rle.camera(float(x), float(z), g + float(rng.uniform(lo, hi)), float(rng.uniform(0, 360)),
                               pitch, fov, scene_height=sy))
    return cams


def test_config2_full_frames(rle, po, torch_cuda):
    torch = torch_cuda
    data = rle.scenegen_rle4(rle.scenegen_default(2048, 256, 2048, 2, caves=True))
    scene, oscene = rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data)
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    view = rle.view_params(1920, 1080, samples=2048)  # the configs' mapping: S = pow2 >= width
    for k, cam in enumerate(_poses(rle, t0, s0, 2048, 256, 2048, 3, 20261203, 10, 80, 90.0)):
        rm = rle.raymap_build(cam, view)
        fr = Frame(torch, rle, scene, rm, hits=True, counters=False)
        gpu = fr.rays_host()
        om = po.raymap_from_product(rm)
        orc = po.render_rays(om, oscene, want_hits=True)
        assert_rays_equal(gpu, orc, f"1080p pose {k}")
        col, dep, _ = fr.resolve_host()
        ocol, odep, _, _ = po.resolve(om, 1920, 1080, orc[0], orc[1], orc[2])
        assert np.array_equal(col, ocol), f"pose {k}: {int((col != ocol).sum())} pixels differ"
        assert np.array_equal(float_bits(dep), float_bits(odep))
    scene.free()


@pytest.fixture(scope="module")
def config5(rle, po, torch_cuda):
    p = _bench().dense_caves_8192(rle, 7)  # the benchmark's large scene, ~12 runs per column
    scene = rle.Scene.generate_on_device(p)
    info = scene.info()
    levels = []
    for m in range(info.nummaps):
        _, words = scene.copy_level(m)
        levels.append((info.sx[m], info.sy[m], info.sz[m], words))
    oscene = po.OracleScene(levels)
    # the device tables equal the oracle's walk of the device slab words
    for m in range(info.nummaps):
        table, _ = scene.copy_level(m)
        assert np.array_equal(table, oscene.levels[m][3]), f"level {m} table"
    yield scene, oscene
    scene.free()


def test_config5_4k_frame(rle, po, torch_cuda, config5):
    scene, oscene = config5
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    view = rle.view_params(3840, 2160, samples=4096, mip_distance=256)
    for k, cam in enumerate(_poses(rle, t0, s0, 8192, 512, 8192, 2, 7, 20, 200, 75.0)):
        rm = rle.raymap_build(cam, view)
        assert rm.samples == 4096
        gpu = Frame(torch_cuda, rle, scene, rm, hits=True, counters=False).rays_host()
        orc = po.render_rays(po.raymap_from_product(rm), oscene, want_hits=True)
        assert_rays_equal(gpu, orc, f"4K pose {k}")


def test_config5_batched_equals_plain(rle, po, torch_cuda, config5):
    """Four 4K views of the large scene in one batch: each equals the plain
    launch and the oracle's screen."""
    torch = torch_cuda
    scene, oscene = config5
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    view = rle.view_params(3840, 2160, samples=4096, mip_distance=256)
    cams = _poses(rle, t0, s0, 8192, 512, 8192, 4, 8, 20, 200, 75.0)
    n = 3840 * 2160
    outs = [(torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda"))
            for _ in cams]
    reqs = [rle.frame_request(c, view, o[0], o[1]) for c, o in zip(cams, outs)]
    b = rle.Batch(len(cams), rle.batch_words_needed(reqs), 4096)
    b.render(scene, reqs)
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    c = torch.empty(n, dtype=torch.int32, device="cuda")
    d = torch.empty(n, dtype=torch.float32, device="cuda")
    for k, cam in enumerate(cams):
        rle.render_frame(scene, cam, view, ws, ws_bytes, c, d)
        torch.cuda.synchronize()
        assert torch.equal(c, outs[k][0]), f"frame {k} colour"
        assert torch.equal(d.view(torch.int32), outs[k][1].view(torch.int32)), f"frame {k} depth"
        got = (outs[k][0].cpu().numpy().view(np.uint32), outs[k][1].cpu().numpy(), None)
        assert_screen_equal(got, oracle_screen(po, rle, oscene, cam, view, hits=False), f"4K batch frame {k}")
    b.free()
