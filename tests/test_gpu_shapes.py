"""Every launch shape of the raycast (lanes per ray x block size x staging
depth) gives the same bits: ray buffer, depths, hit records and work
counters equal the oracle's for a plain terrain and a cave scene."""
from __future__ import annotations

import numpy as np
import pytest

from gpu_util import Frame, assert_rays_equal, counters_dict, oracle_counters

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes(rle, po, torch_cuda):
    out = []
    for n, caves, seed in ((256, False, 1), (256, True, 3)):
        data = rle.scenegen_rle4(rle.scenegen_default(n, 256, n, seed, caves=caves))
        out.append((rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data)))
    yield out
    rle.tuning_set(0, 0, 0, 0)


SHAPES = [(8, 1), (16, 1), (32, 1)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("threads,staging", [(32, 1), (128, 1), (128, 2), (64, 3)])
def test_shapes_bit_exact(rle, po, scenes, torch_cuda, shape, threads, staging):
    lanes, cells = shape
    rle.tuning_set(lanes, cells, threads, staging)
    assert rle.tuning_get() == (lanes, cells, threads, staging)
    try:
        for si, (scene, oscene) in enumerate(scenes):
            t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
            for yaw, pitch, above, W, H in ((30.0, -15.0, 40.0, 320, 240), (210.0, -60.0, 70.0, 240, 180),
                                           (95.0, 12.0, 25.0, 200, 120)):
                x, z = 101.5, 57.25
                g = rle.ground_height(t0, s0, 256, 256, int(x), int(z))
                cam = rle.camera(x, z, g + above, yaw, pitch)
                rm = rle.raymap_build(cam, rle.view_params(W, H, mip_distance=80))
                gpu = Frame(torch_cuda, rle, scene, rm).rays_host()
                om = po.raymap_from_product(rm)
                orc = po.render_rays(om, oscene, want_hits=True, want_counters=True)
                assert_rays_equal(gpu, orc, f"scene {si} shape {shape} threads {threads} staging {staging} yaw {yaw}")
                assert counters_dict(gpu[3]) == oracle_counters(orc[3])
                # without counters/hits the fast path (cells that may draw only)
                fast = Frame(torch_cuda, rle, scene, rm, hits=False, counters=False).rays_host()
                assert np.array_equal(fast[0], gpu[0]) and np.array_equal(fast[1].view(np.uint32),
                                                                          gpu[1].view(np.uint32))
    finally:
        rle.tuning_set(0, 0, 0, 0)


def test_tuning_rejects_bad_shapes(rle):
    for lanes, cells, threads, staging in ((3, 1, 128, 0), (8, 1, 40, 0), (8, 1, 256, 0), (64, 1, 128, 0),
                                           (32, 2, 128, 0), (4, 1, 128, 0), (32, 1, 128, 4), (32, 1, 128, -1)):
        with pytest.raises(rle.RLEError):
            rle.tuning_set(lanes, cells, threads, staging)
