"""GPU parity: the sm_103a raycast and resolve, called through the C ABI,
against the oracle (pinned to the reference) and the reference's golden ray
buffers.  Ray-buffer words, hit records and depths are compared bit for bit;
per-ray work counters must match the oracle's exactly.
"""
from __future__ import annotations

import numpy as np
import pytest

from gpu_util import Frame, assert_rays_equal, counters_dict, float_bits, oracle_counters

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden_scene(rle, po, golden, torch_cuda):
    data = golden["scene_rle4"].tobytes()
    return rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data)


@pytest.fixture(scope="module")
def scene512(rle, po, torch_cuda):
    """Config-1 scene: 512x512x256, seed 1, fBm heightfield, 4 levels."""
    data = rle.scenegen_rle4(rle.scenegen_default(512, 256, 512, 1, caves=False))
    return rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data), data


@pytest.fixture(scope="module")
def caves256(rle, po, torch_cuda):
    p = rle.scenegen_default(256, 256, 256, 5, caves=True)
    data = rle.scenegen_rle4(p)
    return rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data), data


def _oracle_frame(po, rm, oscene):
    om = po.raymap_from_product(rm)
    return po.render_rays(om, oscene, want_hits=True, want_counters=True), om


def test_scene_upload_matches_oracle_tables(rle, po, scene512):
    scene, oscene, data = scene512
    info = scene.info()
    assert info.nummaps == 4
    for m in range(4):
        table, words = scene.copy_level(m)
        sx, sy, sz, otab, owords = oscene.levels[m]
        assert (info.sx[m], info.sy[m], info.sz[m]) == (sx, sy, sz)
        assert np.array_equal(words, owords)
        assert np.array_equal(table, otab)
    assert info.run_headers == int((oscene.levels[0][3][1::2] & 0xFFFF).sum())


@pytest.mark.parametrize("i", range(6))
def test_golden_raybuf_bit_exact(rle, po, golden, golden_scene, torch_cuda, i):
    """The reference's own ray buffer (generated by its host build) for six
    poses is reproduced bit for bit on the GPU."""
    scene, oscene = golden_scene
    S, maxres, mipd, zfar = (int(v) for v in golden["params"])
    cam = rle.Camera()
    c = golden[f"cam_{i}"]
    cam.pos[:] = [float(v) for v in c[:3]]
    cam.rot[:] = [float(v) for v in c[3:]]
    cam.fov_deg = 90.0
    view = rle.view_params(S, int(S * 0.75), samples=S, maxres=maxres, border=float(golden["border"][0]),
                           mip_distance=mipd, z_far=zfar)
    rm = rle.raymap_build(cam, view)
    words, depth, hits, cnt = Frame(torch_cuda, rle, scene, rm).rays_host()
    ref = golden[f"raybuf_{i}"]
    assert words.shape == ref.shape
    assert np.array_equal(words, ref), f"{int((words != ref).sum())} of {ref.size} differ from the reference"
    fast = Frame(torch_cuda, rle, scene, rm, hits=False, counters=False).rays_host()[0]
    assert np.array_equal(fast, ref), "fast path (no counters) differs from the reference"
    orc, _ = _oracle_frame(po, rm, oscene)
    assert_rays_equal((words, depth, hits, cnt), orc, f"golden cam {i}")
    assert counters_dict(cnt) == oracle_counters(orc[3])


def test_config1_frame(rle, po, scene512, torch_cuda):
    """Config 1: 640x480, 90 deg, 40 voxels above the terrain centre,
    yaw 30, pitch -15 -- ray buffer, counters and resolved screen."""
    scene, oscene, _ = scene512
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    top = rle.ground_height(t0, s0, 512, 256, 256, 256)
    cam = rle.camera(256.0, 256.0, top + 40.0, 30.0, -15.0)
    rm = rle.raymap_build(cam, rle.view_params(640, 480))
    fr = Frame(torch_cuda, rle, scene, rm)
    gpu = fr.rays_host()
    orc, om = _oracle_frame(po, rm, oscene)
    assert_rays_equal(gpu, orc, "config 1")
    assert counters_dict(gpu[3]) == oracle_counters(orc[3])
    fast = Frame(torch_cuda, rle, scene, rm, hits=True, counters=False).rays_host()
    assert_rays_equal(fast, orc, "config 1 (no counters)")
    col, dep, hit = fr.resolve_host()
    ocol, odep, ohit, _ = po.resolve(om, 640, 480, orc[0], orc[1], orc[2])
    assert np.array_equal(col, ocol), f"{int((col != ocol).sum())} pixels differ"
    assert np.array_equal(float_bits(dep), float_bits(odep))
    assert np.array_equal(hit, ohit)
    assert (col != 0xFFFFCCB2).mean() > 0.3  # terrain is visible


POSES = [  # (yaw, pitch, eye above ground, fov, width, height)
    (10.0, -20.0, 30.0, 90.0, 320, 240),
    (100.0, 25.0, 60.0, 90.0, 320, 240),      # looking up: mostly sky
    (200.0, -75.0, 80.0, 90.0, 256, 192),     # steep: all four fans
    (290.0, -89.0, 40.0, 90.0, 200, 200),     # straight down, square screen
    (45.0, -5.0, 12.0, 75.0, 400, 225),       # 75 deg, 16:9
    (333.0, -40.0, 500.0, 90.0, 160, 120),    # high camera: LOD switching from the start
    (123.0, -10.0, -30.0, 90.0, 160, 120),    # eye inside the ground
    (77.0, -30.0, 25.0, 90.0, 100, 60),       # samples not a multiple of 32
]


@pytest.mark.parametrize("pose", POSES)
def test_cave_scene_poses(rle, po, caves256, torch_cuda, pose):
    scene, oscene, _ = caves256
    yaw, pitch, above, fov, W, H = pose
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    x, z = 97.5, 161.25
    ground = rle.ground_height(t0, s0, 256, 256, int(x), int(z))
    cam = rle.camera(x, z, ground + above, yaw, pitch, fov_deg=fov)
    rm = rle.raymap_build(cam, rle.view_params(W, H, mip_distance=96))
    fr = Frame(torch_cuda, rle, scene, rm)
    gpu = fr.rays_host()
    orc, om = _oracle_frame(po, rm, oscene)
    assert_rays_equal(gpu, orc, str(pose))
    assert counters_dict(gpu[3]) == oracle_counters(orc[3])
    # without counters the kernel may stop a ray early once nothing more can draw
    fast = Frame(torch_cuda, rle, scene, rm, hits=True, counters=False).rays_host()
    assert_rays_equal(fast, orc, f"{pose} (no counters)")
    col, dep, hit = fr.resolve_host()
    ocol, odep, ohit, _ = po.resolve(om, W, H, orc[0], orc[1], orc[2])
    assert np.array_equal(col, ocol) and np.array_equal(float_bits(dep), float_bits(odep))
    assert np.array_equal(hit, ohit)


def test_random_poses_many(rle, po, caves256, torch_cuda):
    """40 seeded poses (uniform yaw, pitch in +-30, 10-80 above ground)."""
    scene, oscene, _ = caves256
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    rng = np.random.default_rng(17)
    total = 0
    for k in range(40):
        x, z = rng.uniform(0, 256, 2)
        g = rle.ground_height(t0, s0, 256, 256, int(x), int(z))
        pitch = float(rng.uniform(1, 30) * rng.choice([-1, 1]))
        cam = rle.camera(float(x), float(z), g + float(rng.uniform(10, 80)), float(rng.uniform(0, 360)), pitch)
        rm = rle.raymap_build(cam, rle.view_params(192, 108, mip_distance=64, z_far=4000))
        gpu = Frame(torch_cuda, rle, scene, rm, hits=True, counters=False).rays_host()
        orc, _ = _oracle_frame(po, rm, oscene)
        assert_rays_equal(gpu, orc, f"pose {k}")
        total += gpu[0].size
    assert total > 0


@pytest.mark.parametrize("pose", [(30.0, -8.0, 20.0), (215.0, -60.0, 90.0)])
def test_maximum_samples(rle, po, caves256, torch_cuda, pose):
    """16384 samples per column ray (the largest ray buffer row the library
    accepts): a 514-word occupancy mask per ray, rows far beyond the packed
    short-span path; counting and fast launches and the resolve."""
    scene, oscene, _ = caves256
    yaw, pitch, above = pose
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    x, z = 140.5, 60.75
    ground = rle.ground_height(t0, s0, 256, 256, int(x), int(z))
    cam = rle.camera(x, z, ground + above, yaw, pitch)
    rm = rle.raymap_build(cam, rle.view_params(400, 300, samples=16384, maxres=64, mip_distance=128))
    assert rm.samples == 16384 and rm.rays > 0
    orc, om = _oracle_frame(po, rm, oscene)
    fr = Frame(torch_cuda, rle, scene, rm)
    gpu = fr.rays_host()
    assert_rays_equal(gpu, orc, f"S=16384 {pose}")
    assert counters_dict(gpu[3]) == oracle_counters(orc[3])
    fast = Frame(torch_cuda, rle, scene, rm, hits=True, counters=False).rays_host()
    assert_rays_equal(fast, orc, f"S=16384 {pose} (no counters)")
    col, dep, hit = fr.resolve_host()
    ocol, odep, ohit, _ = po.resolve(om, 400, 300, orc[0], orc[1], orc[2])
    assert np.array_equal(col, ocol) and np.array_equal(float_bits(dep), float_bits(odep))
    assert np.array_equal(hit, ohit)
    with pytest.raises(rle.RLEError):
        rle.raymap_build(cam, rle.view_params(400, 300, samples=16385))


def test_config2_scene_frames(rle, po, torch_cuda):
    """The benchmark's scene (2048^2 x 256 caves, seed 2) and camera law at
    960x540: the fast path (early ray termination, no counters) against the
    oracle on 10 poses, hit records included."""
    data = rle.scenegen_rle4(rle.scenegen_default(2048, 256, 2048, 2, caves=True))
    scene, oscene = rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data)
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    rng = np.random.default_rng(99)
    for k in range(10):
        x, z = rng.uniform(0, 2048, 2)
        g = rle.ground_height(t0, s0, 2048, 256, int(x), int(z))
        pitch = float(rng.uniform(1, 30) * rng.choice([-1, 1]))
        cam = rle.camera(float(x), float(z), g + float(rng.uniform(10, 80)), float(rng.uniform(0, 360)), pitch)
        rm = rle.raymap_build(cam, rle.view_params(960, 540))
        gpu = Frame(torch_cuda, rle, scene, rm, hits=True, counters=False).rays_host()
        orc, _ = _oracle_frame(po, rm, oscene)
        assert_rays_equal(gpu, orc, f"config-2 pose {k}")
    scene.free()


def test_render_frame_equals_two_calls(rle, scene512, torch_cuda):
    torch = torch_cuda
    scene, oscene, _ = scene512
    cam = rle.camera(100.0, 400.0, 180.0, 250.0, -25.0)
    view = rle.view_params(320, 200)
    rm = rle.raymap_build(cam, view)
    fr = Frame(torch, rle, scene, rm)
    col, dep, hit = fr.resolve_host()
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    c2 = torch.empty(320 * 200, dtype=torch.int32, device="cuda")
    d2 = torch.empty(320 * 200, dtype=torch.float32, device="cuda")
    h2 = torch.empty(320 * 200 * 8, dtype=torch.uint8, device="cuda")
    rle.render_frame(scene, cam, view, ws, ws_bytes, c2, d2, h2)
    torch.cuda.synchronize()
    assert np.array_equal(c2.cpu().numpy().view(np.uint32), col)
    assert np.array_equal(d2.cpu().numpy().view(np.uint32), dep.view(np.uint32))
    assert np.array_equal(h2.cpu().numpy().view(rle.HIT_DTYPE), hit)
    with pytest.raises(rle.RLEError) as e:
        rle.render_frame(scene, cam, view, ws, ws_bytes - 256, c2, d2, h2)
    assert e.value.name == "RLE_ERR_CAPACITY"


def test_degenerate_scenes(rle, po, torch_cuda):
    """A single-level scene, an all-air scene and an all-solid block."""
    n = 32
    vol_empty = np.zeros((n, n * 2, n), bool)
    vol_full = np.ones((n, n * 2, n), bool)
    for vol in (vol_empty, vol_full):
        bits = po.pack_bits(vol)
        _, words = po.encode_mip(bits, n, n * 2, n, 0)
        data = po.write_rle4([(n, n * 2, n, words)])
        scene, oscene = rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data)
        cam = rle.camera(5.5, 7.25, 100.0, 33.0, -20.0, scene_height=n * 2)
        rm = rle.raymap_build(cam, rle.view_params(96, 64, mip_distance=16, z_far=500))
        gpu = Frame(torch_cuda, rle, scene, rm).rays_host()
        orc, _ = _oracle_frame(po, rm, oscene)
        assert_rays_equal(gpu, orc, "degenerate")
        scene.free()


def test_timed_launch_same_rays_and_sane_times(rle, po, caves256, torch_cuda):
    """rle_render_rays_timed: the same ray buffer as the plain launch and
    the oracle, and one time record per cast ray (end after start on the
    SM's clock and on the device-wide clock, SM index below the SM count,
    every ray inside the launch's span)."""
    torch = torch_cuda
    scene, oscene, _ = caves256
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    g = rle.ground_height(t0, s0, 256, 256, 40, 200)
    cam = rle.camera(40.5, 200.5, g + 30.0, 70.0, -12.0)
    rm = rle.raymap_build(cam, rle.view_params(480, 270, mip_distance=96))
    words = rle.raybuf_words(rm)
    raybuf = torch.empty(words, dtype=torch.int32, device="cuda")
    raydepth = torch.empty(words, dtype=torch.float32, device="cuda")
    times = torch.zeros(rm.rays * rle.RAY_TIME_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    rle.render_rays_timed(scene, rm, raybuf, raydepth, times)
    torch.cuda.synchronize()
    n = rm.rays * rm.samples
    got = (raybuf[:n].cpu().numpy().view(np.uint32), raydepth[:n].cpu().numpy(), None, None)
    orc, _ = _oracle_frame(po, rm, oscene)
    assert_rays_equal(got, orc, "timed launch")
    t = times.cpu().numpy().view(rle.RAY_TIME_DTYPE)
    assert t.size == rm.rays
    assert (t["end_clock"] >= t["start_clock"]).all() and (t["end_ns"] >= t["start_ns"]).all()
    assert (t["start_ns"] > 0).all()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert (t["sm"] < sms).all()
    span_ns = int(t["end_ns"].max() - t["start_ns"].min())
    assert 0 < span_ns < 10_000_000_000
