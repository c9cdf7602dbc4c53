"""Batched rendering (rle_batch_*): many cameras of mixed resolution in one
persistent raycast + resolve, replayed from a captured CUDA graph.  Every
frame must equal the oracle's screen for its camera (the oracle's own ray
map, Render::render_line restatement and resolve: colour and hit records
bit for bit, depth bit for bit with NaN meeting NaN) and the same camera
rendered alone by rle_render_frame, for every launch shape, with and without
the graph, across consecutive batches of different sizes; the config-3 mix
(64 cameras up to 1920x1080 on the 2048^2 cave scene) included."""
from __future__ import annotations

import numpy as np
import pytest

from gpu_util import assert_screen_equal, oracle_screen

pytestmark = pytest.mark.gpu

RES = [(160, 120), (320, 240), (640, 480), (200, 200), (400, 225)]


@pytest.fixture(scope="module")
def scene_pair(rle, po, torch_cuda):
    data = rle.scenegen_rle4(rle.scenegen_default(256, 256, 256, 4, caves=True))
    s = rle.Scene.from_bytes(data)
    yield s, po.OracleScene.from_rle4(data)
    s.free()


@pytest.fixture(scope="module")
def scene(scene_pair):
    return scene_pair[0]


def _cameras(rle, scene, n, seed):
    info = scene.info()
    table, words = scene.copy_level(0)
    rng = np.random.default_rng(seed)
    cams = []
    for i in range(n):
        x, z = rng.uniform(0, 256, 2)
        g = rle.ground_height(table, words, info.sx[0], info.sy[0], int(x), int(z))
        pitch = float(rng.uniform(2, 60) * rng.choice([-1, 1]))
        cam = rle.camera(float(x), float(z), g + float(rng.uniform(10, 80)), float(rng.uniform(0, 360)), pitch)
        w, h = RES[i % len(RES)]
        cams.append((cam, rle.view_params(w, h, mip_distance=96)))
    return cams


def _alone(rle, torch, scene, cam, view):
    n = view.width * view.height
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    c = torch.empty(n, dtype=torch.int32, device="cuda")
    d = torch.empty(n, dtype=torch.float32, device="cuda")
    h = torch.empty(n * 8, dtype=torch.uint8, device="cuda")
    rle.render_frame(scene, cam, view, ws, ws_bytes, c, d, h)
    torch.cuda.synchronize()
    return c.cpu().numpy().view(np.uint32), d.cpu().numpy(), h.cpu().numpy().view(rle.HIT_DTYPE)


class Outputs:
    def __init__(self, torch, rle, cams, hits=True):
        self.bufs = []
        self.reqs = []
        for cam, view in cams:
            n = view.width * view.height
            c = torch.full((n,), 3, dtype=torch.int32, device="cuda")
            d = torch.full((n,), 3.0, dtype=torch.float32, device="cuda")
            h = torch.zeros(n * 8, dtype=torch.uint8, device="cuda") if hits else None
            self.bufs.append((c, d, h))
            self.reqs.append(rle.frame_request(cam, view, c, d, h))

    def host(self, rle, i):
        c, d, h = self.bufs[i]
        return (c.cpu().numpy().view(np.uint32), d.cpu().numpy(),
                h.cpu().numpy().view(rle.HIT_DTYPE) if h is not None else None)


def _check(rle, torch, scene, cams, outs, label, po=None, oscene=None):
    """Every batched frame against the same camera rendered alone and, where
    the oracle scene is given, against the oracle's screen."""
    torch.cuda.synchronize()
    for i, (cam, view) in enumerate(cams):
        want = _alone(rle, torch, scene, cam, view)
        got = outs.host(rle, i)
        assert np.array_equal(got[0], want[0]), f"{label} frame {i}: {int((got[0] != want[0]).sum())} pixels differ"
        assert np.array_equal(got[1].view(np.uint32), want[1].view(np.uint32)), f"{label} frame {i} depth"
        if got[2] is not None:
            assert np.array_equal(got[2], want[2]), f"{label} frame {i} hits"
        if oscene is not None:
            orc = oracle_screen(po, rle, oscene, cam, view, hits=got[2] is not None)
            assert_screen_equal(got, orc, f"{label} frame {i} ({view.width}x{view.height}) vs oracle")


def test_batch_matches_single_frames(rle, po, scene_pair, torch_cuda):
    torch = torch_cuda
    scene, oscene = scene_pair
    cams = _cameras(rle, scene, 12, 1)
    outs = Outputs(torch, rle, cams)
    words = rle.batch_words_needed(outs.reqs)
    assert words > 0
    b = rle.Batch(max_frames=16, raybuf_words=words, max_samples=1024, with_hits=True)
    b.render(scene, outs.reqs)
    _check(rle, torch, scene, cams, outs, "graph", po, oscene)
    # replay the captured graph with another, smaller batch, then the first again
    cams2 = _cameras(rle, scene, 5, 2)
    outs2 = Outputs(torch, rle, cams2)
    b.render(scene, outs2.reqs)
    _check(rle, torch, scene, cams2, outs2, "second batch", po, oscene)
    outs3 = Outputs(torch, rle, cams)
    b.render(scene, outs3.reqs)
    _check(rle, torch, scene, cams, outs3, "third batch", po, oscene)
    b.free()


@pytest.mark.parametrize("shape", [(1, 8, 1, 128, 1, 0), (8, 16, 3, 64, 1, 0), (64, 32, 2, 128, 0, 0),
                                   (16, 32, 1, 32, 1, 0), (1, 32, 1, 128, 1, 1), (1, 16, 1, 64, 0, 1)])
def test_batch_shapes(rle, po, scene_pair, torch_cuda, shape):
    torch = torch_cuda
    scene, oscene = scene_pair
    cams = _cameras(rle, scene, 7, 3)
    outs = Outputs(torch, rle, cams, hits=False)
    b = rle.Batch(max_frames=8, raybuf_words=rle.batch_words_needed(outs.reqs), max_samples=1024)
    b.set_tuning(*shape)
    assert b.tuning().as_tuple() == shape
    b.render(scene, outs.reqs)
    b.render(scene, outs.reqs)  # twice in a row on the same outputs
    _check(rle, torch, scene, cams, outs, f"shape {shape}", po, oscene)
    b.free()


@pytest.mark.parametrize("lanes", [8, 16, 32])
def test_batch_maximum_samples(rle, po, scene_pair, torch_cuda, lanes):
    """A batch created for 16384 samples per ray (the library's limit) mixing
    frames at that row length with ordinary ones equals the plain launches
    and the oracle."""
    torch = torch_cuda
    scene, oscene = scene_pair
    cams = []
    for i, (cam, view) in enumerate(_cameras(rle, scene, 4, 9)):
        if i % 2 == 0:
            view = rle.view_params(320, 240, samples=16384, maxres=48, mip_distance=96)
        cams.append((cam, view))
    outs = Outputs(torch, rle, cams)
    b = rle.Batch(max_frames=4, raybuf_words=rle.batch_words_needed(outs.reqs), max_samples=16384, with_hits=True)
    b.set_tuning(1, lanes, 1, 128)
    b.render(scene, outs.reqs)
    _check(rle, torch, scene, cams, outs, f"S=16384, {lanes} lanes", po, oscene)
    b.free()


def test_batch_refuses_what_it_cannot_hold(rle, scene, torch_cuda):
    torch = torch_cuda
    cams = _cameras(rle, scene, 3, 4)
    outs = Outputs(torch, rle, cams)
    words = rle.batch_words_needed(outs.reqs)
    small = rle.Batch(max_frames=4, raybuf_words=words // 2, max_samples=1024, with_hits=True)
    with pytest.raises(rle.RLEError) as e:
        small.render(scene, outs.reqs)
    assert e.value.name == "RLE_ERR_CAPACITY"
    nohits = rle.Batch(max_frames=4, raybuf_words=words, max_samples=1024, with_hits=False)
    with pytest.raises(rle.RLEError):
        nohits.render(scene, outs.reqs)  # hit outputs asked of a batch without hit storage
    narrow = rle.Batch(max_frames=4, raybuf_words=words, max_samples=256, with_hits=True)
    with pytest.raises(rle.RLEError) as e:
        narrow.render(scene, outs.reqs)  # 640-wide frame: 640 samples per ray
    assert e.value.name == "RLE_ERR_CAPACITY"
    with pytest.raises(rle.RLEError):
        rle.Batch(max_frames=2, raybuf_words=words, max_samples=1024).render(scene, outs.reqs)  # too many frames
    for b in (small, nohits, narrow):
        b.free()


def test_autotune_picks_a_valid_shape(rle, po, scene_pair, torch_cuda):
    torch = torch_cuda
    scene, oscene = scene_pair
    cams = _cameras(rle, scene, 6, 5)
    outs = Outputs(torch, rle, cams, hits=False)
    b = rle.Batch(max_frames=8, raybuf_words=rle.batch_words_needed(outs.reqs), max_samples=1024)
    best, ms = b.autotune(scene, outs.reqs, repeats=1)
    assert best.tile_rays in (1, 2, 4, 8, 16, 32, 64) and best.lanes_per_ray in (8, 16, 32) and best.staging in (1, 2, 3)
    assert best.per_frame in (0, 1)
    assert ms > 0
    assert b.tuning().as_tuple() == best.as_tuple()
    b.render(scene, outs.reqs)
    _check(rle, torch, scene, cams, outs, "autotuned", po, oscene)
    b.free()


CONFIG3_RES = [(320, 240), (640, 480), (1280, 720), (1920, 1080)]


def _pow2_ceil(v):
    p = 1
    while p < v:
        p <<= 1
    return p


def test_config3_mix_against_oracle(rle, po, torch_cuda):
    """Config 3 at its own size: 64 cameras with resolutions drawn from
    {320x240, 640x480, 1280x720, 1920x1080} (samples per ray the power of
    two at or above the width, maxres the width), config-2 poses (10-80
    above the ground, yaw U[0,360), pitch +-[1,30]) on the 2048^2 x 256 cave
    scene (seed 2), in one batch -- autotuned, then under a fixed 32-lane
    shape -- each frame against the oracle's screen."""
    torch = torch_cuda
    data = rle.scenegen_rle4(rle.scenegen_default(2048, 256, 2048, 2, caves=True))
    scene, oscene = rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data)
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    rng = np.random.default_rng(20261204)
    cams = []
    for i in range(64):
        # the first four cameras take every resolution once
        w, h = CONFIG3_RES[i] if i < 4 else CONFIG3_RES[int(rng.integers(0, 4))]
        x, z = rng.uniform(0, 2048, 2)
        g = rle.ground_height(t0, s0, 2048, 256, int(x), int(z))
        pitch = float(rng.uniform(1, 30) * rng.choice([-1, 1]))
        cam = rle.camera(float(x), float(z), g + float(rng.uniform(10, 80)), float(rng.uniform(0, 360)), pitch)
        cams.append((cam, rle.view_params(w, h, samples=_pow2_ceil(w))))
    assert {(v.width, v.height) for _, v in cams} == set(CONFIG3_RES)
    want = [oracle_screen(po, rle, oscene, cam, view, hits=False) for cam, view in cams]
    outs = Outputs(torch, rle, cams, hits=False)
    b = rle.Batch(max_frames=64, raybuf_words=rle.batch_words_needed(outs.reqs), max_samples=2048)
    b.autotune(scene, outs.reqs, repeats=1)
    for label, shape in (("autotuned", None), ("32 lanes, 4-ray claims", (4, 32, 2, 128, 1, 0))):
        if shape:
            b.set_tuning(*shape)
        outs = Outputs(torch, rle, cams, hits=False)
        b.render(scene, outs.reqs)
        torch.cuda.synchronize()
        for i, (cam, view) in enumerate(cams):
            assert_screen_equal(outs.host(rle, i), want[i],
                                f"config 3 {label} frame {i} ({view.width}x{view.height})")
    b.free()
    scene.free()


def test_consecutive_batches_on_two_streams(rle, po, scene_pair, torch_cuda):
    """Two batches of one batch object issued back to back on two streams,
    with nothing ordering the streams: the second call's device work waits
    for the first's (they share the batch's ray buffer and parameter block),
    so both sets of frames equal the oracle's screens."""
    torch = torch_cuda
    scene, oscene = scene_pair
    cams_a = _cameras(rle, scene, 6, 41)
    cams_b = _cameras(rle, scene, 6, 42)
    outs_a = Outputs(torch, rle, cams_a, hits=False)
    outs_b = Outputs(torch, rle, cams_b, hits=False)
    words = max(rle.batch_words_needed(outs_a.reqs), rle.batch_words_needed(outs_b.reqs))
    b = rle.Batch(max_frames=8, raybuf_words=words, max_samples=1024)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    # the persistent launches with and without the graph, and the per-frame
    # launches forked over the batch's worker streams
    for use_graph, per_frame in ((1, 0), (0, 0), (0, 1)):
        b.set_tuning(1, 32 if not per_frame else 16, 1, 128, use_graph, per_frame)
        for _ in range(3):
            b.render(scene, outs_a.reqs, stream=s1.cuda_stream)
            b.render(scene, outs_b.reqs, stream=s2.cuda_stream)
        torch.cuda.synchronize()
        for cams, outs, tag in ((cams_a, outs_a, "stream 1"), (cams_b, outs_b, "stream 2")):
            for i, (cam, view) in enumerate(cams):
                assert_screen_equal(outs.host(rle, i), oracle_screen(po, rle, oscene, cam, view, hits=False),
                                    f"{tag} graph={use_graph} per_frame={per_frame} frame {i}")
    b.free()
