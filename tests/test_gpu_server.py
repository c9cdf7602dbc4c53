"""Render server (rle_server_*): continuous batching over resident scenes.

- every result served in a mixed stream equals the same request rendered
  alone and the oracle's screen for it (bit for bit), for the batching and
  the plain server, at test sizes and in a config-4 mix (two resident
  scenes of different sizes, resolutions up to 1920x1080);
- admission: budgets and per-request limits refuse cleanly;
- failure handling without any device fault: cancelled requests, bounded
  waits that time out, and injected launch failures (host side) that fail
  only their own batch while the server keeps serving.
"""
from __future__ import annotations

import numpy as np
import pytest

from gpu_util import assert_screen_equal, oracle_screen

pytestmark = pytest.mark.gpu

RES = [(256, 256), (640, 480), (320, 240), (400, 300)]


@pytest.fixture(scope="module")
def scene_pairs(rle, po, torch_cuda):
    out = []
    for n, seed in ((256, 3), (128, 4)):
        data = rle.scenegen_rle4(rle.scenegen_default(n, 256, n, seed, caves=True))
        out.append((rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data)))
    yield out
    for s, _ in out:
        s.free()


@pytest.fixture(scope="module")
def scenes(scene_pairs):
    return [s for s, _ in scene_pairs]


def _requests(rle, scenes, n, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        sid = int(rng.integers(0, len(scenes)))
        sc = scenes[sid]
        info = sc.info()
        table, words = sc.copy_level(0)
        x, z = rng.uniform(0, info.sx[0], 2)
        g = rle.ground_height(table, words, info.sx[0], info.sy[0], int(x), int(z))
        cam = rle.camera(float(x), float(z), g + float(rng.uniform(10, 60)), float(rng.uniform(0, 360)),
                         float(rng.uniform(2, 40) * rng.choice([-1, 1])))
        w, h = RES[i % len(RES)]
        reqs.append((sid, cam, rle.view_params(w, h, mip_distance=64)))
    return reqs


def _buffers(torch, reqs):
    return [(torch.full((v.width * v.height,), 5, dtype=torch.int32, device="cuda"),
             torch.full((v.width * v.height,), 5.0, dtype=torch.float32, device="cuda")) for _, _, v in reqs]


def _alone(rle, torch, scene, cam, view):
    n = view.width * view.height
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    c = torch.empty(n, dtype=torch.int32, device="cuda")
    d = torch.empty(n, dtype=torch.float32, device="cuda")
    rle.render_frame(scene, cam, view, ws, ws_bytes, c, d)
    torch.cuda.synchronize()
    return c.cpu().numpy().view(np.uint32), d.cpu().numpy()


# batched: the slots' default launch shape (per-frame launches over worker
# streams); persistent: the slots' persistent pair; plain: one launch per request
MODES = {"batched": None, "persistent": (1, 32, 1, 128, 1, 0), "plain": None}


def _server(rle, mode, **kw):
    tun = MODES[mode]
    return rle.Server(plain=mode == "plain", batch_tuning=rle.BatchTuning(*tun) if tun else None, **kw)


@pytest.mark.parametrize("mode", list(MODES))
def test_served_results_equal_alone(rle, po, scene_pairs, torch_cuda, mode):
    torch = torch_cuda
    plain = mode == "plain"
    scenes = [s for s, _ in scene_pairs]
    srv = _server(rle, mode, hbm_budget_bytes=8 << 30, raybuf_words=8 << 20, max_frames_per_batch=8, max_inflight=3,
                  max_samples=640)
    ids = [srv.add_scene(s) for s in scenes]
    assert ids == [0, 1]
    reqs = _requests(rle, scenes, 24, 7)
    bufs = _buffers(torch, reqs)
    tickets = []
    for (sid, cam, view), (c, d) in zip(reqs, bufs):
        tickets.append(srv.submit(sid, cam, view, c, d))
    for t in tickets:
        assert srv.wait(t, 20000).status == 0
    srv.drain(20000)
    torch.cuda.synchronize()
    for i, ((sid, cam, view), (c, d)) in enumerate(zip(reqs, bufs)):
        wc, wd = _alone(rle, torch, scenes[sid], cam, view)
        gc, gd = c.cpu().numpy().view(np.uint32), d.cpu().numpy()
        assert np.array_equal(gc, wc), f"request {i} colour"
        assert np.array_equal(gd.view(np.uint32), wd.view(np.uint32)), f"request {i} depth"
        orc = oracle_screen(po, rle, scene_pairs[sid][1], cam, view, hits=False)
        assert_screen_equal((gc, gd, None), orc, f"request {i} (scene {sid}, {view.width}x{view.height}) vs oracle")
    st = srv.stats()
    assert st.completed == 24 and st.failed == 0
    assert st.p99_ms >= st.p50_ms > 0 and st.mrays_per_s > 0
    if plain:
        assert st.batches == 24
    else:
        assert st.batches < 24  # requests were batched
    done = srv.poll()
    assert sorted(c.ticket for c in done) == sorted(tickets)
    # every completion carries its launch's device time, within its host span
    for c in done:
        assert 0 < c.gpu_ms <= (c.done_s - c.submit_s) * 1e3 + 1.0
    srv.destroy()


def test_admission_limits(rle, scenes, torch_cuda):
    torch = torch_cuda
    with pytest.raises(rle.RLEError) as e:
        rle.Server(hbm_budget_bytes=1 << 20, raybuf_words=8 << 20)  # ray buffers alone exceed 1 MiB
    assert e.value.name == "RLE_ERR_NO_MEMORY"
    probe = rle.Server(hbm_budget_bytes=8 << 30, raybuf_words=4 << 20, max_frames_per_batch=4, max_inflight=2,
                       max_samples=640)
    buffers = probe.stats().device_bytes
    probe.destroy()
    small = scenes[1].info().device_bytes
    big = rle.Scene.from_bytes(rle.scenegen_rle4(rle.scenegen_default(512, 256, 512, 5)))
    big_bytes = big.info().device_bytes
    assert big_bytes > 1024
    srv = rle.Server(hbm_budget_bytes=buffers + small + big_bytes - 1, raybuf_words=4 << 20, max_frames_per_batch=4,
                     max_inflight=2, max_samples=640)
    srv.add_scene(scenes[1])
    with pytest.raises(rle.RLEError) as e:
        srv.add_scene(big)  # one byte over the budget
    assert e.value.name == "RLE_ERR_NO_MEMORY"
    assert srv.stats().device_bytes == buffers + small
    cam = rle.camera(10.5, 10.5, 200.0, 0.0, -20.0)
    c = torch.empty(1920 * 1080, dtype=torch.int32, device="cuda")
    d = torch.empty(1920 * 1080, dtype=torch.float32, device="cuda")
    with pytest.raises(rle.RLEError) as e:
        srv.submit(0, cam, rle.view_params(1920, 1080), c, d)  # 1920 samples > max_samples 640
    assert e.value.name == "RLE_ERR_CAPACITY"
    with pytest.raises(rle.RLEError):
        srv.submit(7, cam, rle.view_params(320, 240), c, d)  # unknown scene
    srv.destroy()
    # exactly at the budget the scene is admitted
    srv = rle.Server(hbm_budget_bytes=buffers + small + big_bytes, raybuf_words=4 << 20, max_frames_per_batch=4,
                     max_inflight=2, max_samples=640)
    srv.add_scene(scenes[1])
    assert srv.add_scene(big) == 1
    srv.destroy()
    big.free()


def test_cancel_timeout_and_injected_failures(rle, scenes, torch_cuda):
    torch = torch_cuda
    srv = rle.Server(hbm_budget_bytes=8 << 30, raybuf_words=8 << 20, max_frames_per_batch=4, max_inflight=2,
                     max_samples=640)
    srv.add_scene(scenes[0])
    reqs = [(0, cam, view) for _, cam, view in _requests(rle, scenes[:1], 10, 11)]
    bufs = _buffers(torch, reqs)
    srv.pause(True)
    tickets = [srv.submit(sid, cam, view, c, d) for (sid, cam, view), (c, d) in zip(reqs, bufs)]
    # nothing launches while paused: a bounded wait gives up
    with pytest.raises(rle.RLEError) as e:
        srv.wait(tickets[0], 30)
    assert e.value.name == "RLE_ERR_TIMEOUT"
    with pytest.raises(rle.RLEError) as e:
        srv.drain(10)
    assert e.value.name == "RLE_ERR_TIMEOUT"
    # queued requests can be cancelled
    assert srv.cancel(tickets[1]) == 0
    assert srv.cancel(tickets[1]) != 0  # not twice
    assert srv.wait(tickets[1], 100).status == -8  # RLE_ERR_CANCELLED
    # the first launch fails on the host; the rest are served
    srv.inject_launch_failures(1)
    srv.pause(False)
    statuses = [srv.wait(t, 20000).status for t in tickets]
    st = srv.stats()
    assert statuses[1] == -8
    failed = [s for s in statuses if s == -4]  # RLE_ERR_CUDA
    assert 1 <= len(failed) <= 4  # exactly the first batch
    assert statuses.count(0) == 10 - 1 - len(failed)
    assert st.failed == len(failed) and st.cancelled == 1
    # the server still works afterwards
    t = srv.submit(0, reqs[0][1], reqs[0][2], bufs[0][0], bufs[0][1])
    assert srv.wait(t, 20000).status == 0
    srv.destroy()


def test_concurrent_submitters(rle, po, scene_pairs, torch_cuda):
    """Four host threads submit and wait at once; every result equals the
    request rendered alone and the oracle's screen, and every ticket
    completes exactly once."""
    import threading
    torch = torch_cuda
    scenes = [s for s, _ in scene_pairs]
    srv = rle.Server(hbm_budget_bytes=8 << 30, raybuf_words=8 << 20, max_frames_per_batch=8, max_inflight=3,
                     max_samples=640)
    for s in scenes:
        srv.add_scene(s)
    reqs = _requests(rle, scenes, 32, 21)
    bufs = _buffers(torch, reqs)
    torch.cuda.synchronize()
    statuses = {}
    errors = []

    def worker(t):
        try:
            mine = list(range(t, len(reqs), 4))
            tickets = []
            for i in mine:
                sid, cam, view = reqs[i]
                tickets.append((i, srv.submit(sid, cam, view, bufs[i][0], bufs[i][1])))
            for i, tk in tickets:
                statuses[i] = srv.wait(tk, 20000).status
        except Exception as e:  # reported below, on the main thread
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join(60)
    assert not errors, errors
    assert sorted(statuses) == list(range(len(reqs))) and set(statuses.values()) == {0}
    srv.drain(20000)
    torch.cuda.synchronize()
    for i, ((sid, cam, view), (c, d)) in enumerate(zip(reqs, bufs)):
        wc, wd = _alone(rle, torch, scenes[sid], cam, view)
        gc, gd = c.cpu().numpy().view(np.uint32), d.cpu().numpy()
        assert np.array_equal(gc, wc), f"request {i} colour"
        assert np.array_equal(gd.view(np.uint32), wd.view(np.uint32)), f"request {i} depth"
        orc = oracle_screen(po, rle, scene_pairs[sid][1], cam, view, hits=False)
        assert_screen_equal((gc, gd, None), orc, f"request {i} vs oracle")
    st = srv.stats()
    assert st.submitted == 32 and st.completed == 32 and st.failed == 0
    srv.destroy()


SERVE_RES = [((256, 256), 0.4), ((640, 480), 0.3), ((1280, 720), 0.2), ((1920, 1080), 0.1)]


def _pow2_ceil(v):
    p = 1
    while p < v:
        p <<= 1
    return p


@pytest.mark.parametrize("mode", list(MODES))
def test_config4_mix_against_oracle(rle, po, torch_cuda, mode):
    """A config-4 served mix: two resident cave scenes of different sizes
    (1024^2 and 2048^2 x 256, seeds 3 and 4), 40 requests with the config's
    resolution law (256x256 .4, 640x480 .3, 1280x720 .2, 1920x1080 .1; every
    resolution at least once) and config-2 poses, submitted at once so that
    they batch; every served frame equals the oracle's screen and the
    request rendered alone."""
    torch = torch_cuda
    pairs = []
    for n, seed in ((1024, 3), (2048, 4)):
        data = rle.scenegen_rle4(rle.scenegen_default(n, 256, n, seed, caves=True))
        pairs.append((rle.Scene.from_bytes(data), po.OracleScene.from_rle4(data), n))
    plain = mode == "plain"
    srv = _server(rle, mode, hbm_budget_bytes=16 << 30, raybuf_words=32 << 20, max_frames_per_batch=16,
                  max_inflight=3, max_samples=2048)
    for s, _, _ in pairs:
        srv.add_scene(s)
    rng = np.random.default_rng(20261205)
    probs = np.array([p for _, p in SERVE_RES])
    reqs = []
    for i in range(40):
        sid = i % 2 if i < 8 else int(rng.integers(0, 2))
        w, h = SERVE_RES[i % 4][0] if i < 8 else SERVE_RES[int(rng.choice(4, p=probs))][0]
        _, osc, n = pairs[sid]
        t0, s0 = osc.levels[0][3], osc.levels[0][4]
        x, z = rng.uniform(0, n, 2)
        g = rle.ground_height(t0, s0, n, 256, int(x), int(z))
        cam = rle.camera(float(x), float(z), g + float(rng.uniform(10, 80)), float(rng.uniform(0, 360)),
                         float(rng.uniform(1, 30) * rng.choice([-1, 1])))
        reqs.append((sid, cam, rle.view_params(w, h, samples=_pow2_ceil(w))))
    bufs = _buffers(torch, reqs)
    tickets = [srv.submit(sid, cam, view, c, d) for (sid, cam, view), (c, d) in zip(reqs, bufs)]
    for t in tickets:
        assert srv.wait(t, 60000).status == 0
    srv.drain(60000)
    torch.cuda.synchronize()
    st = srv.stats()
    assert st.completed == 40 and st.failed == 0
    if not plain:
        assert st.batches < 40
    for i, ((sid, cam, view), (c, d)) in enumerate(zip(reqs, bufs)):
        gc, gd = c.cpu().numpy().view(np.uint32), d.cpu().numpy()
        label = f"request {i} (scene {sid}, {view.width}x{view.height}, {mode})"
        assert_screen_equal((gc, gd, None), oracle_screen(po, rle, pairs[sid][1], cam, view, hits=False),
                            label + " vs oracle")
        wc, wd = _alone(rle, torch, pairs[sid][0], cam, view)
        assert np.array_equal(gc, wc) and np.array_equal(gd.view(np.uint32), wd.view(np.uint32)), label
    srv.destroy()
    for s, _, _ in pairs:
        s.free()


def test_requests_complete_with_their_own_frame(rle, po, scene_pairs, torch_cuda):
    """Seven 256x256 requests and then a 1920x1080 one taken into one batch
    (the server paused while they queue): in the default per-frame mode
    each request completes with its own frame, so the small frames' device
    times (batch start -> end of the frame) are shorter than the large
    frame's, launched last, instead of all being the batch's; every result
    equals the request rendered alone."""
    torch = torch_cuda
    scene = scene_pairs[0][0]
    srv = rle.Server(hbm_budget_bytes=8 << 30, raybuf_words=32 << 20, max_frames_per_batch=8, max_inflight=1,
                     max_samples=2048)
    sid = srv.add_scene(scene)
    base = _requests(rle, [scene], 8, 33)
    reqs = [(sid, cam, rle.view_params(256, 256, mip_distance=64)) for _, cam, _ in base[:7]]
    reqs.append((sid, base[7][1], rle.view_params(1920, 1080, mip_distance=64)))
    bufs = _buffers(torch, reqs)
    torch.cuda.synchronize()
    srv.pause(True)
    tickets = [srv.submit(s, cam, view, c, d) for (s, cam, view), (c, d) in zip(reqs, bufs)]
    srv.pause(False)
    done = {t: srv.wait(t, 20000) for t in tickets}
    assert all(c.status == 0 for c in done.values())
    assert srv.stats().batches == 1
    small = [done[t].gpu_ms for t in tickets[:7]]
    big = done[tickets[7]].gpu_ms
    assert 0 < min(small) < big, (small, big)
    srv.drain(20000)
    torch.cuda.synchronize()
    for i, ((s, cam, view), (c, d)) in enumerate(zip(reqs, bufs)):
        wc, wd = _alone(rle, torch, scene, cam, view)
        assert np.array_equal(c.cpu().numpy().view(np.uint32), wc), f"request {i} colour"
        assert np.array_equal(d.cpu().numpy().view(np.uint32), wd.view(np.uint32)), f"request {i} depth"
    srv.destroy()
