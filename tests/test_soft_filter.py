"""Soft post-filter (bin/shader/soft.frag): the oracle's restatement on
synthetic frames (CPU), and the CUDA kernel against it on rendered frames
(GPU, bit for bit)."""
from __future__ import annotations

import numpy as np
import pytest

SKY = 0xFFFFCCB2


def _alpha(out):
    return (out >> 24) & 255


def test_oracle_uniform_frame_keeps_colour(po):
    W, H = 64, 48
    c = np.full(W * H, 0xFF336699, np.uint32)
    d = np.full(W * H, 300.0, np.float32)
    out = po.soft_filter(c, d, W, H)
    assert np.all((out & 0xFFFFFF) == 0x336699)
    # alpha is the frame buffer's 0.001/z term: depth16 300 -> z = 44/255/256 + 1/255
    assert len(np.unique(_alpha(out))) == 1


def test_oracle_sky_is_untouched(po):
    W, H = 40, 30
    c = np.full(W * H, SKY, np.uint32)
    d = np.full(W * H, np.inf, np.float32)
    out = po.soft_filter(c, d, W, H)
    assert np.all(out == (SKY & 0xFFFFFF))  # alpha 0: fragz of the sky is 0


def test_oracle_is_edge_aware(po):
    """Near pixels (large 1/z) blend only with near neighbours: a near red
    square over a far green ground keeps pure red inside; far pixels next to
    it may take red (their filter front is the square), never the reverse."""
    W, H = 96, 64
    c = np.full((H, W), 0xFF00FF00, np.uint32)
    d = np.full((H, W), 4000.0, np.float32)
    c[20:44, 30:60] = 0xFF0000FF
    d[20:44, 30:60] = 40.0
    out = po.soft_filter(c.ravel(), d.ravel(), W, H).reshape(H, W)
    inner = out[22:42, 32:58] & 0xFFFFFF
    assert np.all(inner == 0x0000FF)
    far = out[0:10, 0:10] & 0xFFFFFF
    assert np.all(far == 0x00FF00)


def test_invalid_arguments(rle):
    import ctypes as C
    lib = rle.library()
    assert lib.rle_soft_filter(None, None, 64, 48, None, None) == -1
    fake = C.c_void_p(256)  # never dereferenced: the sizes are refused first
    assert lib.rle_soft_filter(fake, fake, 4096, 48, C.c_void_p(512), None) == -1
    assert lib.rle_soft_filter(fake, fake, 64, 48, fake, None) == -1  # output aliases the input


@pytest.mark.gpu
@pytest.mark.parametrize("res", [(320, 240), (640, 480), (1280, 720), (1920, 1080)])
def test_kernel_equals_oracle_on_rendered_frames(rle, po, torch_cuda, res):
    torch = torch_cuda
    W, H = res
    scene = rle.Scene.generate_on_device(rle.scenegen_default(512, 256, 512, 9, caves=True))
    info = scene.info()
    table, words = scene.copy_level(0)
    view = rle.view_params(W, H, mip_distance=64)
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    colour = torch.empty(W * H, dtype=torch.int32, device="cuda")
    depth = torch.empty(W * H, dtype=torch.float32, device="cuda")
    out = torch.full((W * H,), 7, dtype=torch.int32, device="cuda")
    rng = np.random.default_rng(W)
    for _ in range(3):
        x, z = rng.uniform(0, 512, 2)
        g = rle.ground_height(table, words, 512, 256, int(x), int(z))
        cam = rle.camera(float(x), float(z), g + float(rng.uniform(3, 40)), float(rng.uniform(0, 360)),
                         float(rng.uniform(-25, 25)))
        rle.render_frame(scene, cam, view, ws, ws_bytes, colour, depth)
        rle.soft_filter(colour, depth, W, H, out)
        torch.cuda.synchronize()
        c = colour.cpu().numpy().view(np.uint32)
        d = depth.cpu().numpy()
        want = po.soft_filter(c, d, W, H)
        got = out.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} pixels differ"
        # the filter changes something on a real frame (edges and depth steps)
        assert np.count_nonzero((got & 0xFFFFFF) != (c & 0xFFFFFF)) > 0
    scene.free()


@pytest.mark.gpu
@pytest.mark.parametrize("res", [(1, 1), (7, 3), (33, 9), (100, 75), (2048, 17), (17, 2048), (257, 129)])
def test_kernel_equals_oracle_on_random_frames(rle, po, torch_cuda, res):
    """Frame sizes that are not multiples of the kernel's 32 x 8 tile (and
    smaller than its 12-pixel apron), the largest width and height, random
    colours and depths mixing finite values, sky (+inf), no data (0), NaN and
    negative depths."""
    torch = torch_cuda
    W, H = res
    rng = np.random.default_rng(W * 4099 + H)
    c = rng.integers(0, 1 << 32, W * H, dtype=np.uint64).astype(np.uint32)
    d = rng.uniform(1.0, 5000.0, W * H).astype(np.float32)
    kind = rng.integers(0, 10, W * H)
    d[kind == 0] = np.inf
    d[kind == 1] = 0.0
    d[kind == 2] = np.nan
    d[kind == 3] = -d[kind == 3]
    d[kind == 4] = rng.uniform(0.0, 2.0, int((kind == 4).sum())).astype(np.float32)
    colour = torch.from_numpy(c.view(np.int32)).cuda()
    depth = torch.from_numpy(d).cuda()
    out = torch.full((W * H,), 7, dtype=torch.int32, device="cuda")
    rle.soft_filter(colour, depth, W, H, out)
    torch.cuda.synchronize()
    want = po.soft_filter(c, d, W, H)
    got = out.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, want), f"{res}: {np.count_nonzero(got != want)} pixels differ"
