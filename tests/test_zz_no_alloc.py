"""The allocation-free frame entry point (rle_render_frame_noalloc).

It serves callers that may not allocate device memory while they run -- a
render loop with a hard frame budget, or a plug-in whose host application
owns the GPU memory -- by keeping the ray buffer in a fixed array built into
the library.  Its pictures must equal rle_render_frame's (bit for bit, the
tolerance these tests use everywhere), on consecutive calls that reuse the
same array, and frames too large for the array must be refused cleanly.

Kept in a file that sorts last so a failure here comes after every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(rle, torch_cuda):
    data = rle.scenegen_rle4(rle.scenegen_default(256, 256, 256, 9, caves=True))
    s = rle.Scene.from_bytes(data)
    yield s
    s.free()


def _with_workspace(rle, torch, scene, cam, view):
    n = view.width * view.height
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    colour = torch.empty(n, dtype=torch.int32, device="cuda")
    depth = torch.empty(n, dtype=torch.float32, device="cuda")
    rle.render_frame(scene, cam, view, ws, ws_bytes, colour, depth)
    torch.cuda.synchronize()
    return colour.cpu().numpy().view(np.uint32), depth.cpu().numpy()


def _noalloc_c_abi(rle, torch, scene, cam, view):
    """Through the C entry point itself (ctypes), not the Python wrapper."""
    n = view.width * view.height
    colour = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    depth = torch.full((n,), 7.0, dtype=torch.float32, device="cuda")
    lib = rle.library()
    st = lib.rle_render_frame_noalloc(scene.handle, C.byref(cam), C.byref(view), colour.data_ptr(),
                                      depth.data_ptr(), None)
    assert st == 0, lib.rle_last_error()
    torch.cuda.synchronize()
    return colour.cpu().numpy().view(np.uint32), depth.cpu().numpy()


def test_noalloc_matches_workspace_frames(rle, scene, torch_cuda):
    torch = torch_cuda
    info = scene.info()
    table, words = scene.copy_level(0)
    view = rle.view_params(640, 480)
    cams = []
    for x, z, yaw, pitch in ((60.5, 200.25, 35.0, -12.0), (180.75, 40.5, 250.0, -40.0)):
        g = rle.ground_height(table, words, info.sx[0], info.sy[0], int(x), int(z))
        cams.append(rle.camera(x, z, g + 30.0, yaw, pitch))
    # two calls in a row share the built-in ray buffer
    for cam in cams:
        want_c, want_d = _with_workspace(rle, torch, scene, cam, view)
        got_c, got_d = _noalloc_c_abi(rle, torch, scene, cam, view)
        assert np.array_equal(got_c, want_c), f"{int((got_c != want_c).sum())} pixels differ"
        assert np.array_equal(got_d.view(np.uint32), want_d.view(np.uint32))
        assert (got_c != 0xFFFFCCB2).mean() > 0.2  # terrain is in view


def test_noalloc_refuses_frames_beyond_its_buffer(rle, scene, torch_cuda):
    torch = torch_cuda
    limit = rle.render_frame_noalloc_limit()
    assert limit == 64 << 20
    # 8 x rays x samples bytes: a 4096-wide frame looking down casts far more
    view = rle.view_params(4096, 2160)
    cam = rle.camera(100.5, 100.5, 250.0, 10.0, -70.0)
    rm = rle.raymap_build(cam, view)
    assert 8 * rm.rays * rm.samples > limit
    colour = torch.empty(4096 * 2160, dtype=torch.int32, device="cuda")
    depth = torch.empty(4096 * 2160, dtype=torch.float32, device="cuda")
    with pytest.raises(rle.RLEError) as e:
        rle.render_frame_noalloc(scene, cam, view, colour, depth)
    assert e.value.name == "RLE_ERR_CAPACITY"


def test_noalloc_calls_after_the_first_allocate_nothing(rle, scene, torch_cuda):
    """The property the entry point exists for: once the first call on the
    device has reserved the built-in array (and loaded the kernels), further
    calls leave the device's free memory exactly as it was -- no cudaMalloc,
    no allocating library routine -- and their pictures still equal
    rle_render_frame's."""
    torch = torch_cuda
    info = scene.info()
    table, words = scene.copy_level(0)
    view = rle.view_params(480, 270)
    g = rle.ground_height(table, words, info.sx[0], info.sy[0], 120, 130)
    cam = rle.camera(120.5, 130.5, g + 25.0, 140.0, -18.0)
    want_c, want_d = _with_workspace(rle, torch, scene, cam, view)
    n = view.width * view.height
    colour = torch.empty(n, dtype=torch.int32, device="cuda")
    depth = torch.empty(n, dtype=torch.float32, device="cuda")
    lib = rle.library()
    call = lambda: lib.rle_render_frame_noalloc(scene.handle, C.byref(cam), C.byref(view),  # noqa: E731
                                                colour.data_ptr(), depth.data_ptr(), None)
    assert call() == 0, lib.rle_last_error()  # the first call may reserve the array
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        assert call() == 0, lib.rle_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert np.array_equal(colour.cpu().numpy().view(np.uint32), want_c)
    assert np.array_equal(depth.cpu().numpy().view(np.uint32), want_d.view(np.uint32))
