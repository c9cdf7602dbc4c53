"""Run under RLE_GB300_LIB=<librle_gb300_checked.so> by tests/test_gpu_bounds.py.

    python tests/bounds_probe.py clean    frames of valid scenes: no check fires,
                                          ray buffers equal the oracle's
    python tests/bounds_probe.py corrupt  a resident scene whose level-0 table
                                          points every column past the level's
                                          words (one visible run each): the
                                          colour check fires

Prints one line `RESULT <flags> <first index>`.  The corruption stays inside
the checked build's 64 KB zero padding, so even an unchecked read would stay
inside the scene's allocation."""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def main(mode: str) -> int:
    import torch
    from conftest import load_package
    from oracle import pyoracle as po
    rle = load_package()
    assert "checked" in str(rle.api.LIB_PATH), rle.api.LIB_PATH
    rle.bounds_check_read(0, clear=True)
    data = rle.scenegen_rle4(rle.scenegen_default(256, 256, 256, 5, caves=True))
    scene = rle.Scene.from_bytes(data)
    W, H = 320, 240
    view = rle.view_params(W, H, mip_distance=64)
    cam = rle.camera(100.5, 120.25, 170.0, 40.0, -12.0)
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    c = torch.empty(W * H, dtype=torch.int32, device="cuda")
    d = torch.empty(W * H, dtype=torch.float32, device="cuda")
    if mode == "clean":
        oscene = po.OracleScene.from_rle4(data)
        rm = rle.raymap_build(cam, view)
        words = rle.raybuf_words(rm)
        rb = torch.empty(words, dtype=torch.int32, device="cuda")
        rd = torch.empty(words, dtype=torch.float32, device="cuda")
        rh = torch.empty(words * 8, dtype=torch.uint8, device="cuda")
        rle.render_rays(scene, rm, rb, rd, rh, None)
        torch.cuda.synchronize()
        n = rm.rays * rm.samples
        out, dep, hits, _ = po.render_rays(po.raymap_from_product(rm), oscene, want_hits=True)
        assert np.array_equal(rb[:n].cpu().numpy().view(np.uint32), out)
        assert np.array_equal(rh[: n * 8].cpu().numpy().view(rle.HIT_DTYPE), hits)
        for yaw in range(0, 360, 45):
            rle.render_frame(scene, rle.camera(100.5, 120.25, 170.0, float(yaw), -12.0), view, ws, ws_bytes, c, d)
        b = rle.Batch(4, 4 * rle.raybuf_words(rm), 320)
        reqs = [rle.frame_request(rle.camera(60.5 + 20 * i, 90.0, 150.0, 10.0 * i, -8.0), view,
                                  torch.empty(W * H, dtype=torch.int32, device="cuda"),
                                  torch.empty(W * H, dtype=torch.float32, device="cuda")) for i in range(4)]
        b.render(scene, reqs)
        torch.cuda.synchronize()
        b.free()
    else:
        table, _, words = rle.debug_level_pointers(scene, 0)
        info = scene.info()
        cols = info.sx[0] * info.sz[0]
        # every column: offset words-2 (its headers start at the padding),
        # one run whose cached first header says 5 solid voxels after 100
        # empty ones (heights 151-155, just below the camera at 170, which
        # looks down onto them within the level-0 distance)
        bad = np.empty(2 * cols, np.uint32)
        bad[0::2] = words - 2
        bad[1::2] = 1 | (((5 << 10) | 100) << 16)
        src = torch.from_numpy(bad.view(np.int32)).cuda()
        torch.cuda.synchronize()
        rc = _cudart().cudaMemcpy(ctypes.c_void_p(table), ctypes.c_void_p(src.data_ptr()),
                                  ctypes.c_size_t(bad.nbytes), 3)  # device to device
        assert rc == 0, rc
        back, _ = scene.copy_level(0)
        assert np.array_equal(back, bad), "the corrupted table did not reach the device"
        rle.render_frame(scene, cam, view, ws, ws_bytes, c, d)
        torch.cuda.synchronize()
        col = c.cpu().numpy().view(np.uint32)
        print(f"black {int((col == 0xff000000).sum())} sky {int((col == 0xffffccb2).sum())} "
              f"nodata {int((col == 0).sum())} of {col.size}")
    flags, first = rle.bounds_check_read(0, clear=True)
    scene.free()
    print(f"RESULT {flags} {first}")
    return 0


def _cudart():
    """The toolkit's CUDA runtime (device pointers are shared through the
    device's primary context)."""
    import shutil
    nvcc = shutil.which("nvcc")
    home = Path(nvcc).resolve().parent.parent if nvcc else Path("/usr/local/cuda")
    for d in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        f = home / d / "libcudart.so"
        if f.exists():
            return ctypes.CDLL(str(f))
    raise RuntimeError("libcudart.so not found")


if __name__ == "__main__":
    sys.exit(main(sys.argv[1]))
