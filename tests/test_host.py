"""Host-side checks of the product library (no GPU needed).

- every entry point include/rle_gb300.h declares is exported by the built
  librle_gb300.so;
- the host ray map (rle_raymap_build) equals the oracle's restatement bit for
  bit over seeded poses, resolutions and fields of view, and the reference's
  own ray map where its host build exists;
- the synthetic-scene generator's column encoder and mip rule equal the
  oracle's (themselves pinned to the reference's RLE4::compress and
  Tree::get_mipmap);
- argument validation returns status codes instead of faulting.
"""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_exports_match_header(rle):
    header = (ROOT / "include" / "rle_gb300.h").read_text()
    declared = set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(rle_\w+)\s*\(", header, re.M))
    declared = {d for d in declared if not d.endswith("_t")}
    out = subprocess.run(["nm", "-D", "--defined-only", str(rle.api.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = sorted(declared - exported)
    assert not missing, f"declared but not exported: {missing}"
    assert len(declared) >= 18


def test_version_and_status_strings(rle):
    assert "sm_103a" in rle.version()
    lib = rle.library()
    assert lib.rle_status_string(-6) == b"RLE_ERR_CAPACITY"


POSES = [(0.3, 20.0), (-0.3, 300.0), (1.2, 45.0), (-1.2, 200.0), (0.05, 91.0), (1.5, 0.0), (-0.7, 270.0)]


@pytest.mark.parametrize("wh", [(640, 480), (1920, 1080), (1024, 768), (320, 240), (3840, 2160)])
@pytest.mark.parametrize("fov", [90.0, 75.0])
def test_raymap_matches_oracle(rle, po, wh, fov):
    rng = np.random.default_rng(hash(wh) % 1000 + int(fov))
    for pitch_rad, yaw in POSES:
        cam = rle.camera(float(rng.uniform(0, 2048)), float(rng.uniform(0, 2048)), float(rng.uniform(20, 250)),
                         yaw, -np.degrees(pitch_rad), fov_deg=fov)
        pm = rle.raymap_build(cam, rle.view_params(*wh))
        om = po.raymap_build(cam.pos, cam.rot, pm.border, pm.maxres, pm.fov_scale, pm.samples,
                             pm.mip_distance, pm.z_far)
        assert bytes(po.raymap_from_product(pm)) == bytes(om)
        assert pm.rays == min(pm.map_line_count, 4 * pm.maxres)
        if fov == 90.0 and po.ref_available():
            f = po.ref_raymap_fields(po.ref_raymap(cam.pos, cam.rot, pm.border, pm.maxres))
            assert list(f["res"]) == list(pm.res)
            assert np.array_equal(np.array(pm.p_no, np.float32).view(np.uint32), f["p_no"].view(np.uint32))
            assert np.array_equal(np.array(pm.to3d, np.float32).view(np.uint32), f["to3d"].view(np.uint32))


@pytest.mark.parametrize("caves", [False, True])
def test_scenegen_encoder_matches_oracle(rle, po, caves):
    p = rle.scenegen_default(64, 128, 32, 7, caves=caves)
    levels = po.parse_rle4(rle.scenegen_rle4(p))
    assert len(levels) == p.nummaps
    for m in range(p.nummaps):
        sx, sy, sz = p.sx >> m, p.sy >> m, p.sz >> m
        assert levels[m][:3] == (sx, sy, sz)
        bits, cols = rle.scenegen_dense(p, m)
        _, words = po.encode_mip(bits, sx, sy, sz, m, cols)
        assert np.array_equal(words, levels[m][3]), f"level {m}"
        if m + 1 < p.nummaps:
            nxt, _ = rle.scenegen_dense(p, m + 1)
            assert np.array_equal(po.mipmap(bits, sx, sy, sz), nxt)
        po.build_table(levels[m][3], sx, sz)  # walks cleanly


def test_scenegen_deterministic_and_seeded(rle):
    a = rle.scenegen_rle4(rle.scenegen_default(64, 64, 64, 3, caves=True))
    b = rle.scenegen_rle4(rle.scenegen_default(64, 64, 64, 3, caves=True))
    c = rle.scenegen_rle4(rle.scenegen_default(64, 64, 64, 4, caves=True))
    assert a == b and a != c


def test_cave_scene_runs_per_column(rle, po):
    """The cave generator targets a mean of about 8 runs per column at the
    2048^2 x 256 scale; a 256^2 crop of the same settings sits near it."""
    p = rle.scenegen_default(256, 256, 256, 2, caves=True)
    p.base_period = 256 // 4
    sx, sy, sz, words = po.parse_rle4(rle.scenegen_rle4(p))[0]
    runs = po.build_table(words, sx, sz)[1::2] & 0xFFFF
    assert 5.0 < runs.mean() < 12.0


def test_invalid_arguments_return_status(rle):
    with pytest.raises(rle.RLEError) as e:
        rle.raymap_build(rle.camera(0, 0, 10, 0, -10), rle.view_params(100, 200))  # taller than wide
    assert e.value.name == "RLE_ERR_INVALID_ARG"
    cam = rle.camera(0, 0, 10, 0, -10)
    cam.pos[0] = float("nan")
    with pytest.raises(rle.RLEError):
        rle.raymap_build(cam, rle.view_params(64, 48))
    cam = rle.camera(0, 0, 10, 0, -10, fov_deg=180.0)
    with pytest.raises(rle.RLEError):
        rle.raymap_build(cam, rle.view_params(64, 48))
    p = rle.ScenegenParams()
    with pytest.raises(rle.RLEError):
        rle.scenegen_rle4(p)
    lib = rle.library()
    assert lib.rle_render_rays(None, None, None, None, None, None, None) == -1
    assert lib.rle_render_rays_timed(None, None, None, None, None, None) == -1
    h = C.c_void_p()
    assert lib.rle_scene_load_memory(b"\x01\x00", 2, 0, C.byref(h)) == -3  # truncated header
    assert lib.rle_scene_load_file(b"/nonexistent.rle4", 0, C.byref(h)) == -2
    # device scene builders validate before any device work
    assert lib.rle_scenegen_device(C.byref(p), 0, C.byref(h)) == -1
    assert lib.rle_encode_device(None, None, 64, 64, 64, 4, 0, C.byref(h)) == -1  # no bits
    fake = C.c_void_p(16)  # never dereferenced: the sizes are refused first
    assert lib.rle_encode_device(fake, None, 48, 64, 64, 4, 0, C.byref(h)) == -1  # sx not a power of two
    assert lib.rle_encode_device(fake, None, 64, 2048, 64, 4, 0, C.byref(h)) == -1  # sy > 1024
    assert lib.rle_encode_device(fake, None, 8, 64, 64, 5, 0, C.byref(h)) == -1  # 8 >> 4 == 0
    # batch and server limits are checked before any device work
    assert lib.rle_batch_create(0, 0, 1 << 20, 1024, 0, C.byref(h)) == -1        # no frames
    assert lib.rle_batch_create(0, 4, 16, 1024, 0, C.byref(h)) == -1             # ray buffer < 32 words
    assert lib.rle_batch_create(0, 4, 1 << 20, 16385, 0, C.byref(h)) == -1       # samples beyond 16384
    assert lib.rle_batch_create(0, 65537, 1 << 20, 1024, 0, C.byref(h)) == -1    # too many frames
    cfg = rle.ServerConfig(0, 1 << 30, 8, 0, 1 << 20, 1024, 0)                   # no in-flight slot
    assert lib.rle_server_create(C.byref(cfg), C.byref(h)) == -1
    cfg = rle.ServerConfig(0, 1 << 30, 8, 17, 1 << 20, 1024, 0)                  # more than 16 slots
    assert lib.rle_server_create(C.byref(cfg), C.byref(h)) == -1
    cfg = rle.ServerConfig(0, 1 << 30, 8, 2, 1 << 20, 4, 0)                      # samples below 8
    assert lib.rle_server_create(C.byref(cfg), C.byref(h)) == -1
    assert lib.rle_server_create(None, C.byref(h)) == -1
    # the process-wide launch shape accepts only the built shapes
    with pytest.raises(rle.RLEError):
        rle.tuning_set(lanes_per_ray=12)
    with pytest.raises(rle.RLEError):
        rle.tuning_set(threads_per_block=48)
    with pytest.raises(rle.RLEError):
        rle.tuning_set(staging=4)
    assert rle.tuning_get() == (0, 0, 0, 0)


def test_malformed_rle4_rejected_before_upload(rle, po):
    """A column whose run headers claim more colours than it stores, or a
    level that is not level 0 halved, must be refused (RLE_ERR_FORMAT) on
    the host -- the raycast could otherwise read past the slab array."""
    p = rle.scenegen_default(16, 64, 16, 1)
    levels = po.parse_rle4(rle.scenegen_rle4(p))
    sx, sy, sz, w = levels[0]
    bad = w.copy()
    t = po.build_table(w, sx, sz)
    ofs = int(t[0])
    assert int(bad[ofs]) > 0
    bad[ofs + 2] |= 63 << 10  # first run claims 63 more voxels
    lib = rle.library()
    h = C.c_void_p()
    data = po.write_rle4([(sx, sy, sz, bad)] + levels[1:])
    assert lib.rle_scene_load_memory(data, len(data), 0, C.byref(h)) == -3
    wrong = po.write_rle4([levels[0], (sx, sy // 2, sz // 4, levels[1][3])])
    assert lib.rle_scene_load_memory(wrong, len(wrong), 0, C.byref(h)) == -3
