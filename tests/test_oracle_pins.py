"""Pins the CPU oracle to the reference.

1. Against the golden fixtures (tests/golden/golden_v1.npz), which the
   reference's own host build generated: column tables, ray maps and full ray
   buffers must match bit for bit.  Runs everywhere.
2. Against the reference's host build itself (oracle/_ref/libref.so), on
   seeded random scenes and poses: encoder, mip rule, loader table, ray map
   and per-ray raycast.  Runs where that library was built.
"""
from __future__ import annotations

import tempfile
from pathlib import Path

import numpy as np
import pytest


def _golden_scene(po, golden):
    levels = po.parse_rle4(golden["scene_rle4"].tobytes())
    return levels, po.OracleScene(levels)


def test_golden_tables(po, golden):
    levels, _ = _golden_scene(po, golden)
    for m, (sx, sy, sz, words) in enumerate(levels):
        assert np.array_equal(po.build_table(words, sx, sz), golden[f"table_{m}"]), f"level {m}"


def _golden_raymap(po, golden, i):
    S, maxres, mipd, zfar = (int(v) for v in golden["params"])
    border = float(golden["border"][0])
    cam = golden[f"cam_{i}"]
    rm = po.raymap_build(cam[:3], cam[3:], border, maxres, 1.0, S, mipd, zfar)
    return rm


@pytest.mark.parametrize("i", range(6))
def test_golden_raymap(po, golden, i):
    rm = _golden_raymap(po, golden, i)
    f = po.ref_raymap_fields(golden[f"raymap_{i}"].tobytes())
    bits = lambda a: np.asarray(a, np.float32).view(np.uint32)  # noqa: E731
    assert list(rm.res) == list(f["res"])
    assert rm.map_line_count == f["map_line_count"]
    assert np.array_equal(bits([[v.x, v.y, v.z] for v in rm.p_2d]), bits(f["p_2d"]))
    assert np.array_equal(bits([[v.x, v.y, v.z] for v in rm.p_no]), bits(f["p_no"]))
    assert np.array_equal(bits(list(rm.to3d)), bits(f["to3d"]).ravel())
    assert np.array_equal(bits(list(rm.p_ofs_min) + list(rm.p_ofs_max)),
                          bits(np.concatenate([f["p_ofs_min"], f["p_ofs_max"]])))


@pytest.mark.parametrize("i", range(6))
def test_golden_raybuf(po, golden, i):
    _, scene = _golden_scene(po, golden)
    rm = _golden_raymap(po, golden, i)
    out, depth, hits, cnt = po.render_rays(rm, scene, want_hits=True, want_counters=True)
    ref = golden[f"raybuf_{i}"]
    # the reference leaves samples outside a ray's clip range untouched (0 in
    # a zeroed buffer); the oracle writes 0 there too
    assert out.shape == ref.shape
    assert np.array_equal(out, ref), f"{int((out != ref).sum())} of {out.size} samples differ"
    hit = out != 0
    assert ((hits["flags"] == 1) == (hit & (((out >> 16) & 0xFF) != 0xFF))).all()
    assert cnt["pixels"].sum() == int((hits["flags"] == 1).sum())


# ---------------------------------------------------------------------------
# against the reference's host build (where it exists)
# ---------------------------------------------------------------------------

def _ref_built() -> bool:
    from oracle import pyoracle
    return pyoracle.ref_available()


needs_ref = pytest.mark.skipif(not _ref_built(), reason="reference host build (oracle/_ref) not present")


def _random_volume(n, seed):
    rng = np.random.default_rng(seed)
    x = np.arange(n)[None, :]
    z = np.arange(n)[:, None]
    h = n * 0.4 + n * 0.2 * np.sin(x * 2 * np.pi / n * 2 + seed) * np.cos(z * 2 * np.pi / n * 3) \
        + rng.integers(0, 4, (n, n))
    j = np.arange(n)[None, :, None]
    vol = j >= (n - h[:, None, :])
    cave = (rng.random((n // 4, n // 4, n // 4)) < 0.15).repeat(4, 0).repeat(4, 1).repeat(4, 2)
    return vol & ~(cave & (j < n - 2))


@needs_ref
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_encoder_and_mips_match_reference(po, seed):
    n = 64
    bits = po.pack_bits(_random_volume(n, seed))
    for m in range(3):
        s_ref, w_ref = po.ref_compress(bits, n, n, n, m)
        s_orc, w_orc = po.encode_mip(bits, n, n, n, m)
        assert np.array_equal(s_ref, s_orc) and np.array_equal(w_ref, w_orc)
        nb_ref = po.ref_mipmap(bits, n, n, n)
        nb_orc = po.mipmap(bits, n, n, n)
        assert np.array_equal(nb_ref, nb_orc)
        bits, n = nb_orc, n // 2


@needs_ref
def test_long_runs_split_like_reference(po):
    """skip > 1023 and solid > 63 header splitting (src/Rle4.cpp:168-179)."""
    sx, sy, sz = 8, 2048, 8
    vol = np.zeros((sz, sy, sx), bool)
    vol[:, 1500:, :] = True           # skip of 1500 then a thick solid block
    vol[:, 200:330, 3] = True         # 130-voxel column-wide run
    vol[2, :, :] = True               # a full-height wall (all surface at the edge)
    bits = po.pack_bits(vol)
    s_ref, w_ref = po.ref_compress(bits, sx, sy, sz, 0)
    s_orc, w_orc = po.encode_mip(bits, sx, sy, sz, 0)
    assert np.array_equal(w_ref, w_orc) and np.array_equal(s_ref, s_orc)
    assert (w_orc == 1023).any() and ((w_orc >> 10) == 63).any()


@needs_ref
def test_loader_table_matches_reference(po):
    n = 32
    vol = _random_volume(n, 4)
    vol[:, :, 7] = False  # empty columns exercise the read past the column (src/Rle4.cpp:301)
    bits = [po.pack_bits(vol)]
    dims = [(n, n, n)]
    for _ in range(2):
        bits.append(po.mipmap(bits[-1], *dims[-1]))
        dims.append(tuple(d // 2 for d in dims[-1]))
    levels = [(*dims[m], po.encode_mip(bits[m], *dims[m], m)[1]) for m in range(3)]
    with tempfile.TemporaryDirectory() as td:
        p = Path(td) / "t.rle4"
        p.write_bytes(po.write_rle4(levels))
        for m in range(3):
            assert np.array_equal(po.ref_load_table(str(p), m, dims[m][0], dims[m][2]),
                                  po.build_table(levels[m][3], dims[m][0], dims[m][2]))


@needs_ref
def test_raymap_and_raycast_match_reference(po):
    n = 64
    vol = _random_volume(n, 9)
    bits = [po.pack_bits(vol)]
    dims = [(n, n, n)]
    for _ in range(3):
        bits.append(po.mipmap(bits[-1], *dims[-1]))
        dims.append(tuple(d // 2 for d in dims[-1]))
    levels = [(*dims[m], po.encode_mip(bits[m], *dims[m], m)[1]) for m in range(4)]
    scene = po.OracleScene(levels)
    rng = np.random.default_rng(21)
    S, maxres, border = 160, 160, 0.125
    total = diff = 0
    for _ in range(24):
        pos = (float(rng.uniform(0, n)), float(-rng.uniform(10, 40)), float(rng.uniform(0, n)))
        rot = (float(rng.choice([-1, 1]) * rng.uniform(0.05, 1.5)), float(rng.uniform(0, 6.3)), 0.0)
        rb = po.ref_raymap(pos, rot, border, maxres)
        f = po.ref_raymap_fields(rb)
        rm = po.raymap_build(pos, rot, border, maxres, 1.0, S, 40, 1200)
        assert list(rm.res) == list(f["res"])
        assert np.array_equal(np.array(list(rm.to3d), np.float32).view(np.uint32), f["to3d"].ravel().view(np.uint32))
        nr = po.rays_to_render(rm)
        ref = po.ref_render_rays(rb, scene, S, nr, 40, 1200)
        out, _, _, _ = po.render_rays(rm, scene)
        total += out.size
        diff += int((out != ref).sum())
    assert diff == 0, f"{diff} of {total} samples differ"


@needs_ref
@pytest.mark.parametrize("seed", [31, 32, 33])
def test_raycast_matches_reference_random(po, seed):
    """Wider random sweep against the reference's host build: grid 32-128,
    4 mip levels, eyes above the scene's top, inside it and under the
    ground, pitch up to +-89 degrees, ray-buffer rows of 64-256 samples
    (not only multiples of 32), random ray counts, borders, switch and far
    distances."""
    rng = np.random.default_rng(seed)
    n = int(rng.choice([32, 64, 128]))
    vol = _random_volume(n, seed)
    bits = [po.pack_bits(vol)]
    dims = [(n, n, n)]
    for _ in range(3):
        bits.append(po.mipmap(bits[-1], *dims[-1]))
        dims.append(tuple(d // 2 for d in dims[-1]))
    levels = [(*dims[m], po.encode_mip(bits[m], *dims[m], m)[1]) for m in range(4)]
    scene = po.OracleScene(levels)
    total = diff = 0
    for k in range(12):
        S = int(rng.choice([64, 100, 160, 256]))
        maxres = int(rng.integers(16, S + 1))
        border = float(rng.uniform(0.0, 0.3))
        mipd = int(rng.integers(16, 129))
        zfar = int(rng.integers(200, 3001))
        pos = (float(rng.uniform(-0.5 * n, 1.5 * n)), float(rng.uniform(-2.0 * n, 0.5 * n)),
               float(rng.uniform(-0.5 * n, 1.5 * n)))
        rot = (float(rng.choice([-1, 1]) * rng.uniform(0.02, 1.55)), float(rng.uniform(0, 6.3)), 0.0)
        rb = po.ref_raymap(pos, rot, border, maxres)
        rm = po.raymap_build(pos, rot, border, maxres, 1.0, S, mipd, zfar)
        assert list(rm.res) == list(po.ref_raymap_fields(rb)["res"]), f"pose {k}"
        nr = po.rays_to_render(rm)
        ref = po.ref_render_rays(rb, scene, S, nr, mipd, zfar)
        out, _, _, _ = po.render_rays(rm, scene)
        total += out.size
        diff += int((out != ref).sum())
    assert total > 0
    assert diff == 0, f"{diff} of {total} samples differ"


# ---------------------------------------------------------------------------
# at the benchmark's sizes: the 2048^2 cave scene, 1080p and 4K frames
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def cave2048(po):
    """The 2048^2 x 256 cave scene (seed 2) of the plain-frame benchmark,
    made by the library's host generator."""
    from conftest import ensure_built, load_package
    ensure_built()
    rle = load_package()
    data = rle.scenegen_rle4(rle.scenegen_default(2048, 256, 2048, 2, caves=True))
    return rle, po.OracleScene.from_rle4(data)


def _bench_poses(rle, oscene, count, seed, lo, hi, fov=90.0):
    """Cameras by the benchmark's law: uniform over the grid, lo-hi voxels
    above the local ground, yaw U[0,360), pitch +-U[1,30]."""
    sx, sy = oscene.levels[0][0], oscene.levels[0][1]
    t0, s0 = oscene.levels[0][3], oscene.levels[0][4]
    rng = np.random.default_rng(seed)
    cams = []
    for _ in range(count):
        x, z = rng.uniform(0, sx), rng.uniform(0, sx)
        g = rle.ground_height(t0, s0, sx, sy, int(x), int(z))
        pitch = float(rng.uniform(1.0, 30.0) * rng.choice([-1.0, 1.0]))
        cams.append(rle.camera(float(x), float(z), g + float(rng.uniform(lo, hi)), float(rng.uniform(0, 360)),
                               pitch, fov, scene_height=sy))
    return cams


def _pin_frame(po, rle, oscene, cam, view, label):
    rm = rle.raymap_build(cam, view)
    om = po.raymap_build(list(cam.pos), list(cam.rot), rm.border, rm.maxres, 1.0, rm.samples, rm.mip_distance,
                         rm.z_far)
    rb = po.ref_raymap(list(cam.pos), list(cam.rot), rm.border, rm.maxres)
    f = po.ref_raymap_fields(rb)
    assert list(om.res) == list(f["res"]), label
    assert np.array_equal(np.array(list(om.to3d), np.float32).view(np.uint32), f["to3d"].ravel().view(np.uint32))
    nr = po.rays_to_render(om)
    ref = po.ref_render_rays(rb, oscene, rm.samples, nr, rm.mip_distance, rm.z_far)
    out, _, _, _ = po.render_rays(om, oscene)
    assert out.size == nr * rm.samples and nr > 1000, label
    diff = int((out != ref).sum())
    assert diff == 0, f"{label}: {diff} of {out.size} samples differ from the reference"
    # the frame reaches the sizes it is here for: samples in mask word 31 and
    # beyond (y >= 992) drawn, long rows
    drawn = (out.reshape(nr, rm.samples) != 0) & (((out.reshape(nr, rm.samples) >> 16) & 0xFF) != 0xFF)
    assert drawn[:, 992:].any(), label


@needs_ref
@pytest.mark.parametrize("k", range(3))
def test_config2_frames_match_reference(po, cave2048, k):
    """Three poses of the benchmark's camera path (seed 20261203) on its
    2048^2 cave scene at 1920x1080, 2048 samples per column ray: the
    oracle's ray buffer equals the reference's Render::render_line build."""
    rle, oscene = cave2048
    cam = _bench_poses(rle, oscene, 3, 20261203, 10, 80)[k]
    _pin_frame(po, rle, oscene, cam, rle.view_params(1920, 1080, samples=2048), f"config-2 pose {k}")


@needs_ref
@pytest.mark.parametrize("k", range(2))
def test_4k_frames_match_reference(po, cave2048, k):
    """3840x2160 frames, 4096 samples per column ray, level switches at
    256/512/1024 voxels (the 4K benchmark's LOD law), cameras 20-200 above
    the ground, on the 2048^2 cave scene (its slabs fit the harness's
    below-4-GiB placement); 90 degrees, the reference's fixed frustum."""
    rle, oscene = cave2048
    cam = _bench_poses(rle, oscene, 2, 7, 20, 200)[k]
    _pin_frame(po, rle, oscene, cam, rle.view_params(3840, 2160, samples=4096, mip_distance=256),
               f"4K pose {k}")
