"""Scene building on the GPU (rle_scenegen_device, rle_encode_device).

- the device generator equals the host generator + loader bit for bit:
  every level's column table and slab words, the scene statistics, and the
  frames rendered from the two scenes;
- the device encoder equals the oracle's restatement of RLE4::compress_all
  (Tree::get_mipmap + RLE4::compress + RLE4::load's table) on volumes with
  odd heights, both colour modes (caller colours, the reference's
  normal-derived word).
Argument errors (refused before any device work) are covered on the CPU in
test_host.py.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GEN_CASES = [
    # sx, sy, sz, seed, caves, nummaps
    (64, 64, 64, 1, False, 4),
    (128, 256, 128, 4, True, 4),
    (256, 512, 128, 7, True, 4),
    (256, 256, 64, 3, True, 4),
    (64, 64, 64, 9, True, 7),
    (1024, 256, 1024, 5, True, 4),
]


def _levels(rle, scene):
    info = scene.info()
    out = []
    for m in range(info.nummaps):
        t, w = scene.copy_level(m)
        out.append((info.sx[m], info.sy[m], info.sz[m], t, w))
    return info, out


@pytest.mark.parametrize("case", GEN_CASES, ids=lambda c: "x".join(map(str, c[:3])) + f"-s{c[3]}-c{int(c[4])}-m{c[5]}")
def test_device_generator_equals_host(rle, torch_cuda, case):
    sx, sy, sz, seed, caves, nummaps = case
    p = rle.scenegen_default(sx, sy, sz, seed, caves=caves)
    p.nummaps = nummaps
    host = rle.Scene.from_bytes(rle.scenegen_rle4(p))
    dev = rle.Scene.generate_on_device(p)
    hi, hl = _levels(rle, host)
    di, dl = _levels(rle, dev)
    assert di.nummaps == hi.nummaps == nummaps
    for m, (a, b) in enumerate(zip(hl, dl)):
        assert a[:3] == b[:3], f"level {m} size"
        assert np.array_equal(a[3], b[3]), f"level {m} table"
        assert np.array_equal(a[4], b[4]), f"level {m} slab words"
    assert di.device_bytes == hi.device_bytes
    assert di.run_headers == hi.run_headers and di.surface_voxels == hi.surface_voxels
    assert list(di.slab_words) == list(hi.slab_words)
    # frames from both scenes are identical (this also covers the scene's
    # top index, which the early ray termination reads)
    torch = torch_cuda
    view = rle.view_params(320, 240, mip_distance=64)
    ws_bytes = rle.frame_workspace_bytes(view)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    rng = np.random.default_rng(seed)
    t0, w0 = hl[0][3], hl[0][4]
    for _ in range(3):
        x, z = rng.uniform(0, sx), rng.uniform(0, sz)
        g = rle.ground_height(t0, w0, sx, sy, int(x), int(z))
        cam = rle.camera(float(x), float(z), g + float(rng.uniform(5, 40)), float(rng.uniform(0, 360)),
                         float(rng.uniform(-25, 25)), scene_height=sy)
        outs = []
        for sc in (host, dev):
            c = torch.empty(320 * 240, dtype=torch.int32, device="cuda")
            d = torch.empty(320 * 240, dtype=torch.float32, device="cuda")
            rle.render_frame(sc, cam, view, ws, ws_bytes, c, d)
            outs.append((c.cpu().numpy(), d.cpu().numpy().view(np.uint32)))
        assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    host.free()
    dev.free()


def _oracle_levels(po, bits, colours, sx, sy, sz, nummaps):
    """Oracle chain: Tree::get_mipmap, RLE4::compress, RLE4::load's table.
    Level m takes the colour of the level-0 voxel at its lowest corner."""
    sx0, sy0 = sx, sy
    out = []
    b = bits
    for m in range(nummaps):
        if m:
            b = po.mipmap(b, sx, sy, sz)
            sx, sy, sz = sx // 2, sy // 2, sz // 2
        col_m = None
        if colours is not None:
            i = np.arange(sx) << m
            j = np.arange(sy) << m
            k = np.arange(sz) << m
            idx = (k[:, None, None] * sx0 * sy0 + j[None, :, None] * sx0 + i[None, None, :]).ravel()
            col_m = np.ascontiguousarray(colours[idx])
        _, words = po.encode_mip(b, sx, sy, sz, m, col_m)
        out.append((sx, sy, sz, po.build_table(words, sx, sz), words))
    return out


def _blob_volume(sx, sy, sz, seed):
    """Smooth random solid volume [z, y, x] with overhangs and a ground."""
    rng = np.random.default_rng(seed)
    coarse = rng.random((sz // 8 + 2, sy // 4 + 2, sx // 8 + 2))
    z = np.linspace(0, coarse.shape[0] - 1.001, sz)
    y = np.linspace(0, coarse.shape[1] - 1.001, sy)
    x = np.linspace(0, coarse.shape[2] - 1.001, sx)
    zi, yi, xi = z.astype(int), y.astype(int), x.astype(int)
    f = coarse[zi][:, yi][:, :, xi]
    depth = (np.arange(sy) / sy)[None, :, None]  # j grows downwards
    return (f * 0.6 + depth * 0.8) > 0.75


@pytest.mark.parametrize("with_colours", [False, True])
@pytest.mark.parametrize("dims", [(64, 40, 128), (128, 100, 64), (64, 64, 64)])
def test_device_encoder_equals_oracle(rle, po, torch_cuda, dims, with_colours):
    torch = torch_cuda
    sx, sy, sz = dims
    vol = _blob_volume(sx, sy, sz, sx + sy + sz)
    bits = po.pack_bits(vol)
    colours = None
    if with_colours:
        colours = np.random.default_rng(5).integers(0, 65536, sx * sy * sz, dtype=np.uint16)
    want = _oracle_levels(po, bits, colours, sx, sy, sz, 4)
    d_bits = torch.from_numpy(bits).cuda()
    d_col = torch.from_numpy(colours.view(np.int16)).cuda() if colours is not None else None
    scene = rle.Scene.encode_on_device(d_bits, d_col, sx, sy, sz, 4)
    info, got = _levels(rle, scene)
    for m, (a, b) in enumerate(zip(want, got)):
        assert a[:3] == b[:3], f"level {m} size"
        assert np.array_equal(a[4], b[4]), f"level {m} slab words"
        assert np.array_equal(a[3], b[3]), f"level {m} table"
    scene.free()


def test_device_encoder_matches_generator_volume(rle, po, torch_cuda):
    """The generator's dense level 0 (bits + colours) encoded on the device
    gives the generator's own scene (its mips take corner colours too)."""
    torch = torch_cuda
    p = rle.scenegen_default(64, 128, 64, 11, caves=True)
    bits, colours = rle.scenegen_dense(p, 0)
    scene = rle.Scene.encode_on_device(torch.from_numpy(bits).cuda(), torch.from_numpy(colours.view(np.int16)).cuda(),
                                       64, 128, 64, 4)
    ref = rle.Scene.from_bytes(rle.scenegen_rle4(p))
    _, got = _levels(rle, scene)
    _, want = _levels(rle, ref)
    for m in range(4):
        assert np.array_equal(got[m][3], want[m][3]) and np.array_equal(got[m][4], want[m][4]), f"level {m}"
    scene.free()
    ref.free()


def _random_volume_kind(rng, sx, sy, sz, kind):
    """Volumes [z, y, x] of several kinds: noise of a random density, thin
    horizontal layers (many runs per column), a single voxel, empty, full,
    and the smooth blobs."""
    if kind == "noise":
        return rng.random((sz, sy, sx)) < rng.uniform(0.05, 0.95)
    if kind == "layers":
        rows = rng.random(sy) < 0.5
        return np.broadcast_to(rows[None, :, None], (sz, sy, sx)).copy()
    if kind == "voxel":
        v = np.zeros((sz, sy, sx), bool)
        v[rng.integers(0, sz), rng.integers(0, sy), rng.integers(0, sx)] = True
        return v
    if kind == "empty":
        return np.zeros((sz, sy, sx), bool)
    if kind == "full":
        return np.ones((sz, sy, sx), bool)
    return _blob_volume(sx, sy, sz, int(rng.integers(0, 1 << 20)))


@pytest.mark.parametrize("case", range(12))
def test_device_encoder_random_volumes(rle, po, torch_cuda, case):
    """Random grids (x, z powers of two 8-128, heights 1-1024 -- runs longer
    than a 6-bit solid count or a 10-bit skip split as the reference splits
    them --, up to 4 levels) and volume kinds, with or without colours:
    every level's slab words and column table equal the oracle's."""
    torch = torch_cuda
    rng = np.random.default_rng(500 + case)
    sx, sz = (int(rng.choice([8, 16, 32, 64, 128])) for _ in range(2))
    sy = int(rng.choice([1, 7, 64, 100, 257, 1024]))
    kind = ["noise", "layers", "voxel", "empty", "full", "blobs"][case % 6]
    if kind in ("voxel", "full") and case >= 6:
        sy = 1024  # the longest skip (1023) and 16 solid runs per column
    nummaps = int(rng.integers(1, 5))
    # levels keep x and z at 8 or more (the Tree layout packs 8 voxels of x
    # per byte) and at least one voxel of height
    while nummaps > 1 and (min(sx, sz) >> (nummaps - 1) < 8 or sy >> (nummaps - 1) < 1):
        nummaps -= 1
    vol = _random_volume_kind(rng, sx, sy, sz, kind)
    bits = po.pack_bits(vol)
    colours = rng.integers(0, 65536, sx * sy * sz, dtype=np.uint16) if case % 2 else None
    want = _oracle_levels(po, bits, colours, sx, sy, sz, nummaps)
    d_bits = torch.from_numpy(bits).cuda()
    d_col = torch.from_numpy(colours.view(np.int16)).cuda() if colours is not None else None
    scene = rle.Scene.encode_on_device(d_bits, d_col, sx, sy, sz, nummaps)
    _, got = _levels(rle, scene)
    label = f"case {case}: {sx}x{sy}x{sz} {kind} levels {nummaps} colours {colours is not None}"
    assert len(got) == len(want), label
    for m, (a, b) in enumerate(zip(want, got)):
        assert a[:3] == b[:3], f"{label}: level {m} size"
        assert np.array_equal(a[4], b[4]), f"{label}: level {m} slab words"
        assert np.array_equal(a[3], b[3]), f"{label}: level {m} table"
    scene.free()
