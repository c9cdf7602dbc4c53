"""Helpers for the GPU tests: device buffers and one-call renders through
the C ABI, returned as host numpy arrays."""
from __future__ import annotations

import numpy as np


class Frame:
    """Ray buffer, depth, hits and counters of one ray map, plus the resolve."""

    def __init__(self, torch, rle, scene, rm, hits: bool = True, counters: bool = True, stream: int = 0):
        words = rle.raybuf_words(rm)
        dev = "cuda"
        self.raybuf = torch.empty(words, dtype=torch.int32, device=dev)
        self.raydepth = torch.empty(words, dtype=torch.float32, device=dev)
        self.rayhit = torch.empty(words * 8, dtype=torch.uint8, device=dev) if hits else None
        self.counters = torch.zeros(6, dtype=torch.int64, device=dev) if counters else None
        rle.render_rays(scene, rm, self.raybuf, self.raydepth, self.rayhit, self.counters, stream=stream)
        self.rm = rm
        self.torch = torch
        self.rle = rle

    def rays_host(self):
        """(packed words, depth, hits, counters) of the cast rows only."""
        self.torch.cuda.synchronize()
        n = self.rm.rays * self.rm.samples
        words = self.raybuf[:n].cpu().numpy().view(np.uint32)
        depth = self.raydepth[:n].cpu().numpy()
        hits = self.rayhit[: n * 8].cpu().numpy().view(self.rle.HIT_DTYPE) if self.rayhit is not None else None
        cnt = self.counters.cpu().numpy() if self.counters is not None else None
        return words, depth, hits, cnt

    def resolve_host(self, hits: bool = True):
        torch = self.torch
        W, H = self.rm.width, self.rm.height
        colour = torch.empty(W * H, dtype=torch.int32, device="cuda")
        depth = torch.empty(W * H, dtype=torch.float32, device="cuda")
        hit = torch.empty(W * H * 8, dtype=torch.uint8, device="cuda") if hits else None
        self.rle.resolve(self.rm, self.raybuf, self.raydepth, colour, depth, self.rayhit if hits else None, hit)
        torch.cuda.synchronize()
        return (colour.cpu().numpy().view(np.uint32), depth.cpu().numpy(),
                hit.cpu().numpy().view(self.rle.HIT_DTYPE) if hit is not None else None)


def counters_dict(arr) -> dict:
    names = ("cells", "fetched", "headers", "runs", "spans", "pixels")
    return {n: int(v) for n, v in zip(names, arr)}


def oracle_counters(cnt) -> dict:
    return {n: int(cnt[n].sum()) for n in cnt.dtype.names}


def float_bits(a: np.ndarray) -> np.ndarray:
    """The bits of a float32 array with every NaN as 0x7fc00000.  A NaN's
    bit pattern is the platform's (x86 hosts give 0xffc00000, Arm hosts
    0x7fc00000, the GPU 0x7fffffff); a degenerate span (zero screen height,
    a camera inside the ground) makes NaN depths on every platform, so NaN
    must meet NaN at the same sample, and every other value bit for bit."""
    bits = a.view(np.uint32).copy()
    bits[np.isnan(a)] = 0x7FC00000
    return bits


def assert_rays_equal(gpu, orc, label=""):
    """Packed words and hits bit-exact; depth bit-exact too, NaN matching NaN
    (the stated bar is 1e-5 relative, the implementation meets it with zero
    error)."""
    gw, gd, gh, _ = gpu
    ow, od, oh, _ = orc
    assert gw.shape == ow.shape, label
    bad = int((gw != ow).sum())
    assert bad == 0, f"{label}: {bad} of {gw.size} ray-buffer words differ"
    dbad = int((float_bits(gd) != float_bits(od)).sum())
    assert dbad == 0, f"{label}: {dbad} depths differ"
    if gh is not None and oh is not None:
        assert np.array_equal(gh, oh), f"{label}: {int((gh != oh).sum())} hit records differ"


def oracle_screen(po, rle, oscene, cam, view, hits: bool = True, nthreads: int = 0):
    """The oracle's screen for one camera and view: the oracle's own ray map
    (built from the camera and the view's resolved sizes), the oracle's
    Render::render_line restatement and its resolve -- no product code on
    the path but the call that resolves the view's defaults (maxres,
    samples, distances), whose ray map must then equal the oracle's.
    Returns (colour u32, depth f32, hits or None)."""
    rm = rle.raymap_build(cam, view)
    om = po.raymap_build(list(cam.pos), list(cam.rot), rm.border, rm.maxres, rm.fov_scale, rm.samples,
                         rm.mip_distance, rm.z_far)
    assert list(om.res) == list(rm.res), "oracle and product ray maps disagree on the fan sizes"
    out, dep, hit, _ = po.render_rays(om, oscene, want_hits=hits, nthreads=nthreads)
    col, d, h, _ = po.resolve(om, view.width, view.height, out, dep, hit)
    return col, d, h


def assert_screen_equal(got, want, label=""):
    """Screen colour and hit records bit for bit; depth bit for bit with NaN
    meeting NaN (the stated bar for depth is 1e-5 relative; the renderer
    meets it with zero error)."""
    gc, gd, gh = got
    wc, wd, wh = want
    assert gc.shape == wc.shape, label
    bad = int((gc != wc).sum())
    assert bad == 0, f"{label}: {bad} of {gc.size} pixels differ from the oracle"
    dbad = int((float_bits(gd) != float_bits(wd)).sum())
    assert dbad == 0, f"{label}: {dbad} depths differ from the oracle"
    if gh is not None and wh is not None:
        hbad = int((gh != wh).sum())
        assert hbad == 0, f"{label}: {hbad} hit records differ from the oracle"
