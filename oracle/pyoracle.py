"""ctypes binding of the CPU oracle (oracle/liboracle.so) and of the
reference's own host build (oracle/_ref/libref.so, present only where the
reference checkout was available to build it).

Test infrastructure: imported by tests/, the smoke check and the CPU-baseline
leg of bench.py only.  See rle_oracle.h for what each function restates.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path
from typing import Optional

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref.so"
# The reference checkout is located by the recipe in ref/Makefile: the
# RLE_REF_SRC environment variable, else the recipe's default location.
REF_RECIPE = HERE / "ref"


def _foreign(path: Path) -> bool:
    """True if `path` is an ELF file for another CPU than this host's."""
    import platform
    import struct
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    try:
        head = path.read_bytes()[:20]
    except OSError:
        return False
    return (want is not None and len(head) == 20 and head[:4] == b"\x7fELF"
            and struct.unpack_from("<H", head, 18)[0] != want)


def build_oracle(force: bool = False) -> Path:
    """Compile rle_oracle.c (gcc, -ffp-contract=off, OpenMP)."""
    src = HERE / "rle_oracle.c"
    if force or not ORACLE_LIB.exists() or _foreign(ORACLE_LIB) or ORACLE_LIB.stat().st_mtime < max(
            src.stat().st_mtime, (HERE / "rle_oracle.h").stat().st_mtime):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        subprocess.run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
                        "-shared", "-o", str(tmp), str(src), "-lm"], check=True)
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def ref_checkout_present() -> bool:
    """Whether the recipe finds the reference checkout (RLE_REF_SRC or its
    default location)."""
    try:
        r = subprocess.run(["make", "-s", "-C", str(REF_RECIPE), "check-ref"], stdout=subprocess.DEVNULL,
                           stderr=subprocess.DEVNULL)
    except OSError:  # no make on this host
        return False
    return r.returncode == 0


def build_ref() -> Optional[Path]:
    """Compile the reference's host sources where the checkout exists (see
    ref/Makefile); elsewhere return the library built earlier, or None (the
    tests that need it then skip, saying so)."""
    if not ref_checkout_present():
        return REF_LIB if REF_LIB.exists() and not _foreign(REF_LIB) else None
    subprocess.run(["make", "-s", "-C", str(REF_RECIPE)], check=True, stdout=subprocess.DEVNULL)
    return REF_LIB


class V3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class OrcRayMap(C.Structure):
    _fields_ = [("vanishing_point_2d", V3), ("map_line_count", C.c_int), ("rotation", V3), ("position", V3),
                ("border", C.c_float), ("clip_min", C.c_float), ("clip_max", C.c_float), ("maxres", C.c_int),
                ("res", C.c_int * 4), ("p4", V3), ("p_2d", V3 * 8), ("p_no", V3 * 8), ("to3d", C.c_float * 16),
                ("p_ofs_min", C.c_float * 4), ("p_ofs_max", C.c_float * 4), ("samples", C.c_int),
                ("mip_distance", C.c_int), ("z_far", C.c_int), ("fov_scale", C.c_float)]


class OrcMip(C.Structure):
    _fields_ = [("sx", C.c_int), ("sy", C.c_int), ("sz", C.c_int), ("table", C.c_void_p), ("slabs", C.c_void_p),
                ("slabs_words", C.c_longlong)]


COUNTER_FIELDS = ("cells", "fetched", "headers", "runs", "spans", "pixels")
COUNTERS_DTYPE = np.dtype([(n, "<i8") for n in COUNTER_FIELDS])
HIT_DTYPE = np.dtype([("x", "<u2"), ("z", "<u2"), ("y", "<u2"), ("mip", "u1"), ("flags", "u1")])

_orc: Optional[C.CDLL] = None
_ref: Optional[C.CDLL] = None


def oracle() -> C.CDLL:
    global _orc
    if _orc is None:
        lib = C.CDLL(str(build_oracle()))
        lib.orc_encode_mip.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                       C.POINTER(C.POINTER(C.c_uint16)), C.POINTER(C.c_longlong)]
        lib.orc_mipmap.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        lib.orc_build_table.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_void_p]
        lib.orc_raymap_build.argtypes = [C.POINTER(OrcRayMap)] + [C.c_float] * 7 + [C.c_int, C.c_float, C.c_int,
                                                                                      C.c_int, C.c_int]
        lib.orc_render_rays.argtypes = [C.POINTER(OrcRayMap), C.POINTER(OrcMip), C.c_int, C.c_int, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        lib.orc_resolve.argtypes = [C.POINTER(OrcRayMap), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.orc_raybuf_rows.argtypes = [C.POINTER(OrcRayMap)]
        lib.orc_soft_filter.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        lib.orc_soft_filter.restype = None
        lib.orc_rays_to_render.argtypes = [C.POINTER(OrcRayMap)]
        _orc = lib
    return _orc


def ref_available() -> bool:
    return REF_LIB.exists() and not _foreign(REF_LIB)


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise FileNotFoundError("oracle/_ref/libref.so not built: it needs the reference checkout "
                                    "(set RLE_REF_SRC to its RLE-Raycaster folder and run build_ref())")
        lib = C.CDLL(str(REF_LIB))
        lib.ref_get_ray_map.argtypes = [C.c_float] * 7 + [C.c_int, C.c_void_p]
        lib.ref_render_rays.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                        C.c_int]
        lib.ref_compress.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                     C.POINTER(C.POINTER(C.c_uint16)), C.POINTER(C.c_longlong)]
        lib.ref_mipmap.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        lib.ref_load_table.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.c_void_p]
        lib.ref_free.argtypes = [C.c_void_p]
        _ref = lib
    return _ref


# ---------------------------------------------------------------------------
# scene format
# ---------------------------------------------------------------------------

def pack_bits(vol: np.ndarray) -> np.ndarray:
    """Boolean volume indexed [z, y, x] -> the reference's Tree bit layout."""
    return np.packbits(vol.astype(np.uint8), axis=-1, bitorder="little").ravel()


def encode_mip(bits: np.ndarray, sx: int, sy: int, sz: int, mip: int,
               colours: Optional[np.ndarray] = None) -> tuple[np.ndarray, np.ndarray]:
    starts = np.zeros(sx * sz, np.uint32)
    p = C.POINTER(C.c_uint16)()
    n = C.c_longlong()
    oracle().orc_encode_mip(bits.ctypes.data, None if colours is None else colours.ctypes.data, sx, sy, sz, mip,
                            starts.ctypes.data, C.byref(p), C.byref(n))
    words = np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0, np.uint16)
    C.CDLL(None).free(p)
    return starts, words


def mipmap(bits: np.ndarray, sx: int, sy: int, sz: int) -> np.ndarray:
    out = np.zeros((sx // 2 // 8) * (sy // 2) * (sz // 2), np.uint8)
    oracle().orc_mipmap(bits.ctypes.data, sx, sy, sz, out.ctypes.data)
    return out


def build_table(words: np.ndarray, sx: int, sz: int) -> np.ndarray:
    table = np.zeros(2 * sx * sz, np.uint32)
    rc = oracle().orc_build_table(words.ctypes.data, len(words), sx, sz, table.ctypes.data)
    if rc != 0:
        raise ValueError("column walk left the slab array")
    return table


def parse_rle4(data: bytes) -> list[tuple[int, int, int, np.ndarray]]:
    """.rle4 bytes -> [(sx, sy, sz, words)] per level."""
    n = int(np.frombuffer(data, "<i4", 1, 0)[0])
    ofs = 4
    levels = []
    for _ in range(n):
        sx, sy, sz, cnt = (int(v) for v in np.frombuffer(data, "<u4", 4, ofs))
        ofs += 16
        levels.append((sx, sy, sz, np.frombuffer(data, "<u2", cnt, ofs).copy()))
        ofs += 2 * cnt
    return levels


def write_rle4(levels: list[tuple[int, int, int, np.ndarray]]) -> bytes:
    out = [np.array([len(levels)], "<i4").tobytes()]
    for sx, sy, sz, words in levels:
        out.append(np.array([sx, sy, sz, len(words)], "<i4").tobytes())
        out.append(np.asarray(words, "<u2").tobytes())
    return b"".join(out)


class OracleScene:
    """Host-resident scene for the oracle: per level (sx, sy, sz, table, words)."""

    def __init__(self, levels: list[tuple[int, int, int, np.ndarray]]):
        self.levels = []
        for sx, sy, sz, words in levels:
            self.levels.append((sx, sy, sz, build_table(words, sx, sz), np.ascontiguousarray(words, np.uint16)))
        self._mips = (OrcMip * len(self.levels))(*[
            OrcMip(sx, sy, sz, t.ctypes.data, w.ctypes.data, len(w)) for sx, sy, sz, t, w in self.levels])

    @classmethod
    def from_rle4(cls, data: bytes) -> "OracleScene":
        return cls(parse_rle4(data))

    @property
    def nummaps(self) -> int:
        return len(self.levels)


# ---------------------------------------------------------------------------
# ray map, raycast, resolve
# ---------------------------------------------------------------------------

def raymap_build(pos, rot, border: float, maxres: int, fov_scale: float, samples: int, mip_distance: int,
                 z_far: int) -> OrcRayMap:
    rm = OrcRayMap()
    oracle().orc_raymap_build(C.byref(rm), *[float(v) for v in pos], *[float(v) for v in rot], border, maxres,
                              fov_scale, samples, mip_distance, z_far)
    return rm


def rays_to_render(rm: OrcRayMap) -> int:
    return int(oracle().orc_rays_to_render(C.byref(rm)))


def render_rays(rm: OrcRayMap, scene: OracleScene, nrays: Optional[int] = None, want_hits: bool = False,
                want_counters: bool = False, nthreads: int = 0):
    n = rays_to_render(rm) if nrays is None else nrays
    S = rm.samples
    out = np.zeros(n * S, np.uint32)
    depth = np.zeros(n * S, np.float32)
    hits = np.zeros(n * S, HIT_DTYPE) if want_hits else None
    cnt = np.zeros(n, COUNTERS_DTYPE) if want_counters else None
    oracle().orc_render_rays(C.byref(rm), scene._mips, scene.nummaps, n, out.ctypes.data, depth.ctypes.data,
                             None if hits is None else hits.ctypes.data, None if cnt is None else cnt.ctypes.data,
                             nthreads)
    return out, depth, hits, cnt


def resolve(rm: OrcRayMap, width: int, height: int, raybuf: np.ndarray, raydepth: np.ndarray,
            rayhit: Optional[np.ndarray] = None, want_index: bool = False):
    rows = int(oracle().orc_raybuf_rows(C.byref(rm)))
    S = rm.samples
    full = np.zeros(rows * S, np.uint32)
    fdep = np.zeros(rows * S, np.float32)
    full[:len(raybuf)] = raybuf
    fdep[:len(raydepth)] = raydepth
    fhit = None
    if rayhit is not None:
        fhit = np.zeros(rows * S, HIT_DTYPE)
        fhit[:len(rayhit)] = rayhit
    colour = np.zeros(width * height, np.uint32)
    depth = np.zeros(width * height, np.float32)
    hit = np.zeros(width * height, HIT_DTYPE) if rayhit is not None else None
    idx = np.zeros(width * height, np.int64) if want_index else None
    oracle().orc_resolve(C.byref(rm), width, height, rows, full.ctypes.data, fdep.ctypes.data,
                         None if fhit is None else fhit.ctypes.data, colour.ctypes.data, depth.ctypes.data,
                         None if hit is None else hit.ctypes.data, None if idx is None else idx.ctypes.data)
    return colour, depth, hit, idx


def soft_filter(colour: np.ndarray, depth: np.ndarray, width: int, height: int) -> np.ndarray:
    """The soft post-filter (bin/shader/soft.frag) of one resolved frame."""
    c = np.ascontiguousarray(colour, dtype=np.uint32)
    d = np.ascontiguousarray(depth, dtype=np.float32)
    out = np.zeros(width * height, np.uint32)
    oracle().orc_soft_filter(c.ctypes.data, d.ctypes.data, width, height, out.ctypes.data)
    return out


def raymap_from_product(pm) -> OrcRayMap:
    """The oracle's view of a product rle_raymap (api.RayMap): same fields."""
    rm = OrcRayMap()
    rm.vanishing_point_2d = V3(*pm.vanishing_point_2d)
    rm.map_line_count = pm.map_line_count
    rm.rotation = V3(*pm.rotation)
    rm.position = V3(*pm.position)
    rm.border, rm.clip_min, rm.clip_max = pm.border, pm.clip_min, pm.clip_max
    rm.maxres = pm.maxres
    rm.res[:] = list(pm.res)
    rm.p4 = V3(*pm.p4)
    for i in range(8):
        rm.p_2d[i] = V3(*pm.p_2d[i])
        rm.p_no[i] = V3(*pm.p_no[i])
    rm.to3d[:] = [pm.to3d[r][c] for r in range(4) for c in range(4)]
    rm.p_ofs_min[:] = list(pm.p_ofs_min)
    rm.p_ofs_max[:] = list(pm.p_ofs_max)
    rm.samples, rm.mip_distance, rm.z_far, rm.fov_scale = pm.samples, pm.mip_distance, pm.z_far, pm.fov_scale
    return rm


# ---------------------------------------------------------------------------
# the reference's host build
# ---------------------------------------------------------------------------

REF_RAYMAP_BYTES = 896  # sizeof(RayMap_GPU) on LP64


def ref_raymap(pos, rot, border: float, maxres: int) -> bytes:
    b = (C.c_uint8 * REF_RAYMAP_BYTES)()
    ref().ref_get_ray_map(*[float(v) for v in pos], *[float(v) for v in rot], border, maxres, b)
    return bytes(b)


def ref_raymap_fields(b: bytes) -> dict:
    """Fields of a RayMap_GPU (src/RayMap.h:16-54) from its LP64 bytes."""
    f = np.frombuffer(b, np.float32)
    i = np.frombuffer(b, np.int32)
    return {
        "vanishing_point_2d": f[0:3], "map_line_count": int(i[3]), "rotation": f[5:8], "position": f[8:11],
        "border": f[11], "clip_min": f[12], "clip_max": f[13], "maxres": int(i[143]), "res": i[144:148],
        "p4": f[148:151], "p_2d": f[151:175].reshape(8, 3), "p_no": f[175:199].reshape(8, 3),
        "to3d": f[199:215].reshape(4, 4), "p_ofs_min": f[215:219], "p_ofs_max": f[219:223],
    }


def ref_render_rays(raymap_bytes: bytes, scene: OracleScene, S: int, nrays: int, mip_distance: int, z_far: int,
                    nthreads: int = 0) -> np.ndarray:
    lv = scene.levels
    n = len(lv)
    ia = lambda xs: (C.c_int * n)(*xs)  # noqa: E731
    out = np.zeros(nrays * S, np.uint32)
    ref().ref_render_rays(raymap_bytes, n, ia([l[0] for l in lv]), ia([l[1] for l in lv]), ia([l[2] for l in lv]),
                          (C.c_void_p * n)(*[l[3].ctypes.data for l in lv]),
                          (C.c_void_p * n)(*[l[4].ctypes.data for l in lv]),
                          (C.c_longlong * n)(*[len(l[4]) for l in lv]), S, nrays, mip_distance, z_far,
                          out.ctypes.data, nthreads)
    return out


def ref_compress(bits: np.ndarray, sx: int, sy: int, sz: int, mip: int) -> tuple[np.ndarray, np.ndarray]:
    starts = np.zeros(sx * sz, np.uint32)
    p = C.POINTER(C.c_uint16)()
    n = C.c_longlong()
    ref().ref_compress(bits.ctypes.data, sx, sy, sz, mip, starts.ctypes.data, C.byref(p), C.byref(n))
    words = np.ctypeslib.as_array(p, shape=(n.value,)).copy()
    ref().ref_free(p)
    return starts, words


def ref_mipmap(bits: np.ndarray, sx: int, sy: int, sz: int) -> np.ndarray:
    out = np.zeros((sx // 2 // 8) * (sy // 2) * (sz // 2), np.uint8)
    ref().ref_mipmap(bits.ctypes.data, sx, sy, sz, out.ctypes.data)
    return out


def ref_load_table(path: str, mip: int, sx: int, sz: int) -> np.ndarray:
    table = np.zeros(2 * sx * sz, np.uint32)
    dims = np.zeros(5, np.int32)
    rc = ref().ref_load_table(str(path).encode(), mip, table.ctypes.data, dims.ctypes.data)
    if rc != 0:
        raise IOError(f"reference loader failed ({rc})")
    return table
