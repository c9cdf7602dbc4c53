"""Python mirror of the rle_gb300 C ABI (include/rle_gb300.h), over ctypes.

The names, argument meaning and errors follow the C entry points, which in
turn replace the reference's render path: ``raymap_build`` is
RayMap::get_ray_map (src/RayMap.h:98-402), ``render_rays`` is
cuda_main_render2 / Render::render_line (src/Cuda_Main.cu:183-271,
src/Cuda_Render.h:96-737), ``resolve`` is the colorize shader
(bin/shader/colorize_buddha_soft.frag:12-80) and ``Scene`` is
RLE4::load + all_to_gpu (src/Rle4.cpp:244-448).

Device buffers are passed as raw device pointers (int) or any object with a
``data_ptr()`` method (a CUDA torch.Tensor).  The CUDA library must be built
(``build.py``); importing without it raises ImportError -- there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from pathlib import Path
from typing import Optional

import numpy as np

_HERE = Path(__file__).resolve().parent
# RLE_GB300_LIB selects another build of the library (the range-checked
# debug build, librle_gb300_checked.so); the default is the regular one.
LIB_PATH = Path(os.environ["RLE_GB300_LIB"]) if os.environ.get("RLE_GB300_LIB") else _HERE / "librle_gb300.so"
RLE_MAX_MIPS = 8
# rotation.x of the reference grows as the view turns down (src/RayMap.h:121);
# camera() takes pitch with negative = down.
PITCH_SIGN = -1.0

STATUS = {
    0: "RLE_OK", -1: "RLE_ERR_INVALID_ARG", -2: "RLE_ERR_IO", -3: "RLE_ERR_FORMAT", -4: "RLE_ERR_CUDA",
    -5: "RLE_ERR_NO_MEMORY", -6: "RLE_ERR_CAPACITY", -7: "RLE_ERR_TIMEOUT", -8: "RLE_ERR_CANCELLED",
    -9: "RLE_ERR_UNSUPPORTED",
}


class RLEError(RuntimeError):
    def __init__(self, status: int, where: str, message: str = ""):
        self.status = status
        self.name = STATUS.get(status, str(status))
        super().__init__(f"{where}: {self.name}" + (f" ({message})" if message else ""))


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("rot", C.c_float * 3), ("fov_deg", C.c_float)]


class ViewParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("samples", C.c_int), ("maxres", C.c_int),
                ("border", C.c_float), ("mip_distance", C.c_int), ("z_far", C.c_int)]


class RayMap(C.Structure):
    _fields_ = [
        ("vanishing_point_2d", C.c_float * 3), ("map_line_count", C.c_int), ("rotation", C.c_float * 3),
        ("position", C.c_float * 3), ("border", C.c_float), ("clip_min", C.c_float), ("clip_max", C.c_float),
        ("maxres", C.c_int), ("res", C.c_int * 4), ("p4", C.c_float * 3), ("p_2d", (C.c_float * 3) * 8),
        ("p_no", (C.c_float * 3) * 8), ("to3d", (C.c_float * 4) * 4), ("p_ofs_min", C.c_float * 4),
        ("p_ofs_max", C.c_float * 4), ("samples", C.c_int), ("mip_distance", C.c_int), ("z_far", C.c_int),
        ("fov_scale", C.c_float), ("sin_x", C.c_float), ("cos_x", C.c_float), ("sin_y", C.c_float),
        ("cos_y", C.c_float), ("sin_neg_y", C.c_float), ("cos_neg_y", C.c_float), ("width", C.c_int),
        ("height", C.c_int), ("rows", C.c_int), ("rays", C.c_int),
    ]


class Hit(C.Structure):
    _fields_ = [("x", C.c_uint16), ("z", C.c_uint16), ("y", C.c_uint16), ("mip", C.c_uint8), ("flags", C.c_uint8)]


HIT_DTYPE = np.dtype([("x", "<u2"), ("z", "<u2"), ("y", "<u2"), ("mip", "u1"), ("flags", "u1")])
COUNTER_FIELDS = ("cells", "fetched", "headers", "runs", "spans", "pixels")


class Counters(C.Structure):
    _fields_ = [(n, C.c_ulonglong) for n in COUNTER_FIELDS]


class Tuning(C.Structure):
    _fields_ = [("lanes_per_ray", C.c_int), ("cells_per_lane", C.c_int), ("threads_per_block", C.c_int),
                ("staging", C.c_int)]


RAYCAST_SHAPES = [(8, 1), (16, 1), (32, 1)]


class FrameRequest(C.Structure):
    _fields_ = [("cam", Camera), ("view", ViewParams), ("d_colour", C.c_void_p), ("d_depth", C.c_void_p),
                ("d_hit", C.c_void_p)]


class BatchTuning(C.Structure):
    _fields_ = [("tile_rays", C.c_int), ("lanes_per_ray", C.c_int), ("staging", C.c_int),
                ("threads_per_block", C.c_int), ("use_graph", C.c_int), ("per_frame", C.c_int)]

    def as_tuple(self):
        return (self.tile_rays, self.lanes_per_ray, self.staging, self.threads_per_block, self.use_graph,
                self.per_frame)


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget_bytes", C.c_size_t), ("max_frames_per_batch", C.c_int),
                ("max_inflight", C.c_int), ("raybuf_words", C.c_size_t), ("max_samples", C.c_int), ("plain", C.c_int),
                ("batch_tuning", BatchTuning)]


class Request(C.Structure):
    _fields_ = [("scene_id", C.c_int), ("cam", Camera), ("view", ViewParams), ("d_colour", C.c_void_p),
                ("d_depth", C.c_void_p)]


class Completion(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("status", C.c_int), ("submit_s", C.c_double), ("launch_s", C.c_double),
                ("done_s", C.c_double), ("gpu_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("cancelled", C.c_uint64), ("batches", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double), ("pixels", C.c_double), ("busy_s", C.c_double),
                ("mrays_per_s", C.c_double), ("device_bytes", C.c_uint64)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class SceneInfo(C.Structure):
    _fields_ = [("device", C.c_int), ("nummaps", C.c_int), ("sx", C.c_int * RLE_MAX_MIPS),
                ("sy", C.c_int * RLE_MAX_MIPS), ("sz", C.c_int * RLE_MAX_MIPS),
                ("slab_words", C.c_uint64 * RLE_MAX_MIPS), ("device_bytes", C.c_uint64),
                ("run_headers", C.c_uint64), ("surface_voxels", C.c_uint64)]


class ScenegenParams(C.Structure):
    _fields_ = [("sx", C.c_int), ("sy", C.c_int), ("sz", C.c_int), ("seed", C.c_uint64), ("nummaps", C.c_int),
                ("height_min", C.c_float), ("height_max", C.c_float), ("octaves", C.c_int),
                ("base_period", C.c_int), ("caves", C.c_int), ("cave_y0", C.c_float), ("cave_y1", C.c_float),
                ("cave_threshold", C.c_float), ("cave_period", C.c_float)]


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is not built; run build.py (the renderer has no CPU fallback)")
    lib = C.CDLL(str(LIB_PATH))
    vp = C.c_void_p
    sig = {
        "rle_status_string": (C.c_char_p, [C.c_int]),
        "rle_version": (C.c_char_p, []),
        "rle_last_error": (C.c_char_p, []),
        "rle_scene_load_file": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(vp)]),
        "rle_scene_load_memory": (C.c_int, [vp, C.c_size_t, C.c_int, C.POINTER(vp)]),
        "rle_scene_free": (C.c_int, [vp]),
        "rle_scene_get_info": (C.c_int, [vp, C.POINTER(SceneInfo)]),
        "rle_scene_copy_level": (C.c_int, [vp, C.c_int, vp, vp]),
        "rle_scenegen_default": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int, C.POINTER(ScenegenParams)]),
        "rle_scenegen_rle4": (C.c_int, [C.POINTER(ScenegenParams), C.POINTER(vp), C.POINTER(C.c_size_t)]),
        "rle_scenegen_dense": (C.c_int, [C.POINTER(ScenegenParams), C.c_int, vp, vp]),
        "rle_host_free": (None, [vp]),
        "rle_scenegen_device": (C.c_int, [C.POINTER(ScenegenParams), C.c_int, C.POINTER(vp)]),
        "rle_soft_filter": (C.c_int, [vp, vp, C.c_int, C.c_int, vp, vp]),
        "rle_bounds_check_read": (C.c_int, [C.c_int, C.POINTER(C.c_uint32), C.c_int]),
        "rle_debug_level_pointers": (C.c_int, [vp, C.c_int, C.POINTER(vp), C.POINTER(vp), C.POINTER(C.c_uint64)]),
        "rle_encode_device": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(vp)]),
        "rle_raymap_build": (C.c_int, [C.POINTER(Camera), C.POINTER(ViewParams), C.POINTER(RayMap)]),
        "rle_raybuf_words": (C.c_size_t, [C.POINTER(RayMap)]),
        "rle_tuning_set": (C.c_int, [C.POINTER(Tuning)]),
        "rle_tuning_get": (C.c_int, [C.POINTER(Tuning)]),
        "rle_render_rays": (C.c_int, [vp, C.POINTER(RayMap), vp, vp, vp, vp, vp]),
        "rle_render_rays_timed": (C.c_int, [vp, C.POINTER(RayMap), vp, vp, vp, vp]),
        "rle_resolve": (C.c_int, [C.POINTER(RayMap), vp, vp, vp, vp, vp, vp, vp]),
        "rle_frame_workspace_bytes": (C.c_size_t, [C.POINTER(ViewParams)]),
        "rle_render_frame": (C.c_int, [vp, C.POINTER(Camera), C.POINTER(ViewParams), vp, C.c_size_t, vp, vp, vp, vp]),
        "rle_batch_create": (C.c_int, [C.c_int, C.c_int, C.c_size_t, C.c_int, C.c_int, C.POINTER(vp)]),
        "rle_batch_free": (C.c_int, [vp]),
        "rle_batch_set_tuning": (C.c_int, [vp, C.POINTER(BatchTuning)]),
        "rle_batch_get_tuning": (C.c_int, [vp, C.POINTER(BatchTuning)]),
        "rle_batch_words_needed": (C.c_size_t, [C.POINTER(FrameRequest), C.c_int]),
        "rle_batch_render": (C.c_int, [vp, vp, C.POINTER(FrameRequest), C.c_int, vp]),
        "rle_batch_autotune": (C.c_int, [vp, vp, C.POINTER(FrameRequest), C.c_int, C.c_int, C.POINTER(BatchTuning),
                                         C.POINTER(C.c_float)]),
        "rle_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(vp)]),
        "rle_server_add_scene": (C.c_int, [vp, vp, C.POINTER(C.c_int)]),
        "rle_server_submit": (C.c_int, [vp, C.POINTER(Request), C.POINTER(C.c_uint64)]),
        "rle_server_cancel": (C.c_int, [vp, C.c_uint64]),
        "rle_server_wait": (C.c_int, [vp, C.c_uint64, C.c_int, C.POINTER(Completion)]),
        "rle_server_drain": (C.c_int, [vp, C.c_int]),
        "rle_server_poll": (C.c_int, [vp, C.POINTER(Completion), C.c_int, C.POINTER(C.c_int)]),
        "rle_server_get_stats": (C.c_int, [vp, C.POINTER(ServerStats)]),
        "rle_server_reset_stats": (C.c_int, [vp]),
        "rle_server_inject_launch_failures": (C.c_int, [vp, C.c_int]),
        "rle_server_pause": (C.c_int, [vp, C.c_int]),
        "rle_server_destroy": (C.c_int, [vp]),
        "rle_render_frame_noalloc_limit": (C.c_size_t, []),
        "rle_render_frame_noalloc": (C.c_int, [vp, C.POINTER(Camera), C.POINTER(ViewParams), vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


_lib = _load()


def library() -> C.CDLL:
    """The loaded librle_gb300.so (for entry points without a wrapper)."""
    return _lib


def _check(status: int, where: str) -> None:
    if status != 0:
        msg = _lib.rle_last_error()
        raise RLEError(status, where, msg.decode() if msg else "")


def ptr(x) -> Optional[int]:
    """Device pointer of an int, None or a tensor-like with data_ptr()."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    raise TypeError(f"cannot take a device pointer of {type(x).__name__}")


def version() -> str:
    return _lib.rle_version().decode()


# ---------------------------------------------------------------------------
# scenes
# ---------------------------------------------------------------------------

def scenegen_default(sx: int, sy: int, sz: int, seed: int, caves: bool = False) -> ScenegenParams:
    p = ScenegenParams()
    _check(_lib.rle_scenegen_default(sx, sy, sz, seed, int(caves), C.byref(p)), "rle_scenegen_default")
    return p


def scenegen_rle4(params: ScenegenParams) -> bytes:
    """Seeded synthetic scene as .rle4 bytes."""
    buf = C.c_void_p()
    n = C.c_size_t()
    _check(_lib.rle_scenegen_rle4(C.byref(params), C.byref(buf), C.byref(n)), "rle_scenegen_rle4")
    try:
        return C.string_at(buf, n.value)
    finally:
        _lib.rle_host_free(buf)


def scenegen_dense(params: ScenegenParams, mip: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """Solid bits (Tree layout) and RGB565 colours of one level of a small scene."""
    sx, sy, sz = params.sx >> mip, params.sy >> mip, params.sz >> mip
    bits = np.zeros((sx * sy * sz + 7) // 8, np.uint8)
    cols = np.zeros(sx * sy * sz, np.uint16)
    _check(_lib.rle_scenegen_dense(C.byref(params), mip, bits.ctypes.data, cols.ctypes.data), "rle_scenegen_dense")
    return bits, cols


class Scene:
    """A scene resident on one GPU (column tables + slab words per level)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle

    @classmethod
    def generate_on_device(cls, params: ScenegenParams, device: int = 0) -> "Scene":
        """rle_scenegen_device: the seeded generator, mips and encoder run as
        kernels straight into device memory (same scene as from_bytes of
        scenegen_rle4(params))."""
        h = C.c_void_p()
        _check(_lib.rle_scenegen_device(C.byref(params), device, C.byref(h)), "rle_scenegen_device")
        return cls(h)

    @classmethod
    def encode_on_device(cls, bits, colours, sx: int, sy: int, sz: int, nummaps: int = 4,
                         device: int = 0) -> "Scene":
        """rle_encode_device: RLE4::compress_all of a device bit volume in the
        reference's Tree layout (optional u16 colour per voxel, same index)."""
        h = C.c_void_p()
        _check(_lib.rle_encode_device(ptr(bits), ptr(colours), sx, sy, sz, nummaps, device, C.byref(h)),
               "rle_encode_device")
        return cls(h)

    @classmethod
    def from_file(cls, path: str, device: int = 0) -> "Scene":
        h = C.c_void_p()
        _check(_lib.rle_scene_load_file(str(path).encode(), device, C.byref(h)), "rle_scene_load_file")
        return cls(h)

    @classmethod
    def from_bytes(cls, data: bytes, device: int = 0) -> "Scene":
        h = C.c_void_p()
        buf = C.create_string_buffer(data, len(data))
        _check(_lib.rle_scene_load_memory(buf, len(data), device, C.byref(h)), "rle_scene_load_memory")
        return cls(h)

    @property
    def handle(self) -> C.c_void_p:
        if not self._h:
            raise RLEError(-1, "Scene", "scene was freed")
        return self._h

    def info(self) -> SceneInfo:
        i = SceneInfo()
        _check(_lib.rle_scene_get_info(self.handle, C.byref(i)), "rle_scene_get_info")
        return i

    def copy_level(self, mip: int) -> tuple[np.ndarray, np.ndarray]:
        """Host copies of one level's uint2 table (as 2*sx*sz u32) and slab words."""
        i = self.info()
        table = np.zeros(2 * i.sx[mip] * i.sz[mip], np.uint32)
        slabs = np.zeros(int(i.slab_words[mip]), np.uint16)
        _check(_lib.rle_scene_copy_level(self.handle, mip, table.ctypes.data, slabs.ctypes.data),
               "rle_scene_copy_level")
        return table, slabs

    def free(self) -> None:
        if self._h:
            _check(_lib.rle_scene_free(self._h), "rle_scene_free")
            self._h = C.c_void_p()

    def __enter__(self) -> "Scene":
        return self

    def __exit__(self, *a) -> None:
        self.free()

    def __del__(self):
        try:
            if self._h:
                _lib.rle_scene_free(self._h)
        except Exception:
            pass


# ---------------------------------------------------------------------------
# cameras and ray maps
# ---------------------------------------------------------------------------

def camera(x: float, z: float, eye_height: float, yaw_deg: float, pitch_deg: float,
           fov_deg: float = 90.0, scene_height: int = 256) -> Camera:
    """Camera at (x, z) on the grid, eye_height voxels above the bottom of a
    scene scene_height voxels tall, looking along yaw; negative pitch looks
    down.  In the reference's convention the column axis points down (word 0
    of a column is the top) and position.y is the eye's coordinate on it,
    negated: a voxel at index j lies j + position.y below the eye."""
    c = Camera()
    c.pos[:] = (x, eye_height - scene_height, z)
    c.rot[:] = (PITCH_SIGN * math.radians(pitch_deg), math.radians(yaw_deg), 0.0)
    c.fov_deg = fov_deg
    return c


def view_params(width: int, height: int, samples: int = 0, maxres: int = 0, border: float = 0.0,
                mip_distance: int = 0, z_far: int = 0) -> ViewParams:
    return ViewParams(width, height, samples, maxres, border, mip_distance, z_far)


def raymap_build(cam: Camera, view: ViewParams) -> RayMap:
    rm = RayMap()
    _check(_lib.rle_raymap_build(C.byref(cam), C.byref(view), C.byref(rm)), "rle_raymap_build")
    return rm


def raybuf_words(rm: RayMap) -> int:
    return int(_lib.rle_raybuf_words(C.byref(rm)))


def tuning_set(lanes_per_ray: int = 0, cells_per_lane: int = 0, threads_per_block: int = 0, staging: int = 0) -> None:
    """Process-wide launch shape of the raycast (0 = built-in default)."""
    _check(_lib.rle_tuning_set(C.byref(Tuning(lanes_per_ray, cells_per_lane, threads_per_block, staging))),
           "rle_tuning_set")


def tuning_get() -> tuple[int, int, int, int]:
    """(lanes_per_ray, cells_per_lane, threads_per_block, staging)."""
    t = Tuning()
    _check(_lib.rle_tuning_get(C.byref(t)), "rle_tuning_get")
    return t.lanes_per_ray, t.cells_per_lane, t.threads_per_block, t.staging


# ---------------------------------------------------------------------------
# rendering
# ---------------------------------------------------------------------------

def render_rays(scene: Scene, rm: RayMap, raybuf, raydepth, rayhit=None, counters=None, stream: int = 0) -> None:
    _check(_lib.rle_render_rays(scene.handle, C.byref(rm), ptr(raybuf), ptr(raydepth), ptr(rayhit),
                                ptr(counters), stream or None), "rle_render_rays")


# rle_ray_time: per-ray start/end of one raycast launch (rle_render_rays_timed)
RAY_TIME_DTYPE = np.dtype([("start_ns", "<u8"), ("end_ns", "<u8"), ("start_clock", "<u8"), ("end_clock", "<u8"),
                           ("sm", "<u4"), ("reserved", "<u4")])


def render_rays_timed(scene: Scene, rm: RayMap, raybuf, raydepth, times, stream: int = 0) -> None:
    """rle_render_rays (production kernel, no hits or counters) that also
    writes an rle_ray_time record per cast ray into `times` (a device buffer
    of at least rm.rays * 40 bytes)."""
    _check(_lib.rle_render_rays_timed(scene.handle, C.byref(rm), ptr(raybuf), ptr(raydepth), ptr(times),
                                      stream or None), "rle_render_rays_timed")


def resolve(rm: RayMap, raybuf, raydepth, colour, depth, rayhit=None, hit=None, stream: int = 0) -> None:
    _check(_lib.rle_resolve(C.byref(rm), ptr(raybuf), ptr(raydepth), ptr(rayhit), ptr(colour), ptr(depth),
                            ptr(hit), stream or None), "rle_resolve")


def frame_workspace_bytes(view: ViewParams) -> int:
    return int(_lib.rle_frame_workspace_bytes(C.byref(view)))


def render_frame(scene: Scene, cam: Camera, view: ViewParams, workspace, workspace_bytes: int, colour, depth,
                 hit=None, stream: int = 0) -> None:
    _check(_lib.rle_render_frame(scene.handle, C.byref(cam), C.byref(view), ptr(workspace), workspace_bytes,
                                 ptr(colour), ptr(depth), ptr(hit), stream or None), "rle_render_frame")


def frame_request(cam: Camera, view: ViewParams, colour, depth, hit=None) -> FrameRequest:
    return FrameRequest(cam, view, ptr(colour), ptr(depth), ptr(hit))


def _requests(frames) -> tuple:
    arr = (FrameRequest * len(frames))(*frames)
    return arr, len(frames)


def batch_words_needed(frames) -> int:
    arr, n = _requests(frames)
    return int(_lib.rle_batch_words_needed(arr, n))


class Batch:
    """Many cameras per launch (rle_batch_*): one persistent raycast and one
    persistent resolve, captured into a CUDA graph and replayed."""

    def __init__(self, max_frames: int, raybuf_words: int, max_samples: int = 4096, with_hits: bool = False,
                 device: int = 0):
        h = C.c_void_p()
        _check(_lib.rle_batch_create(device, max_frames, raybuf_words, max_samples, int(with_hits), C.byref(h)),
               "rle_batch_create")
        self._h = h

    @property
    def handle(self):
        if not self._h:
            raise RLEError(-1, "Batch", "batch was freed")
        return self._h

    def tuning(self) -> BatchTuning:
        t = BatchTuning()
        _check(_lib.rle_batch_get_tuning(self.handle, C.byref(t)), "rle_batch_get_tuning")
        return t

    def set_tuning(self, tile_rays: int, lanes_per_ray: int, staging: int = 1, threads_per_block: int = 128,
                   use_graph: bool = True, per_frame: bool = False) -> None:
        t = BatchTuning(tile_rays, lanes_per_ray, staging, threads_per_block, int(use_graph), int(per_frame))
        _check(_lib.rle_batch_set_tuning(self.handle, C.byref(t)), "rle_batch_set_tuning")

    def render(self, scene: Scene, frames, stream: int = 0) -> None:
        arr, n = _requests(frames)
        _check(_lib.rle_batch_render(self.handle, scene.handle, arr, n, stream or None), "rle_batch_render")

    def autotune(self, scene: Scene, frames, repeats: int = 3) -> tuple[BatchTuning, float]:
        arr, n = _requests(frames)
        best = BatchTuning()
        ms = C.c_float()
        _check(_lib.rle_batch_autotune(self.handle, scene.handle, arr, n, repeats, C.byref(best), C.byref(ms)),
               "rle_batch_autotune")
        return best, ms.value

    def free(self) -> None:
        if self._h:
            _check(_lib.rle_batch_free(self._h), "rle_batch_free")
            self._h = C.c_void_p()

    def __del__(self):
        try:
            if self._h:
                _lib.rle_batch_free(self._h)
        except Exception:
            pass


class Server:
    """Render server (rle_server_*): resident scenes, a request queue and a
    scheduler thread doing continuous batching (or, with plain=True, one
    launch per request)."""

    def __init__(self, hbm_budget_bytes: int, raybuf_words: int, max_frames_per_batch: int = 64,
                 max_inflight: int = 2, max_samples: int = 1920, plain: bool = False, device: int = 0,
                 batch_tuning: Optional[BatchTuning] = None):
        cfg = ServerConfig(device, hbm_budget_bytes, max_frames_per_batch, max_inflight, raybuf_words, max_samples,
                           int(plain), batch_tuning if batch_tuning is not None else BatchTuning())
        h = C.c_void_p()
        _check(_lib.rle_server_create(C.byref(cfg), C.byref(h)), "rle_server_create")
        self._h = h

    @property
    def handle(self):
        if not self._h:
            raise RLEError(-1, "Server", "server was destroyed")
        return self._h

    def add_scene(self, scene: Scene) -> int:
        sid = C.c_int()
        _check(_lib.rle_server_add_scene(self.handle, scene.handle, C.byref(sid)), "rle_server_add_scene")
        return sid.value

    def submit(self, scene_id: int, cam: Camera, view: ViewParams, colour, depth) -> int:
        r = Request(scene_id, cam, view, ptr(colour), ptr(depth))
        t = C.c_uint64()
        _check(_lib.rle_server_submit(self.handle, C.byref(r), C.byref(t)), "rle_server_submit")
        return t.value

    def cancel(self, ticket: int) -> int:
        return _lib.rle_server_cancel(self.handle, ticket)

    def wait(self, ticket: int, timeout_ms: int = 10000) -> Completion:
        c = Completion()
        _check(_lib.rle_server_wait(self.handle, ticket, timeout_ms, C.byref(c)), "rle_server_wait")
        return c

    def drain(self, timeout_ms: int = 60000) -> None:
        _check(_lib.rle_server_drain(self.handle, timeout_ms), "rle_server_drain")

    def poll(self, max_n: int = 4096) -> list:
        arr = (Completion * max_n)()
        n = C.c_int()
        _check(_lib.rle_server_poll(self.handle, arr, max_n, C.byref(n)), "rle_server_poll")
        return [arr[i] for i in range(n.value)]

    def stats(self) -> ServerStats:
        s = ServerStats()
        _check(_lib.rle_server_get_stats(self.handle, C.byref(s)), "rle_server_get_stats")
        return s

    def reset_stats(self) -> None:
        _check(_lib.rle_server_reset_stats(self.handle), "rle_server_reset_stats")

    def inject_launch_failures(self, count: int) -> None:
        _check(_lib.rle_server_inject_launch_failures(self.handle, count), "rle_server_inject_launch_failures")

    def pause(self, paused: bool = True) -> None:
        _check(_lib.rle_server_pause(self.handle, int(paused)), "rle_server_pause")

    def destroy(self) -> None:
        if self._h:
            _check(_lib.rle_server_destroy(self._h), "rle_server_destroy")
            self._h = C.c_void_p()

    def __del__(self):
        try:
            if self._h:
                _lib.rle_server_destroy(self._h)
        except Exception:
            pass


def render_frame_noalloc(scene: Scene, cam: Camera, view: ViewParams, colour, depth, stream: int = 0) -> None:
    """rle_render_frame for callers that may not allocate device memory: the
    ray buffer is a fixed array inside the library (render_frame_noalloc_limit()
    bytes per device).  Calls share that array, so keep them on one stream."""
    _check(_lib.rle_render_frame_noalloc(scene.handle, C.byref(cam), C.byref(view), ptr(colour), ptr(depth),
                                         stream or None), "rle_render_frame_noalloc")


def soft_filter(colour, depth, width: int, height: int, out, stream: int = 0) -> None:
    """rle_soft_filter: the reference's soft post-filter (bin/shader/soft.frag)
    over one resolved frame; RGBA8 out (must not alias colour)."""
    _check(_lib.rle_soft_filter(ptr(colour), ptr(depth), width, height, ptr(out), stream or None), "rle_soft_filter")


def bounds_check_read(device: int = 0, clear: bool = True) -> tuple[int, int]:
    """(failed-check flags, first failing index) of the range-checked debug
    library; raises RLEError(UNSUPPORTED) with the regular library."""
    out = (C.c_uint32 * 4)()
    _check(_lib.rle_bounds_check_read(device, out, int(clear)), "rle_bounds_check_read")
    return int(out[0]), int(out[1]) | (int(out[2]) << 32)


def debug_level_pointers(scene: "Scene", mip: int) -> tuple[int, int, int]:
    """(table, slabs, words) device pointers of a level (range-checked debug
    library only)."""
    t, sl, w = C.c_void_p(), C.c_void_p(), C.c_uint64()
    _check(_lib.rle_debug_level_pointers(scene.handle, mip, C.byref(t), C.byref(sl), C.byref(w)),
           "rle_debug_level_pointers")
    return int(t.value), int(sl.value), int(w.value)


def render_frame_noalloc_limit() -> int:
    return int(_lib.rle_render_frame_noalloc_limit())


def ground_height(table: np.ndarray, slabs: np.ndarray, sx: int, sy: int, x: int, z: int) -> int:
    """Height above the bottom of the topmost stored voxel's upper face in
    column (x, z) of a level (0 for an empty column), from host copies of the
    level's table and slab words.  Column words run from the top down."""
    c = (z * sx + x) * 2
    ofs, count = int(table[c]), int(table[c + 1]) & 0xFFFF
    depth = 0
    for r in range(count):
        w = int(slabs[ofs + 2 + r])
        depth += w & 1023
        if w >> 10:
            return sy - depth
    return 0
