"""rle_gb300: GB300-native renderer for run-length-encoded voxel-column scenes.

The product is the CUDA/C++ library librle_gb300.so behind the C ABI in
include/rle_gb300.h; this package is its Python mirror (``api``) and build
script (``build``).  The folder name is not a Python identifier, so load it
by path, e.g. ``importlib.util.spec_from_file_location("rle_gb300", <dir>/__init__.py)``.
"""
from .api import *  # noqa: F401,F403
from .api import (Camera, Counters, Hit, HIT_DTYPE, RayMap, RLEError, Scene, SceneInfo,  # noqa: F401
                  ScenegenParams, ViewParams, camera, ground_height, frame_workspace_bytes, library, ptr,
                  raybuf_words, raymap_build, render_frame, render_rays, resolve, scenegen_default,
                  scenegen_dense, scenegen_rle4, tuning_get, tuning_set, version, view_params)
