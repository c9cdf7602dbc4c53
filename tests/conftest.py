"""Shared set-up: the `gpu` marker, the package loader and common scenes.

GPU tests run on a CUDA device and call the renderer through its C ABI;
everything else runs on the host (oracle, host C++ entry points, golden
fixtures, the reference's host build where it exists).
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / "rle-based-voxel-raycasting_gb300"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


def load_package():
    """Import the renderer's Python mirror (the folder name is not an identifier)."""
    if "rle_gb300" in sys.modules:
        return sys.modules["rle_gb300"]
    spec = importlib.util.spec_from_file_location("rle_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["rle_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def ensure_built():
    sys.path.insert(0, str(PKG_DIR))
    try:
        import build as pkg_build  # noqa: WPS433 (the package's build script)
    finally:
        sys.path.pop(0)
    pkg_build.build()


@pytest.fixture(scope="session")
def rle():
    ensure_built()
    return load_package()


@pytest.fixture(scope="session")
def po():
    from oracle import pyoracle
    pyoracle.build_oracle()
    return pyoracle


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(ROOT / "tests" / "golden" / "golden_v1.npz"))


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def torch_cuda():
    if not cuda_available():
        pytest.skip("no CUDA device")
    import torch
    return torch
