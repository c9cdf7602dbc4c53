"""A plain C program (tests/c/abi_client.c) compiled with gcc against
include/rle_gb300.h and linked to the library: the C ABI works from C as a
reference-side integration would use it.  Host checks run everywhere; the
GPU run renders one frame through rle_render_frame."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "rle-based-voxel-raycasting_gb300"


def _cuda_lib_dir() -> Path:
    nvcc = shutil.which("nvcc")
    home = Path(nvcc).resolve().parent.parent if nvcc else Path("/usr/local/cuda")
    for d in (home / "lib64", home / "lib", home / "targets" / "sbsa-linux" / "lib",
              home / "targets" / "x86_64-linux" / "lib"):
        if (d / "libcudart.so").exists():
            return d
    pytest.skip("libcudart.so not found")


@pytest.fixture(scope="module")
def client(rle, tmp_path_factory):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    out = tmp_path_factory.mktemp("abi") / "abi_client"
    cuda = _cuda_lib_dir()
    cmd = ["gcc", "-std=c11", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "c" / "abi_client.c"), "-o", str(out),
           "-L", str(PKG), "-lrle_gb300", "-L", str(cuda), "-lcudart", "-lm",
           f"-Wl,-rpath,{PKG}", f"-Wl,-rpath,{cuda}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_c_client_host(client):
    r = subprocess.run([str(client), "host"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")


@pytest.mark.gpu
def test_c_client_renders_a_frame(client, torch_cuda):
    r = subprocess.run([str(client), "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "terrain" in r.stdout and r.stdout.strip().endswith("ok")
