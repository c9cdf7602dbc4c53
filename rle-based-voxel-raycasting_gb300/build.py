"""Builds librle_gb300.so in place: CUDA sources for sm_103a with nvcc,
host C++ with g++, linked against the static CUDA runtime.

    python rle-based-voxel-raycasting_gb300/build.py [--jobs N] [--force] [--bounds-check]

Floating point: the traversal and resolve kernels are compiled with
-fmad=false, IEEE division and square root and no flush-to-zero; host code
with -ffp-contract=off (aarch64 compilers contract into FMA by default).
That keeps every float operation a single IEEE operation, which the
bit-exact parity with the reference depends on.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "librle_gb300.so"
# Debug variant: every device table, slab and ray-buffer index range-checked
# (-DRLE_BOUNDS_CHECK); a failed check is recorded, not executed.
BUILD_CHECKED = PKG / "_build_checked"
LIB_CHECKED = PKG / "librle_gb300_checked.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def sources() -> tuple[list[Path], list[Path]]:
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    return cu, cpp


_ELF_MACHINE = {"x86_64": 62, "aarch64": 183, "arm64": 183}


def foreign_binary(path: Path) -> bool:
    """True if `path` is an ELF file built for another CPU than this host's."""
    import platform
    import struct
    want = _ELF_MACHINE.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if len(head) < 20 or head[:4] != b"\x7fELF" or want is None:
        return False
    return struct.unpack_from("<H", head, 18)[0] != want


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists() or foreign_binary(obj):
        return True
    deps = [src, *CSRC.glob("*.h"), *INCLUDE.glob("*.h"), Path(__file__)]
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(jobs: int | None = None, force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    home = cuda_home()
    nvcc = str(home / "bin" / "nvcc")
    bdir, lib = (BUILD_CHECKED, LIB_CHECKED) if checked else (BUILD, LIB)
    bdir.mkdir(exist_ok=True)
    cu, cpp = sources()
    common_inc = [f"-I{INCLUDE}", f"-I{CSRC}"] + (["-DRLE_BOUNDS_CHECK"] if checked else [])
    steps = []
    objs = []
    for src in cu:
        obj = bdir / (src.stem + ".cu.o")
        objs.append(obj)
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
               "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "-Xptxas", "-v" if verbose else "-O3", *common_inc, "-c", str(src), "-o", str(obj)]
        if force or _stale(obj, src):
            steps.append(cmd)
    for src in cpp:
        obj = bdir / (src.stem + ".cpp.o")
        objs.append(obj)
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
               "-Wall", *common_inc, f"-I{home / 'include'}", "-c", str(src), "-o", str(obj)]
        if force or _stale(obj, src):
            steps.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        list(ex.map(_run, steps))
    if steps or not lib.exists() or foreign_binary(lib):
        lib_dirs = [home / "lib64", home / "lib", home / "targets" / "sbsa-linux" / "lib",
                    home / "targets" / "x86_64-linux" / "lib"]
        ldirs = [f"-L{d}" for d in lib_dirs if d.exists()]
        tmp = lib.with_suffix(".so.tmp")
        _run(["g++", "-shared", "-fopenmp", "-o", str(tmp), *map(str, objs), *ldirs,
              "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
        os.replace(tmp, lib)
    return lib


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true", help="pass -Xptxas -v (registers, spills)")
    ap.add_argument("--bounds-check", action="store_true",
                    help="build the range-checked debug library librle_gb300_checked.so")
    a = ap.parse_args(argv)
    try:
        lib = build(a.jobs, a.force, a.verbose, a.bounds_check)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        return 1
    print(lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
