"""Build the in-tree native parts: libdarcy_gpu.so (sm_103a CUDA + C ABI) and
the `_core` Python extension over it. No cmake: two nvcc translation units and
one g++ unit, compiled in parallel.

    python darcy_cpp_gb300/build.py [-v] [--force]

(run by path: importing the package needs the extension this script builds)
"""

from __future__ import annotations

import importlib.util
import os
import re
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
LIB = PKG / "libdarcy_gpu.so"
EXT = PKG / ("_core" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))
VERSION = "1.0.0"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build darcy_cpp_gb300")


def _pybind11_include() -> str:
    spec = importlib.util.find_spec("torch")
    if spec and spec.submodule_search_locations:
        inc = Path(list(spec.submodule_search_locations)[0]) / "include"
        if (inc / "pybind11" / "pybind11.h").exists():
            return str(inc)
    spec = importlib.util.find_spec("pybind11")
    if spec and spec.submodule_search_locations:
        inc = Path(list(spec.submodule_search_locations)[0]) / "include"
        if (inc / "pybind11" / "pybind11.h").exists():
            return str(inc)
    raise RuntimeError("pybind11 headers not found (looked in torch/include and the pybind11 package)")


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build(verbose: bool = False, force: bool = False) -> tuple[Path, Path]:
    """Compile libdarcy_gpu.so and the _core extension (in place, incremental)."""
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [INCLUDE / "darcy_gpu.h"]
    units = ["kernels", "solver", "noalloc", "learn", "fieldgen"]
    units = [u for u in units if (CSRC / f"{u}.cu").exists()]
    objs = [BUILD / f"{u}.o" for u in units]
    flags = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]

    def compile_unit(u: str) -> None:
        src, obj = CSRC / f"{u}.cu", BUILD / f"{u}.o"
        if force or _stale(obj, [src, *headers]):
            _run([nvcc, *flags, "-c", str(src), "-o", str(obj)], verbose)

    with ThreadPoolExecutor(max_workers=len(units)) as pool:
        list(pool.map(compile_unit, units))
    if force or _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-o", str(LIB), *map(str, objs)], verbose)

    nvcc_version = re.search(r"release ([0-9.]+)", subprocess.run([nvcc, "--version"], capture_output=True,
                                                                   text=True).stdout)
    bind = CSRC / "bindings.cpp"
    if force or _stale(EXT, [bind, LIB, INCLUDE / "darcy_gpu.h"]):
        _run([
            os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
            f"-DDARCY_VERSION=\"{VERSION}\"",
            f"-DDARCY_NVCC_VERSION=\"{nvcc_version.group(1) if nvcc_version else '?'}\"",
            "-I", _pybind11_include(), "-I", sysconfig.get_paths()["include"], str(bind),
            "-o", str(EXT), f"-L{PKG}", "-ldarcy_gpu", "-Wl,-rpath,$ORIGIN",
        ], verbose)
    return LIB, EXT


if __name__ == "__main__":
    lib, ext = build(verbose="-v" in sys.argv, force="--force" in sys.argv)
    print("built", lib, ext)
