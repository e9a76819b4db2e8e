"""Build the reference itself (darcy-cpp v1.0.0) for the oracle pin and the CPU
baseline -- test and measurement infrastructure, never part of the product.

Two outputs, both git-ignored:

* ``oracle/_ref/libdarcy_ref.so``: the reference's header-only solver
  (include/darcy/*.hpp) behind the small C-ABI shim ``oracle/ref_driver.cpp``.
  The golden-vector script and the oracle tests run it to pin the C
  restatement bit for bit.
* ``baseline/_ref/``: the reference's own Python package, installed unmodified
  with ``pip install --no-deps --target baseline/_ref`` (from a copy in a
  temporary directory: its build writes into the source tree), plus its
  C++ sources (include/darcy/*.hpp, src/bindings.cpp) staged unmodified in
  ``baseline/_ref/_src`` so that a machine without the checkout -- the Arm
  GPU host, where the x86 extension cannot load -- compiles the reference's
  own ``_core`` extension from them. bench.py's reference arm imports that
  package (``import darcy``) and times the reference through its public API.

The reference's own build system (CMake via scikit-build-core) runs only in
the pip install. Everywhere else g++ compiles the sources directly with the
flags of the reference's Release build (CMakeLists.txt:4-6, :68-71, :88):
C++17 without extensions, -O3 -DNDEBUG -fno-math-errno, OpenMP,
DARCY_VERSION="1.0.0". pybind11's headers come from the torch install (they
ship with it) or the pybind11 package.

    python oracle/build_ref.py [--ref PATH]   (PATH defaults to $DARCY_REFERENCE)
"""

from __future__ import annotations

import argparse
import importlib.util
import os
import shutil
import subprocess
import sys
import sysconfig
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REF_OUT = HERE / "_ref"
BASE = ROOT / "baseline" / "_ref"
STAGE = BASE / "_src"
# where this build's checkout of the reference lives unless --ref or
# $DARCY_REFERENCE says otherwise
DEFAULT_REF = "/root/reference"
CXXFLAGS = ["-O3", "-DNDEBUG", "-fno-math-errno", "-std=c++17", "-fopenmp", "-fPIC", "-shared"]


def _pybind11_include() -> str | None:
    for mod in ("torch", "pybind11"):
        spec = importlib.util.find_spec(mod)
        if spec and spec.submodule_search_locations:
            inc = Path(list(spec.submodule_search_locations)[0]) / "include"
            if (inc / "pybind11" / "pybind11.h").exists():
                return str(inc)
    return None


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, sources: list[Path]) -> bool:
    return not target.exists() or any(s.stat().st_mtime > target.stat().st_mtime for s in sources)


def build_shim(include: Path) -> Path:
    """oracle/_ref/libdarcy_ref.so from the reference headers under `include`."""
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "libdarcy_ref.so"
    srcs = [HERE / "ref_driver.cpp", *sorted((include / "darcy").glob("*.hpp"))]
    if _stale(out, srcs):
        _run([os.environ.get("CXX", "g++"), *CXXFLAGS, f"-I{include}", str(HERE / "ref_driver.cpp"), "-o", str(out)])
    return out


def install_package(ref: Path) -> None:
    """pip install of the unmodified reference into baseline/_ref (offline,
    no dependencies: numpy and scipy are already present)."""
    if (BASE / "darcy" / "__init__.py").exists():
        return
    with tempfile.TemporaryDirectory() as tmp:
        copy = Path(tmp) / "darcy-cpp"
        shutil.copytree(ref, copy, ignore=shutil.ignore_patterns(".git", "build"))
        _run([sys.executable, "-m", "pip", "install", "--quiet", "--no-index", "--no-build-isolation", "--no-deps",
              "--find-links", "/opt/wheelhouse", "--target", str(BASE), str(copy)])


def stage_sources(ref: Path) -> None:
    """The reference's C++ sources, unmodified, beside its installed package."""
    (STAGE / "include" / "darcy").mkdir(parents=True, exist_ok=True)
    (STAGE / "src").mkdir(exist_ok=True)
    for hpp in sorted((ref / "include" / "darcy").glob("*.hpp")):
        shutil.copy2(hpp, STAGE / "include" / "darcy" / hpp.name)
    shutil.copy2(ref / "src" / "bindings.cpp", STAGE / "src" / "bindings.cpp")


def build_extension() -> Path | None:
    """baseline/_ref/darcy/_core<EXT_SUFFIX> for this machine, from the staged
    sources (skipped when pip already built it here)."""
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = BASE / "darcy" / f"_core{suffix}"
    bind = STAGE / "src" / "bindings.cpp"
    if not bind.exists() or not (BASE / "darcy").is_dir():
        return None
    pyb = _pybind11_include()
    if pyb is None:
        raise RuntimeError("pybind11 headers not found (torch/include or the pybind11 package)")
    srcs = [bind, *sorted((STAGE / "include" / "darcy").glob("*.hpp"))]
    if _stale(out, srcs):
        _run([os.environ.get("CXX", "g++"), *CXXFLAGS, "-fvisibility=hidden", '-DDARCY_VERSION="1.0.0"',
              f"-I{STAGE / 'include'}", f"-I{pyb}", f"-I{sysconfig.get_paths()['include']}", str(bind),
              "-o", str(out)])
    return out


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--ref", type=Path, default=Path(os.environ.get("DARCY_REFERENCE", DEFAULT_REF)))
    args = ap.parse_args()
    if (args.ref / "include" / "darcy" / "solver.hpp").exists():
        print("built", build_shim(args.ref / "include"))
        # the installed package is for the CPU baseline only: without it the
        # benchmark falls back to the oracle port, so a failed install is
        # reported, not fatal
        try:
            install_package(args.ref)
            stage_sources(args.ref)
        except (RuntimeError, OSError) as exc:
            print(f"reference package not installed into {BASE}: {exc}", file=sys.stderr)
    elif (STAGE / "include" / "darcy" / "solver.hpp").exists():
        print("built", build_shim(STAGE / "include"))
    else:
        print(f"reference sources not found (checkout {args.ref}, staged {STAGE}); skipping", file=sys.stderr)
        return
    try:
        ext = build_extension()
    except RuntimeError as exc:
        print(f"reference extension not built: {exc}", file=sys.stderr)
        ext = None
    if ext is not None:
        print("built", ext)


if __name__ == "__main__":
    main()
