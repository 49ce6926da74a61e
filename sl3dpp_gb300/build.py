"""Build recipe of the sl3dgpu shared library (CUDA for sm_103a plus C++ host code).

Compiles every translation unit under csrc/ in parallel with nvcc (one
-gencode, sm_103a only) and links libsl3dgpu.so into this package directory,
in tree. No CMake; a minute or two on the target's cores.
"""

from __future__ import annotations

import concurrent.futures
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIBRARY = HERE / "libsl3dgpu.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++20", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", str(INCLUDE), "-I", str(CSRC)]
CXX_FLAGS = ["-O2", "-std=c++23", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC)]


def _nvcc() -> str:
    found = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return found


def _sources() -> list[pathlib.Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("host/*.cpp")))


def _stale(sources: list[pathlib.Path]) -> bool:
    if not LIBRARY.exists():
        return True
    built = LIBRARY.stat().st_mtime
    inputs = sources + list(CSRC.rglob("*.cuh")) + list(CSRC.rglob("*.hpp")) + list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > built for p in inputs)


def _compile(src: pathlib.Path) -> pathlib.Path:
    obj = BUILD / (src.relative_to(CSRC).as_posix().replace("/", "_") + ".o")
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXX_FLAGS, "-I", "/usr/local/cuda/include", "-c", str(src), "-o", str(obj)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"compiling {src.name} failed:\n{' '.join(cmd)}\n{result.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """Compile and link libsl3dgpu.so if any source is newer than it."""
    sources = _sources()
    if not force and not _stale(sources):
        return LIBRARY
    BUILD.mkdir(exist_ok=True)
    workers = max(1, min(len(sources), os.cpu_count() or 1))
    with concurrent.futures.ThreadPoolExecutor(workers) as pool:
        objects = list(pool.map(_compile, sources))
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objects), "-lcudart"]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"linking failed:\n{' '.join(cmd)}\n{result.stderr}")
    os.replace(tmp, LIBRARY)
    if verbose:
        print(f"built {LIBRARY}", file=sys.stderr)
    return LIBRARY


APP = HERE / "sl3d"
APP_DIR = CSRC / "app"


def build_app(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """The sl3d front end (csrc/app, host C++ over the C ABI) linked against
    libsl3dgpu.so beside it (found through $ORIGIN)."""
    library = build(verbose=verbose)
    sources = sorted(APP_DIR.glob("*.cpp"))
    inputs = sources + list(APP_DIR.glob("*.hpp")) + list(INCLUDE.glob("*.h")) + [library]
    if not force and APP.exists() and all(p.stat().st_mtime <= APP.stat().st_mtime for p in inputs):
        return APP
    cuda = pathlib.Path(_nvcc()).resolve().parent.parent
    tmp = APP.with_suffix(".tmp")
    cmd = ["g++", "-O2", "-std=c++23", "-I", str(INCLUDE), "-I", str(cuda / "include"), *map(str, sources),
           "-o", str(tmp), "-L", str(HERE), "-lsl3dgpu", "-Wl,-rpath,$ORIGIN", "-L", str(cuda / "lib64"),
           "-lcudart"]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"building sl3d failed:\n{' '.join(cmd)}\n{result.stderr}")
    os.replace(tmp, APP)
    if verbose:
        print(f"built {APP}", file=sys.stderr)
    return APP


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    build_app(force="--force" in sys.argv, verbose=True)
