"""Build recipe of the oracle (test infrastructure only).

Compiles the CPU FP64 restatement under oracle/ into oracle/_build/liboracle.so
with g++ (OpenMP). Only tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline leg load it, as the checker.
"""

from __future__ import annotations

import os
import pathlib
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIBRARY = BUILD / "liboracle.so"


def _sources() -> list[pathlib.Path]:
    # the oracle's own restatement alone: it shares no source with the library
    return sorted(HERE.glob("*.cpp"))


def _stale(sources: list[pathlib.Path]) -> bool:
    if not LIBRARY.exists():
        return True
    built = LIBRARY.stat().st_mtime
    inputs = sources + list(HERE.glob("*.h")) + list(HERE.glob("*.hpp")) + [pathlib.Path(__file__)]
    return any(p.stat().st_mtime > built for p in inputs)


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    sources = _sources()
    if not force and not _stale(sources):
        return LIBRARY
    BUILD.mkdir(exist_ok=True)
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++23", "-fPIC", "-shared", "-fopenmp", "-I", str(HERE),
           *map(str, sources), "-o", str(tmp)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"building the oracle failed:\n{' '.join(cmd)}\n{result.stderr}")
    os.replace(tmp, LIBRARY)
    if verbose:
        print(f"built {LIBRARY}", file=sys.stderr)
    return LIBRARY


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
