"""sl3dpp_gb300: the GB300-native (sm_103a) 3D viscoelastic hot path of sl3dpp.

The compute lives in libsl3dgpu.so (hand-written CUDA behind a C ABI,
include/sl3dgpu.h); this package is its host-side mirror of the reference's
C++ API for the path (band solvers, SurfaceGrid, the degree systems, the 3D
step). Importing the package does not touch the GPU; the first call that
needs the library loads it and fails loudly if it was not built.
"""

from ._lib import Sl3dgpuError, exported_symbols, lib  # noqa: F401

__all__ = ["Sl3dgpuError", "exported_symbols", "lib"]
