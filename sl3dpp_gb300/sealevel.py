"""The sea-level equation on the GPU: GRDSolver (include/sl3dpp/SeaLevel.hpp,
src/SeaLevel.cpp) for a direct surface load on a body without rotational
feedback, in the solver's non-dimensional units.

`SeaLevelSolver(grid, h, k, l, g, water_density, radius)` holds the per-degree
load Love numbers (the sums h_u + h_phi and k_u + k_phi the reference's
constructor forms, src/SeaLevel.cpp:163-171; the tangential l optional) and
the body's constants; `solve_generalised(ocean, direct_load)` is
GRDSolver::SolveGeneralised (src/SeaLevel.cpp:397-736) with
GeneralisedForcing's directLoad alone and RotationalFeedback::None: the load
fixed point under Anderson mixing with the water's conservation imposed as a
uniform shift, returning the relative sea level change, displacement,
potential and tangential potential on the grid and the Response scalars.
Fields are torch CUDA tensors (float64, the grid's colatitude-major layout).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import P_double, SleResult, check, lib
from .grid import SurfaceGrid


class SeaLevelSolver:
    def __init__(self, grid: SurfaceGrid, h, k, l=None, g: float = 1.0, water_density: float = 1.0,
                 radius: float = 1.0):
        lmax = grid.lmax
        self.grid = grid
        self.h = np.ascontiguousarray(h, dtype=np.float64)
        self.k = np.ascontiguousarray(k, dtype=np.float64)
        self.l = None if l is None else np.ascontiguousarray(l, dtype=np.float64)
        for name, v in (("h", self.h), ("k", self.k), ("l", self.l)):
            if v is not None and v.size < lmax + 1:
                raise ValueError(f"the Love numbers {name} reach degree {v.size - 1}, the grid needs {lmax}")
        self.g, self.water_density, self.radius = float(g), float(water_density), float(radius)

    def solve_generalised(self, ocean: torch.Tensor, direct_load: torch.Tensor, rtol: float = 1e-9,
                          max_iterations: int = 1000, anderson_memory: int = 5) -> dict:
        size = self.grid.FieldSize()
        for name, f in (("ocean function", ocean), ("direct load", direct_load)):
            if f.dtype != torch.float64 or not f.is_cuda or f.numel() != size or not f.is_contiguous():
                raise ValueError(f"the {name} must be a contiguous float64 CUDA field on the grid")
        out = {key: torch.empty(size, dtype=torch.float64, device=ocean.device)
               for key in ("sea_level_change", "displacement", "potential", "tangential_potential")}
        res = SleResult()
        stream = torch.cuda.current_stream().cuda_stream
        lt = self.l.ctypes.data_as(P_double) if self.l is not None else None
        check(lib().sl3dgpu_sle_solve(self.grid._handle, self.h.ctypes.data_as(P_double),
                                      self.k.ctypes.data_as(P_double), lt, self.g, self.water_density, self.radius,
                                      float(rtol), int(max_iterations), int(anderson_memory), ocean.data_ptr(),
                                      direct_load.data_ptr(), out["sea_level_change"].data_ptr(),
                                      out["displacement"].data_ptr(), out["potential"].data_ptr(),
                                      out["tangential_potential"].data_ptr(), ctypes.byref(res), stream))
        out.update(uniform_shift=res.uniform_shift, error=res.error, iterations=res.iterations,
                   converged=bool(res.converged))
        return out
