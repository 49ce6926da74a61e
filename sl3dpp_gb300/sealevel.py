"""The sea-level equation on the GPU: GRDSolver (include/sl3dpp/SeaLevel.hpp,
src/SeaLevel.cpp), in the solver's non-dimensional units.

`SeaLevelSolver(grid, h, k, l, ht, kt, lt, g, water_density, radius,
rotation, ...)` holds the per-degree load Love numbers (the sums h_u + h_phi
and k_u + k_phi the reference's constructor forms, src/SeaLevel.cpp:163-171),
the tangential and tidal ones, the body's constants and, for rotational
feedback, its rotation constants; `solve_generalised(ocean, ...)` is
GRDSolver::SolveGeneralised (src/SeaLevel.cpp:397-736) for GeneralisedForcing's
channels of the coupled Evolution3D closure (src/Evolution3D.cpp:320-333):
the direct load in and outside the water budget, a layer on the solid
surface, the displacement and potential loads and the tangential traction
(through the channel numbers), the ready displacement, potential, tangential and toroidal
responses, a tide, and the inertia-moment and angular-momentum changes. It
returns the relative sea level change, displacement, potential, tangential
and toroidal potentials on the grid and the Response scalars (with the
angular velocity). Fields and coefficients are torch CUDA tensors (float64
fields in the grid's colatitude-major layout; complex128 (l, m >= 0)
coefficients).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import P_double, SleBody, SleForcing, SleResult, check, lib
from .grid import SurfaceGrid

_FIELDS = ("direct_load", "direct_load_outside", "solid_surface_change", "displacement_load", "potential_load",
           "tangential_traction")
_CHANNEL_NUMBERS = ("h_u", "k_u", "l_u", "h_phi", "k_phi", "l_phi", "h_v", "k_v", "l_v")
_COEFFS = ("displacement_response", "potential_response", "tangential_response", "toroidal_response", "tide")


class SeaLevelSolver:
    def __init__(self, grid: SurfaceGrid, h, k, l=None, ht=None, kt=None, lt=None, g: float = 1.0,
                 water_density: float = 1.0, radius: float = 1.0, rotation: int = 0, omega: float = 0.0,
                 polar_moment: float = 0.0, equatorial_moment: float = 0.0, gravitational_constant: float = 0.0,
                 hc: float = 0.0, kc: float = 0.0, m_u: float = 0.0, m_phi: float = 0.0, m_c: float = 0.0,
                 channel_numbers: dict | None = None):
        """rotation: RotationalFeedback 0 None, 1 Axial, 2 Full, with the
        body's non-dimensional rotation frequency, moments of inertia,
        gravitational constant, centrifugal (h_c, k_c) and inertia-trace
        (m_u, m_phi, m_c) numbers (src/SeaLevel.cpp:194-247).
        channel_numbers: the load channels' own per-degree numbers, keys
        h_u, k_u, l_u (a displacement load), h_phi, k_phi, l_phi (a potential
        load), h_v, k_v, l_v (a tangential traction)."""
        lmax = grid.lmax
        self.grid = grid
        self.arrays = {}
        channel_numbers = dict(channel_numbers or {})
        unknown = set(channel_numbers) - set(_CHANNEL_NUMBERS)
        if unknown:
            raise ValueError(f"unknown channel numbers {sorted(unknown)}")
        named = [("h", h), ("k", k), ("l", l), ("ht", ht), ("kt", kt), ("lt", lt)]
        named += [(n, channel_numbers.get(n)) for n in _CHANNEL_NUMBERS]
        for name, v in named:
            if v is None:
                self.arrays[name] = None
                continue
            a = np.ascontiguousarray(v, dtype=np.float64)
            if a.size < lmax + 1:
                raise ValueError(f"the Love numbers {name} reach degree {a.size - 1}, the grid needs {lmax}")
            self.arrays[name] = a
        if self.arrays["h"] is None or self.arrays["k"] is None:
            raise ValueError("the load Love numbers h and k are required")
        self.g, self.water_density, self.radius = float(g), float(water_density), float(radius)
        self.rotation = (int(rotation), float(omega), float(polar_moment), float(equatorial_moment),
                         float(gravitational_constant), float(hc), float(kc), float(m_u), float(m_phi), float(m_c))

    def solve_generalised(self, ocean: torch.Tensor, rtol: float = 1e-9, max_iterations: int = 1000,
                          anderson_memory: int = 5, inertia_moment_change: float = 0.0,
                          angular_momentum_change=(0.0, 0.0, 0.0), **forcing) -> dict:
        size, ncoef = self.grid.FieldSize(), self.grid.CoefficientSize()
        unknown = set(forcing) - set(_FIELDS) - set(_COEFFS)
        if unknown:
            raise ValueError(f"unknown forcing channels {sorted(unknown)}")

        def field(name, f):
            if f.dtype != torch.float64 or not f.is_cuda or f.numel() != size or not f.is_contiguous():
                raise ValueError(f"the {name} must be a contiguous float64 CUDA field on the grid")
            return f

        field("ocean function", ocean)
        f = SleForcing()
        f.inertia_moment_change = float(inertia_moment_change)
        for i in range(3):
            f.angular_momentum_change[i] = float(angular_momentum_change[i])
        keep = []
        for name in _FIELDS:
            if forcing.get(name) is not None:
                setattr(f, name, field(name, forcing[name]).data_ptr())
        for name in _COEFFS:
            c = forcing.get(name)
            if c is None:
                continue
            if c.dtype != torch.complex128 or not c.is_cuda or c.numel() != ncoef or not c.is_contiguous():
                raise ValueError(f"the {name} must be contiguous complex128 CUDA coefficients of the grid")
            keep.append(c)
            setattr(f, name, c.data_ptr())
        a = self.arrays
        ptr = lambda n: a[n].ctypes.data_as(P_double) if a[n] is not None else None
        body = SleBody(*(ptr(n) for n in ("h", "k", "l", "ht", "kt", "lt")), self.g, self.water_density,
                       self.radius, *self.rotation, *(ptr(n) for n in _CHANNEL_NUMBERS))
        out = {key: torch.empty(size, dtype=torch.float64, device=ocean.device)
               for key in ("sea_level_change", "displacement", "potential", "tangential_potential",
                           "toroidal_potential")}
        res = SleResult()
        stream = torch.cuda.current_stream().cuda_stream
        check(lib().sl3dgpu_sle_solve(self.grid._handle, ctypes.byref(body), ocean.data_ptr(), ctypes.byref(f),
                                      float(rtol), int(max_iterations), int(anderson_memory),
                                      out["sea_level_change"].data_ptr(), out["displacement"].data_ptr(),
                                      out["potential"].data_ptr(), out["tangential_potential"].data_ptr(),
                                      out["toroidal_potential"].data_ptr(), ctypes.byref(res), stream))
        out.update(uniform_shift=res.uniform_shift, error=res.error, iterations=res.iterations,
                   converged=bool(res.converged), angular_velocity=tuple(res.angular_velocity))
        return out
