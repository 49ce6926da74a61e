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
angular velocity). `solve_nonlinear(state, ...)` is GRDSolver::
SolveNonlinear (src/SeaLevel.cpp:970-1289), the solve with migrating
shorelines from a `State` (ice thickness, sea level, flotation's ocean
function, a held land mask); `make_state` is MakeState (:279-300). Fields
and coefficients are torch CUDA tensors (float64 fields in the grid's
colatitude-major layout; complex128 (l, m >= 0) coefficients; uint8 masks).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import P_double, SleBody, SleForcing, SleNonlinearForcing, SleResult, SleState, check, lib
from .grid import SurfaceGrid

_FIELDS = ("direct_load", "direct_load_outside", "solid_surface_change", "displacement_load", "potential_load",
           "tangential_traction")
_CHANNEL_NUMBERS = ("h_u", "k_u", "l_u", "h_phi", "k_phi", "l_phi", "h_v", "k_v", "l_v")
_COEFFS = ("displacement_response", "potential_response", "tangential_response", "toroidal_response", "tide")


_NONLINEAR_FIELDS = ("ice_thickness_change", "direct_load", "direct_load_outside", "solid_surface_change",
                     "dynamic_sea_level_change")
_NONLINEAR_COEFFS = ("displacement_response", "potential_response", "tangential_response", "toroidal_response",
                     "tide")
_UNSET = object()


class State:
    """GRDSolver::State on the device: the ice thickness, the sea level (the
    sea surface over the solid surface), the ocean function and the land
    held at C = 0 (None: none)."""

    def __init__(self, ice_thickness, sea_level, ocean_function, forced_land=None):
        self.ice_thickness, self.sea_level, self.ocean_function = ice_thickness, sea_level, ocean_function
        self.forced_land = forced_land


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

    def _body(self):
        a = self.arrays
        ptr = lambda n: a[n].ctypes.data_as(P_double) if a[n] is not None else None
        return SleBody(*(ptr(n) for n in ("h", "k", "l", "ht", "kt", "lt")), self.g, self.water_density,
                       self.radius, *self.rotation, *(ptr(n) for n in _CHANNEL_NUMBERS))

    def _field(self, name, f):
        if f.dtype != torch.float64 or not f.is_cuda or f.numel() != self.grid.FieldSize() or not f.is_contiguous():
            raise ValueError(f"the {name} must be a contiguous float64 CUDA field on the grid")
        return f

    def _mask(self, name, m):
        if m is None:
            return None
        if m.dtype != torch.uint8 or not m.is_cuda or m.numel() != self.grid.FieldSize() or not m.is_contiguous():
            raise ValueError(f"the {name} must be a contiguous uint8 CUDA mask on the grid")
        return m

    def make_state(self, ice_thickness: torch.Tensor, sea_level: torch.Tensor, ice_density: float,
                   forced_land: torch.Tensor | None = None) -> State:
        """MakeState (src/SeaLevel.cpp:279-300): the ocean function by
        flotation, rho_w SL - rho_i I > 0 where no land is held."""
        self._field("ice thickness", ice_thickness)
        self._field("sea level", sea_level)
        self._mask("land held", forced_land)
        ocean = torch.empty_like(ice_thickness)
        stream = torch.cuda.current_stream().cuda_stream
        check(lib().sl3dgpu_sle_flotation(ice_thickness.numel(), self.water_density, float(ice_density),
                                          ice_thickness.data_ptr(), sea_level.data_ptr(),
                                          None if forced_land is None else forced_land.data_ptr(), ocean.data_ptr(),
                                          stream))
        return State(ice_thickness, sea_level, ocean, forced_land)

    def solve_nonlinear(self, state: State, ice_density: float, rtol: float = 1e-9, max_iterations: int = 50,
                        inertia_moment_change: float = 0.0, forced_land=_UNSET, **forcing) -> dict:
        """SolveNonlinear: the relative sea level change, displacement,
        potential, tangential and toroidal potentials, the final state's sea
        level and ocean function, the carried load's coefficients and the
        Response scalars. forced_land: the land held at this solve (None:
        none held); left out, the state's."""
        size, ncoef = self.grid.FieldSize(), self.grid.CoefficientSize()
        unknown = set(forcing) - set(_NONLINEAR_FIELDS) - set(_NONLINEAR_COEFFS)
        if unknown:
            raise ValueError(f"unknown forcing channels {sorted(unknown)}")
        st = SleState(self._field("ice thickness", state.ice_thickness).data_ptr(),
                      self._field("sea level", state.sea_level).data_ptr(),
                      self._field("ocean function", state.ocean_function).data_ptr(),
                      None if state.forced_land is None else self._mask("land held", state.forced_land).data_ptr())
        f = SleNonlinearForcing()
        f.inertia_moment_change = float(inertia_moment_change)
        if forced_land is not _UNSET:
            f.hold_land = 1
            f.forced_land = None if forced_land is None else self._mask("land held", forced_land).data_ptr()
        for name in _NONLINEAR_FIELDS:
            if forcing.get(name) is not None:
                setattr(f, name, self._field(name, forcing[name]).data_ptr())
        for name in _NONLINEAR_COEFFS:
            c = forcing.get(name)
            if c is None:
                continue
            if c.dtype != torch.complex128 or not c.is_cuda or c.numel() != ncoef or not c.is_contiguous():
                raise ValueError(f"the {name} must be contiguous complex128 CUDA coefficients of the grid")
            setattr(f, name, c.data_ptr())
        body = self._body()
        dev = state.ice_thickness.device
        out = {key: torch.empty(size, dtype=torch.float64, device=dev)
               for key in ("sea_level_change", "displacement", "potential", "tangential_potential",
                           "toroidal_potential", "sea_level", "ocean_function")}
        out["load_coefficients"] = torch.empty(ncoef, dtype=torch.complex128, device=dev)
        res = SleResult()
        stream = torch.cuda.current_stream().cuda_stream
        check(lib().sl3dgpu_sle_solve_nonlinear(
            self.grid._handle, ctypes.byref(body), float(ice_density), ctypes.byref(st), ctypes.byref(f), float(rtol),
            int(max_iterations), *(out[k].data_ptr() for k in ("sea_level_change", "displacement", "potential",
                                                                "tangential_potential", "toroidal_potential",
                                                                "sea_level", "ocean_function", "load_coefficients")),
            ctypes.byref(res), stream))
        out.update(uniform_shift=res.uniform_shift, error=res.error, iterations=res.iterations,
                   converged=bool(res.converged), angular_velocity=tuple(res.angular_velocity))
        return out
