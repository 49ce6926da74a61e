"""The oracle's ocean closure: a restatement of Evolution3D's Coupled::Closure
(src/Evolution3D.cpp:296-339, frozen and migrating shorelines) and of the
pieces it uses
-- GRDSolver's constructor constants (src/SeaLevel.cpp:142-247),
TotalLoadCoefficients (:237-249 of Evolution3D.cpp) and
CentrifugalCoefficients (src/SeaLevel.cpp:249-258) -- around the numpy
sea-level solve of oracle/sealevel.py. Test infrastructure: the checker the
GPU's coupled step (sl3dgpu_v3d_step_ocean) is compared with.

The oracle's 3D step (oracle_step.cpp) calls `closure(t, love, U, V, phi,
inertia)` in every pass after its degree solves, with the stage's end time,
the pass flavour's effective Love numbers and the responses' surface
coefficients and inertia moment; it gets back the pass's load and tide
channels. Everything is in the 3D operator's model units.
"""

from __future__ import annotations

import numpy as np

from oracle import sealevel


class OceanClosure:
    """The closure of one operator's passes over an ocean with frozen
    shorelines. `transforms` = (synthesise, expand, integrate) of the
    sea-level grid (real fields, (l, m >= 0) coefficients, the unit-sphere
    quadrature); `body` = dict(radius, g, G, length, mass, time) of the
    model; the SI constants are SeaLevelParameters' (include/sl3dpp/
    SeaLevel.hpp:54-68)."""

    def __init__(self, lmax, transforms, body, ocean, rotation=1, water_density=1000.0,
                 rotation_frequency=7.27220521664304e-05, polar_moment=8.0359e37, equatorial_moment=8.0096e37,
                 rtol=1e-10, max_iterations=200, anderson_memory=5):
        self.lmax = lmax
        self.synthesise, self.expand, self.integrate = transforms
        self.ocean = np.asarray(ocean, dtype=np.float64)
        density = body["mass"] / body["length"] ** 3
        moment = body["mass"] * body["length"] ** 2
        self.radius, self.g, self.G = body["radius"], body["g"], body["G"]
        self.water_density = water_density / density
        self.rotation = rotation
        self.omega = rotation_frequency * body["time"]
        self.polar, self.equatorial = polar_moment / moment, equatorial_moment / moment
        self.rtol, self.max_iterations, self.anderson_memory = rtol, max_iterations, anderson_memory
        self.loads = None  # ((t0, field0), (t1, field1)) of the running step
        self.last = None   # the last solve's outputs

    def set_step_loads(self, t0, load0, t1, load1):
        """The direct (non-ocean) load fields at the step's two ends."""
        self.loads = ((float(t0), np.asarray(load0, dtype=np.float64)), (float(t1), np.asarray(load1, dtype=np.float64)))

    def direct_load(self, t):
        """detail::AtStage: the two ends' fields combined linearly in the
        stage's position t."""
        (t0, a), (t1, b) = self.loads
        c = 1.0 if t1 == t0 else (t - t0) / (t1 - t0)  # a zero-length step: its end's load
        return (1.0 - c) * a + c * b

    def centrifugal(self, omega):
        """CentrifugalCoefficients: (0, 0), (2, 0) and (2, 1) of the
        potential of the angular velocity change."""
        psi = np.zeros((self.lmax + 1) * (self.lmax + 2) // 2, dtype=np.complex128)
        if not self.rotation:
            return psi
        a, w = self.radius, self.omega
        rotation = np.sqrt(4.0 * np.pi / 15.0) * w * a * a
        psi[0] = -np.sqrt(16.0 * np.pi / 9.0) * w * a * a * omega[2]
        psi[3] = np.sqrt(16.0 * np.pi / 45.0) * w * a * a * omega[2]
        psi[4] = -complex(rotation * omega[0], -rotation * omega[1]) / np.sqrt(2.0)  # ComplexFromRealPair, m = 1
        return psi

    def __call__(self, t, love, U, V, phi, inertia):
        L = self.lmax
        n = L + 1
        h, k, l, ht, kt, lt = (love[i * n:(i + 1) * n] for i in range(6))
        hc, kc, m, mc = love[6 * n:6 * n + 4]
        direct = self.direct_load(t)
        out = sealevel.solve_generalised(
            self.synthesise, self.expand, self.integrate, h, k, l, self.g, self.water_density, self.radius,
            self.ocean, direct_load=direct, rtol=self.rtol, max_iterations=self.max_iterations,
            anderson_memory=self.anderson_memory, displacement_response=U, potential_response=phi,
            tangential_response=V, ht=ht, kt=kt, lt_tide=lt, rotation=self.rotation, omega=self.omega,
            polar=self.polar, equatorial=self.equatorial, G=self.G, hc=hc, kc=kc, m_u=m, m_phi=0.0, m_c=mc,
            inertia_moment_change=inertia)
        self.last = out
        # TotalLoadCoefficients: the direct load and the ocean's
        sigma = self.expand(direct + self.water_density * self.ocean * out["sea_level_change"])
        return sigma, self.centrifugal(out["angular_velocity"])


class MigratingClosure(OceanClosure):
    """The closure under migrating shorelines (Coupled::Closure's migrating
    branch, src/Evolution3D.cpp:308-319): each pass solves the nonlinear
    sea-level equation (oracle/sealevel.py solve_nonlinear, GRDSolver::
    SolveNonlinear) from the background state, the stage's ice thickness
    change from the background's and the responses entering as ready
    channels; the pass's load channel is the solve's carried load (grounded
    ice, water and direct loads relative to the background), its tide
    channel the centrifugal potential. `state` = dict(ice, sea_level,
    forced_land) in model units; its ocean function is flotation's
    (CheckMigratingStart, src/Shorelines.cpp:9-35)."""

    def __init__(self, lmax, transforms, body, state, ice_density=917.0, max_nonlinear_iterations=50, **kw):
        density = body["mass"] / body["length"] ** 3
        self.ice_density = ice_density / density
        super().__init__(lmax, transforms, body, np.zeros_like(np.asarray(state["ice"], dtype=np.float64)), **kw)
        ice = np.asarray(state["ice"], dtype=np.float64)
        sea = np.asarray(state["sea_level"], dtype=np.float64)
        land = state.get("forced_land")
        self.ocean = sealevel.flotation(ice, sea, self.water_density, self.ice_density, land)
        self.state = dict(ice=ice, sea_level=sea, ocean=self.ocean, forced_land=land)
        self.max_nonlinear_iterations = max_nonlinear_iterations
        self.ice = None
        self.current_ocean = self.ocean.copy()

    def set_step_ice(self, t0, ice0, t1, ice1):
        """The ice thickness at the step's two ends (model length)."""
        self.ice = ((float(t0), np.asarray(ice0, dtype=np.float64)), (float(t1), np.asarray(ice1, dtype=np.float64)))

    def _ice_at(self, t):
        (t0, a), (t1, b) = self.ice
        c = 1.0 if t1 == t0 else (t - t0) / (t1 - t0)
        return (1.0 - c) * a + c * b

    def __call__(self, t, love, U, V, phi, inertia):
        n = self.lmax + 1
        h, k, l, ht, kt, lt = (love[i * n:(i + 1) * n] for i in range(6))
        hc, kc, m, mc = love[6 * n:6 * n + 4]
        direct = self.direct_load(t) if self.loads is not None else None
        out = sealevel.solve_nonlinear(
            self.synthesise, self.expand, self.integrate, h, k, l, self.g, self.water_density, self.ice_density,
            self.radius, self.state, ice_change=self._ice_at(t) - self.state["ice"], direct_load=direct,
            displacement_response=U, potential_response=phi, tangential_response=V, ht=ht, kt=kt, lt_tide=lt,
            rotation=self.rotation, omega=self.omega, polar=self.polar, equatorial=self.equatorial, G=self.G, hc=hc,
            kc=kc, m_u=m, m_phi=0.0, m_c=mc, inertia_moment_change=inertia, rtol=self.rtol,
            max_iterations=self.max_nonlinear_iterations)
        self.last = out
        self.current_ocean = out["ocean"]
        return out["load_coefficients"], self.centrifugal(out["angular_velocity"])
