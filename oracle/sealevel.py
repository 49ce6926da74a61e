"""The oracle's sea-level equation: a numpy restatement of GRDSolver::
SolveGeneralised (src/SeaLevel.cpp:397-736) for a direct surface load on a
body without rotational feedback, and of the plain Anderson mixer it runs
(include/sl3dpp/detail/AndersonMixer.hpp:65-219). Test infrastructure: the
checker the GPU solver (sl3dgpu_sle_solve) is compared with; it takes the
grid's transforms and quadrature as arguments.

Parity unpinned against the reference itself: the reference's own tests for
this function (tests/TestSeaLevel.cpp:135-206) read a Love-number file and an
analytic ice state; the tests here check the same structural identities (the
rigid-earth eustatic limit, the ocean gaining the mass the load lost) on
synthetic Love numbers, plus agreement of the two implementations.
"""

from __future__ import annotations

import numpy as np


class AndersonMixer:
    """AndersonMixer::Update (AndersonMixer.hpp:65-219): the first call takes
    the image, later ones the least-squares mix of `memory` difference columns
    (Gram matrix by columns, minimum-norm solve with the machine-precision cut
    of dgelss's rcond < 0)."""

    def __init__(self, memory: int):
        self.memory = memory
        self.count = 0
        self.slot = 0
        self.x_prev = None

    def update(self, x: np.ndarray, gx: np.ndarray) -> np.ndarray:
        if self.memory <= 0:
            return gx.copy()
        if self.x_prev is None:
            n = x.size
            self.dG = np.zeros((self.memory, n))
            self.dF = np.zeros((self.memory, n))
            self.gram = np.zeros((self.memory, self.memory))
            self.x_prev = x.copy()
            self.f_prev = gx - x
            return gx.copy()
        slot = self.slot
        m = min(self.count + 1, self.memory)
        f = gx - x
        self.dF[slot] = f - self.f_prev
        self.dG[slot] = (x - self.x_prev) + self.dF[slot]
        self.x_prev = x.copy()
        self.f_prev = f
        column = self.dF[:m] @ self.dF[slot]
        rhs = self.dF[:m] @ f
        self.count = m
        self.slot = (slot + 1) % self.memory
        self.gram[slot, :m] = column
        self.gram[:m, slot] = column
        a = self.gram[:m, :m]
        # symmetric: singular values are the eigenvalues' magnitudes
        lam, v = np.linalg.eigh(0.5 * (a + a.T))
        cut = np.finfo(float).eps * np.max(np.abs(lam)) if lam.size else 0.0
        keep = np.abs(lam) > cut
        gamma = v[:, keep] @ ((v[:, keep].T @ rhs) / lam[keep])
        return gx - gamma @ self.dG[:m]


def solve_generalised(synthesise, expand, integrate, h, k, lt, g, water_density, radius, ocean, direct_load=None,
                      rtol=1e-9, max_iterations=1000, anderson_memory=5, direct_load_outside=None,
                      solid_surface_change=None, displacement_response=None, potential_response=None,
                      tangential_response=None, toroidal_response=None, tide=None, ht=None, kt=None, lt_tide=None):
    """The load fixed point of the sea-level equation (SeaLevel.cpp:397-736
    with RotationalFeedback::None) for the channels the coupled Evolution3D
    closure uses. synthesise(coeffs) and expand(field) are the grid's real
    transforms in the reference's (l, m >= 0) layout, integrate(field) its
    quadrature over the unit sphere."""
    h = np.asarray(h, dtype=np.float64)
    k = np.asarray(k, dtype=np.float64)
    lmax = h.size - 1
    degree = np.concatenate([np.full(l + 1, l) for l in range(lmax + 1)])
    ncoef = degree.size
    size = ocean.size
    out = {"uniform_shift": 0.0, "iterations": 0, "error": 0.0, "converged": True}
    nz = lambda a: a is not None and np.max(np.abs(a)) > 0.0
    # the toroidal potential is carried, whatever else is solved (:561-563)
    toroidal = synthesise(toroidal_response) if toroidal_response is not None else np.zeros(size)
    any_static = nz(displacement_response) or nz(potential_response) or nz(tide) or nz(solid_surface_change)
    any_tan = nz(displacement_response) or nz(potential_response) or nz(tangential_response) or nz(tide)
    if not (nz(direct_load) or nz(direct_load_outside) or any_static or any_tan):
        zeros = np.zeros(size)
        out.update(sea_level_change=zeros, displacement=zeros, potential=zeros, tangential_potential=zeros,
                   toroidal_potential=toroidal)
        return out
    zc = np.zeros(ncoef, dtype=np.complex128)
    static_disp, static_grav, static_tan = zc.copy(), zc.copy(), zc.copy()
    if nz(displacement_response):
        static_disp += displacement_response
    if nz(potential_response):
        static_grav += potential_response
    if nz(tangential_response):
        static_tan += tangential_response
    if nz(tide):  # :533-545
        lt_t = np.zeros(lmax + 1) if lt_tide is None else np.array(lt_tide, dtype=np.float64)
        ht_, kt_ = np.array(ht, dtype=np.float64), np.array(kt, dtype=np.float64)
        ht_[0] = kt_[0] = lt_t[0] = 0.0
        static_disp += ht_[degree] * tide
        static_grav += kt_[degree] * tide
        static_tan += lt_t[degree] * tide
    static_slc = -(static_disp + static_grav / g)  # :590-600
    if nz(tide):
        static_slc -= tide / g
    if nz(solid_surface_change):
        static_slc -= expand(solid_surface_change)
    surface = lambda f: radius * radius * integrate(f)  # IntegrateSurface
    ocean_area = surface(ocean)
    per_area = 1.0 / ocean_area if ocean_area > 0.0 else 0.0  # InverseOceanArea
    direct = np.zeros(size)
    mean_slc = 0.0
    if direct_load is not None:
        direct = direct_load.copy()
        mean_slc = -surface(direct_load) * per_area / water_density
    if direct_load_outside is not None:
        direct = direct + direct_load_outside
    slc_factor = -(h + k / g)
    load_lm = expand(direct + water_density * ocean * mean_slc)
    mixer = AndersonMixer(anderson_memory)
    prev = None
    slc = np.zeros(size)
    err = np.inf
    converged = False
    count = 0
    shift = 0.0
    while count < max_iterations:
        lm = slc_factor[degree] * load_lm
        if any_static:
            lm = lm + static_slc
        slc = synthesise(lm)
        shift = mean_slc - surface(ocean * slc) * per_area
        slc = slc + shift
        ocean_slc = ocean * slc
        if prev is not None:
            scale = np.max(np.abs(ocean_slc))
            err = np.max(np.abs(ocean_slc - prev)) / scale if scale > 0.0 else 0.0
            if err <= rtol:
                converged = True
                break
        prev = ocean_slc
        new_lm = expand(direct + water_density * prev)
        mixed = mixer.update(load_lm.view(np.float64), new_lm.view(np.float64))
        load_lm = mixed.view(np.complex128)
        count += 1
    tan = np.zeros(lmax + 1) if lt is None else np.array(lt, dtype=np.float64)
    tan[0] = 0.0
    out.update(sea_level_change=slc, displacement=synthesise(h[degree] * load_lm + static_disp),
               potential=synthesise(k[degree] * load_lm + static_grav),
               tangential_potential=synthesise(tan[degree] * load_lm + static_tan), toroidal_potential=toroidal,
               uniform_shift=shift, iterations=count, error=err, converged=converged)
    return out
