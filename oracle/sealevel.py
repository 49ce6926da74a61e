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


def solve_generalised(synthesise, expand, integrate, h, k, lt, g, water_density, radius, ocean, direct_load,
                      rtol=1e-9, max_iterations=1000, anderson_memory=5):
    """The load fixed point of the sea-level equation (SeaLevel.cpp:563-713
    with no static terms, tide, layer or rotation). synthesise(coeffs) and
    expand(field) are the grid's real transforms in the reference's (l, m >= 0)
    layout, integrate(field) its quadrature over the unit sphere."""
    h = np.asarray(h, dtype=np.float64)
    k = np.asarray(k, dtype=np.float64)
    lmax = h.size - 1
    degree = np.concatenate([np.full(l + 1, l) for l in range(lmax + 1)])
    out = {"uniform_shift": 0.0, "iterations": 0, "error": 0.0, "converged": True}
    zeros = np.zeros_like(direct_load)
    if np.max(np.abs(direct_load)) == 0.0:  # no forcing (:562)
        out.update(sea_level_change=zeros, displacement=zeros, potential=zeros, tangential_potential=zeros)
        return out
    surface = lambda f: radius * radius * integrate(f)  # IntegrateSurface
    ocean_area = surface(ocean)
    per_area = 1.0 / ocean_area if ocean_area > 0.0 else 0.0  # InverseOceanArea
    mean_slc = -surface(direct_load) * per_area / water_density
    slc_factor = -(h + k / g)
    load_lm = expand(direct_load + water_density * ocean * mean_slc)
    mixer = AndersonMixer(anderson_memory)
    prev = None
    slc = zeros
    err = np.inf
    converged = False
    count = 0
    shift = 0.0
    while count < max_iterations:
        slc = synthesise(slc_factor[degree] * load_lm)
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
        new_lm = expand(direct_load + water_density * prev)
        mixed = mixer.update(load_lm.view(np.float64), new_lm.view(np.float64))
        load_lm = mixed.view(np.complex128)
        count += 1
    tan = np.zeros(lmax + 1) if lt is None else np.array(lt, dtype=np.float64)
    tan[0] = 0.0
    out.update(sea_level_change=slc, displacement=synthesise(h[degree] * load_lm),
               potential=synthesise(k[degree] * load_lm), tangential_potential=synthesise(tan[degree] * load_lm),
               uniform_shift=shift, iterations=count, error=err, converged=converged)
    return out
