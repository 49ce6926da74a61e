"""Synthetic inputs of the measured configurations.

The log-viscosity perturbation delta: a seeded random real spherical-harmonic
field with coefficients a_lm ~ N(0, sigma_l^2), sigma_l^2 proportional to
(l + 1)^-2 for 1 <= l <= L_delta, scaled to a given RMS over the sphere, and
multiplied by a radial indicator that is one between 100 and 670 km depth.
The load: a spherical ice cap of half-angle alpha at the pole, 917 kg m^-3
(SeaLevel.hpp's ice density), thickness growing linearly in time. All inputs
are synthetic, seeded with numpy's default_rng.
"""

from __future__ import annotations

import numpy as np

RHO_ICE = 917.0
EARTH_RADIUS = 6371e3
SECONDS_PER_YEAR = 3.15576e7


def real_index(l: int, m: int) -> int:
    return l * (l + 1) // 2 + m


def delta_coefficients(lmax: int, ldelta: int, rms: float, seed: int) -> np.ndarray:
    """Real spin-0 coefficients (l(l+1)/2 + m layout) of the delta pattern."""
    rng = np.random.default_rng(seed)
    c = np.zeros((lmax + 1) * (lmax + 2) // 2, dtype=np.complex128)
    for l in range(1, min(ldelta, lmax) + 1):
        s = 1.0 / (l + 1)
        c[real_index(l, 0)] = rng.normal(0.0, s)
        for m in range(1, l + 1):
            c[real_index(l, m)] = complex(rng.normal(0.0, s / np.sqrt(2.0)), rng.normal(0.0, s / np.sqrt(2.0)))
    # mean square over the sphere: (1 / 4 pi) sum over every order, m < 0 the twins
    ms = 0.0
    for l in range(lmax + 1):
        ms += abs(c[real_index(l, 0)]) ** 2 + 2.0 * sum(abs(c[real_index(l, m)]) ** 2 for m in range(1, l + 1))
    ms /= 4.0 * np.pi
    return c * (rms / np.sqrt(ms)) if ms > 0 else c


def land_field_coefficients(lmax: int, seed: int, ldegree: int = 12) -> np.ndarray:
    """A seeded smooth field (degrees 1..ldegree, amplitude 1/(l + 1)) whose
    upper part becomes land: real spin-0 coefficients."""
    rng = np.random.default_rng(seed)
    c = np.zeros((lmax + 1) * (lmax + 2) // 2, dtype=np.complex128)
    for l in range(1, min(lmax, ldegree) + 1):
        for m in range(l + 1):
            a = rng.standard_normal() + (1j * rng.standard_normal() if m else 0.0)
            c[real_index(l, m)] = a / (l + 1)
    return c


def ocean_from_field(field: np.ndarray, weights: np.ndarray, nphi: int, land_fraction: float = 0.3) -> np.ndarray:
    """The ocean function (1 ocean, 0 land) of thresholding a field on a
    grid so that its largest values cover `land_fraction` of the area."""
    area = np.repeat(np.asarray(weights)[:, None], nphi, axis=1).ravel()
    order = np.argsort(np.asarray(field).ravel(), kind="stable")[::-1]
    covered = np.cumsum(area[order]) / area.sum()
    land = np.zeros(area.size)
    land[order[covered <= land_fraction]] = 1.0
    return 1.0 - land


def delta_indicator(radius_nd: np.ndarray, top_depth: float = 100e3, bottom_depth: float = 670e3,
                    surface: float = EARTH_RADIUS) -> np.ndarray:
    """1 where a (non-dimensional) radius lies between the two depths."""
    r = radius_nd * surface
    return ((r > surface - bottom_depth) & (r < surface - top_depth)).astype(np.float64)


def delta_samples(pattern_field: np.ndarray, radius_nd: np.ndarray) -> np.ndarray:
    """delta over every node's grid from the pattern's values on one grid."""
    ind = delta_indicator(radius_nd)
    return (ind[:, None] * pattern_field.ravel()[None, :]).ravel()


def cap_field(theta: np.ndarray, nphi: int, alpha_deg: float, thickness: float) -> np.ndarray:
    """Surface density (kg m^-2) of a polar cap on a grid, colatitude-major."""
    ring = np.where(theta < np.radians(alpha_deg), RHO_ICE * thickness, 0.0)
    return np.repeat(ring, nphi)


def legacy_deck_layers(knots: np.ndarray, max_element: float = 20e3):
    """Layers from a legacy sl3d 1D model's knots (rows r [m], rho [kg m^-3],
    kappa [GPa], mu [GPa], log10 viscosity [Pa s], 0 meaning none; a radius
    repeated at a discontinuity): one layer per interval of non-zero
    thickness, its fields linear between the knots, fluid where the shear
    modulus vanishes at both ends, the interval's viscosity from its lower
    knot, and elements no wider than max_element. The reference reads the
    same format (Deck::ReadLegacySl3d) and interpolates by natural cubic
    splines; with knots 20-40 km apart the linear form differs from it by
    far less than the physical comparisons made with it."""
    from .viscoelastic3d import Layer

    out = []
    for a, b in zip(knots[:-1], knots[1:]):
        if not b[0] > a[0]:
            continue
        fluid = a[3] == 0.0 and b[3] == 0.0
        out.append(Layer(r0=a[0], r1=b[0], fluid=int(fluid),
                         elements=max(1, int(np.ceil((b[0] - a[0]) / max_element))),
                         rho0=a[1], rho1=b[1], kappa0=a[2] * 1e9, kappa1=b[2] * 1e9,
                         mu0=0.0 if fluid else a[3] * 1e9, mu1=0.0 if fluid else b[3] * 1e9,
                         viscosity=10.0 ** a[4] if a[4] > 0.0 else 0.0, kelvin_fraction=0.0, kelvin_viscosity=0.0))
    return (Layer * len(out))(*out)


def fortran_gate_delta(theta: np.ndarray, nphi: int) -> np.ndarray:
    """The Fortran visco_test's lateral pattern s = s(r) exp(0.3 (Y_2,-2 +
    Y_2,2)) as a log-viscosity perturbation on a grid: delta = -0.6 c22
    sin^2 theta cos 2 phi, c22 = sqrt(15 / (2 pi)) / 4, as the reference's
    gate writes it (benchmarks/fortran_gate.cpp)."""
    c22 = 0.25 * np.sqrt(15.0 / (2.0 * np.pi))
    phi = 2.0 * np.pi * np.arange(nphi) / nphi
    return (-0.6 * c22 * np.sin(theta)[:, None] ** 2 * np.cos(2.0 * phi)[None, :]).ravel()


def fortran_gate_load_rate(lmax: int) -> np.ndarray:
    """The visco_test's zonal load rate per degree, kg m^-2 s^-1 (degree 0 none):
    exp(-2 pi (l + 1) / 10.5) sqrt((2 l + 1) / 4 pi) 5515 / 30 yr."""
    l = np.arange(lmax + 1, dtype=np.float64)
    rate = np.exp(-2.0 * np.pi * (l + 1) / 10.5) * np.sqrt((2 * l + 1) / (4 * np.pi)) * 5515.0 / (30 * SECONDS_PER_YEAR)
    rate[0] = 0.0
    return rate
