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
