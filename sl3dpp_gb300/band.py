"""The banded solvers of the degree systems, on the GPU.

Mirrors include/sl3dpp/detail/BandSolvers.hpp:24-49 (BandCholeskyFactor,
BandCholeskySolve, BandLuFactor, BandLuSolve): LAPACK band storage, zero-based
pivots, LAPACK-style info returns; each call runs the batched sm_103a kernels
on one system through the C ABI.
"""

from __future__ import annotations

import ctypes

import numpy as np

from ._lib import P_double, P_int, check, lib


def _f64(a: np.ndarray) -> np.ndarray:
    if a.dtype != np.float64 or not a.flags.c_contiguous or not a.flags.writeable:
        raise ValueError("expected a writeable contiguous float64 array")
    return a


def BandCholeskyFactor(ab: np.ndarray, n: int, kd: int) -> int:
    """A = U^T U in place (dpbtrf "U"); 0 or k + 1 for a non-positive minor."""
    _f64(ab)
    if ab.size < (kd + 1) * n:
        raise ValueError("ab holds fewer than (kd + 1) n values")
    return check(lib().sl3dgpu_band_cholesky_factor(ab.ctypes.data_as(P_double), n, kd))


def BandCholeskySolve(ab: np.ndarray, n: int, kd: int, b: np.ndarray, nrhs: int) -> None:
    """Overwrites the column-major n x nrhs b with A^-1 b (dpbtrs)."""
    _f64(b)
    ab = np.ascontiguousarray(ab, dtype=np.float64)
    check(lib().sl3dgpu_band_cholesky_solve(ab.ctypes.data_as(P_double), n, kd,
                                            b.ctypes.data_as(P_double), nrhs))


def BandLuFactor(ab: np.ndarray, n: int, kl: int, ku: int, pivots: np.ndarray) -> int:
    """A = P L U in place (dgbtrf); pivots zero-based; 0 or k + 1 for U(k, k) = 0."""
    _f64(ab)
    if pivots.dtype != np.int32 or pivots.size < n:
        raise ValueError("pivots must be an int32 array of n entries")
    return check(lib().sl3dgpu_band_lu_factor(ab.ctypes.data_as(P_double), n, kl, ku,
                                              pivots.ctypes.data_as(P_int)))


def BandLuSolve(ab: np.ndarray, n: int, kl: int, ku: int, pivots: np.ndarray, b: np.ndarray,
                nrhs: int) -> None:
    """Overwrites the column-major n x nrhs b with A^-1 b (dgbtrs "N")."""
    _f64(b)
    ab = np.ascontiguousarray(ab, dtype=np.float64)
    pivots = np.ascontiguousarray(pivots, dtype=np.int32)
    check(lib().sl3dgpu_band_lu_solve(ab.ctypes.data_as(P_double), n, kl, ku,
                                      pivots.ctypes.data_as(P_int),
                                      b.ctypes.data_as(P_double), nrhs))
