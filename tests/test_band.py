"""Banded factorisations and solves: the oracle against LAPACK (the pin), and
the GPU kernels against both. Cases and tolerances follow
tests/TestBandSolvers.cpp:87-176 of the reference (1e-12 relative, identical
pivots and failure indices, the operators' shape n = 200, kd = 14)."""

import numpy as np
import pytest
from scipy.linalg import lapack

from tests import _oracle

TOL = 1e-12


def uniform(count, seed):
    return np.random.default_rng(seed).uniform(-1.0, 1.0, count)


def rel(got, want):
    return np.max(np.abs(got - want)) / np.max(np.abs(want))


def symmetric_band(n, kd, shift, seed):
    ld = kd + 1
    ab = uniform(ld * n, seed)
    for j in range(n):
        ab[j * ld + kd] += shift
        for i in range(j - kd, 0):
            ab[j * ld + kd + i - j] = 0.0
    return ab


def general_band(n, kl, ku, diagonal, seed):
    ld = 2 * kl + ku + 1
    kv = kl + ku
    values = uniform(ld * n, seed)
    ab = np.zeros(ld * n)
    for j in range(n):
        for i in range(max(0, j - ku), min(n - 1, j + kl) + 1):
            at = j * ld + kv + i - j
            ab[at] = values[at] * (diagonal if i == j else 1.0)
    return ab


def lapack_cholesky(ab, n, kd, b, nrhs):
    u, info = lapack.dpbtrf(ab.reshape(n, kd + 1).T.copy(), lower=0)
    assert info == 0
    x, info = lapack.dpbtrs(u, b.reshape(nrhs, n).T.copy(), lower=0)
    assert info == 0
    return u.T.ravel(), x.T.ravel()


def lapack_lu(ab, n, kl, ku, b, nrhs):
    ld = 2 * kl + ku + 1
    lu, piv, info = lapack.dgbtrf(ab.reshape(n, ld).T.copy(), kl, ku)
    assert info == 0
    x, info = lapack.dgbtrs(lu, kl, ku, b.reshape(nrhs, n).T.copy(), piv)
    assert info == 0
    return lu.T.ravel(), piv.astype(np.int32), x.T.ravel()


CHOLESKY_CASES = [(200, 14, 4, 1), (60, 5, 1, 2), (4, 7, 2, 3), (1, 0, 1, 4)]
LU_CASES = [(200, 14, 14, 4, 5), (80, 3, 6, 2, 6), (80, 6, 3, 1, 7), (6, 9, 9, 2, 8)]


@pytest.mark.parametrize("n,kd,nrhs,seed", CHOLESKY_CASES)
def test_oracle_cholesky_matches_lapack(n, kd, nrhs, seed):
    o = _oracle.load()
    ours = symmetric_band(n, kd, 2.0 * kd + 1.0, seed)
    b = uniform(n * nrhs, seed + 1)
    want_u, want_x = lapack_cholesky(ours.copy(), n, kd, b.copy(), nrhs)
    assert o.oracle_band_cholesky_factor(_oracle.ptr(ours), n, kd) == 0
    # entries outside the matrix (i < 0) are not part of U
    mask = np.ones_like(ours, dtype=bool)
    for j in range(n):
        for i in range(j - kd, 0):
            mask[j * (kd + 1) + kd + i - j] = False
    assert rel(ours[mask], want_u[mask]) < TOL
    x = b.copy()
    o.oracle_band_cholesky_solve(_oracle.ptr(ours), n, kd, _oracle.ptr(x), nrhs)
    assert rel(x, want_x) < TOL


@pytest.mark.parametrize("n,kl,ku,nrhs,seed", LU_CASES)
def test_oracle_lu_matches_lapack(n, kl, ku, nrhs, seed):
    o = _oracle.load()
    ours = general_band(n, kl, ku, 0.05, seed)
    b = uniform(n * nrhs, seed + 1)
    want_lu, want_piv, want_x = lapack_lu(ours.copy(), n, kl, ku, b.copy(), nrhs)
    pivots = np.zeros(n, dtype=np.int32)
    assert o.oracle_band_lu_factor(_oracle.ptr(ours), n, kl, ku, _oracle.ptr(pivots)) == 0
    assert np.array_equal(pivots, want_piv)
    if n > 10:
        assert np.any(pivots != np.arange(n))  # the case exercises the pivoting
    assert rel(ours, want_lu) < TOL
    x = b.copy()
    o.oracle_band_lu_solve(_oracle.ptr(ours), n, kl, ku, _oracle.ptr(pivots), _oracle.ptr(x), nrhs)
    assert rel(x, want_x) < TOL


def test_oracle_cholesky_reports_the_indefinite_minor():
    o = _oracle.load()
    n, kd = 40, 4
    ours = symmetric_band(n, kd, 2.0 * kd + 1.0, 9)
    ours[17 * (kd + 1) + kd] = -1.0
    _, info = lapack.dpbtrf(ours.reshape(n, kd + 1).T.copy(), lower=0)
    assert info > 0
    assert o.oracle_band_cholesky_factor(_oracle.ptr(ours), n, kd) == info


def zero_pivot_band():
    n, kl, ku = 30, 3, 3
    ours = general_band(n, kl, ku, 1.0, 10)
    ld = 2 * kl + ku + 1
    zero = 11
    for i in range(zero - ku, zero + kl + 1):
        ours[zero * ld + kl + ku + i - zero] = 0.0
    return ours, n, kl, ku


def test_oracle_lu_reports_the_zero_pivot():
    o = _oracle.load()
    ours, n, kl, ku = zero_pivot_band()
    _, _, info = lapack.dgbtrf(ours.reshape(n, 2 * kl + ku + 1).T.copy(), kl, ku)
    assert info > 0
    pivots = np.zeros(n, dtype=np.int32)
    assert o.oracle_band_lu_factor(_oracle.ptr(ours), n, kl, ku, _oracle.ptr(pivots)) == info


# -- the GPU kernels ----------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("n,kd,nrhs,seed", CHOLESKY_CASES + [(1803, 17, 514, 11), (300, 17, 65, 13)])
def test_gpu_cholesky_matches_oracle_and_lapack(gpu, n, kd, nrhs, seed):
    from sl3dpp_gb300.band import BandCholeskyFactor, BandCholeskySolve

    o = _oracle.load()
    ab = symmetric_band(n, kd, 2.0 * kd + 1.0, seed)
    b = uniform(n * nrhs, seed + 1)
    ref = ab.copy()
    assert o.oracle_band_cholesky_factor(_oracle.ptr(ref), n, kd) == 0
    ours = ab.copy()
    assert BandCholeskyFactor(ours, n, kd) == 0
    assert rel(ours, ref) < TOL
    want = b.copy()
    o.oracle_band_cholesky_solve(_oracle.ptr(ref), n, kd, _oracle.ptr(want), nrhs)
    x = b.copy()
    BandCholeskySolve(ours, n, kd, x, nrhs)
    assert rel(x, want) < TOL
    if n <= 200:
        _, lx = lapack_cholesky(ab.copy(), n, kd, b.copy(), nrhs)
        assert rel(x, lx) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("n,kl,ku,nrhs,seed", LU_CASES + [(1803, 17, 17, 66, 12), (150, 5, 7, 129, 14)])
def test_gpu_lu_matches_oracle_and_lapack(gpu, n, kl, ku, nrhs, seed):
    from sl3dpp_gb300.band import BandLuFactor, BandLuSolve

    o = _oracle.load()
    ab = general_band(n, kl, ku, 0.05, seed)
    b = uniform(n * nrhs, seed + 1)
    ref = ab.copy()
    ref_piv = np.zeros(n, dtype=np.int32)
    assert o.oracle_band_lu_factor(_oracle.ptr(ref), n, kl, ku, _oracle.ptr(ref_piv)) == 0
    ours = ab.copy()
    piv = np.zeros(n, dtype=np.int32)
    assert BandLuFactor(ours, n, kl, ku, piv) == 0
    assert np.array_equal(piv, ref_piv)
    assert rel(ours, ref) < TOL
    want = b.copy()
    o.oracle_band_lu_solve(_oracle.ptr(ref), n, kl, ku, _oracle.ptr(ref_piv), _oracle.ptr(want), nrhs)
    x = b.copy()
    BandLuSolve(ours, n, kl, ku, piv, x, nrhs)
    assert rel(x, want) < TOL


@pytest.mark.gpu
def test_gpu_failure_indices_match(gpu):
    from sl3dpp_gb300.band import BandCholeskyFactor, BandLuFactor

    o = _oracle.load()
    n, kd = 40, 4
    ab = symmetric_band(n, kd, 2.0 * kd + 1.0, 9)
    ab[17 * (kd + 1) + kd] = -1.0
    want = o.oracle_band_cholesky_factor(_oracle.ptr(ab.copy()), n, kd)
    assert want > 0
    assert BandCholeskyFactor(ab.copy(), n, kd) == want
    ours, n, kl, ku = zero_pivot_band()
    pivots = np.zeros(n, dtype=np.int32)
    want = o.oracle_band_lu_factor(_oracle.ptr(ours.copy()), n, kl, ku, _oracle.ptr(pivots))
    assert want > 0
    assert BandLuFactor(ours.copy(), n, kl, ku, np.zeros(n, dtype=np.int32)) == want
