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


@pytest.mark.gpu
@pytest.mark.parametrize("scaled", [False, True])
def test_gpu_fp32_row_windows_complete_to_the_every_row_solve(gpu, scaled):
    """The FP32 solves of the mixed form's correction passes, whose forces
    reach a band of rows: right-hand sides zero outside rows [lo, hi] solved
    over rows lo..n-1 (mode 1) and then below lo (mode 2) give the every-row
    FP32 solve (mode 0) -- the rows from lo up identically (the skipped
    products are exact zeros), the rows below within FP32 rounding (the
    completion restarts from the stored, scaled solution) -- and that solve
    agrees with the FP64 oracle to FP32 accuracy. Windows cover an empty
    range, the first row, an interior band and the last rows."""
    import torch

    from sl3dpp_gb300 import _lib
    from sl3dpp_gb300.band import BandCholeskyFactor

    o = _oracle.load()
    shapes = [(1803, 17, 130, (1210, 1400)), (481, 5, 64, (0, 30)), (300, 14, 66, (100, 90)),
              (200, 4, 7, (150, 199)), (97, 17, 514, (40, 60))]
    systems, bands, rhs64, scales, windows = [], [], [], [], []
    band_off = rhs_off = scale_off = 0
    for k, (n, kd, nrhs, (lo, hi)) in enumerate(shapes):
        ab = symmetric_band(n, kd, 2.0 * kd + 1.0, 40 + k)
        assert BandCholeskyFactor(ab, n, kd) == 0
        b = uniform(n * nrhs, 50 + k).reshape(n, nrhs)
        b[:lo] = 0.0
        b[hi + 1:] = 0.0
        s = _lib.BandSystem(n=n, kl=kd, ku=kd, nrhs=nrhs, band=band_off, pivots=0, rhs=rhs_off,
                            scale=scale_off if scaled else -1, pinned0=-1, pinned1=-1)
        systems.append(s)
        bands.append(ab)
        rhs64.append(b)
        scales.append(np.random.default_rng(60 + k).uniform(0.5, 2.0, n))
        windows.append((lo if lo <= hi else n, hi))
        band_off += ab.size
        rhs_off += b.size
        scale_off += n
    host = (_lib.BandSystem * len(systems))(*systems)
    count = _lib.lib().sl3dgpu_band_work_items(host, len(systems), None, 0)
    items = np.zeros(2 * count, dtype=np.int32)
    assert _lib.lib().sl3dgpu_band_work_items(host, len(systems), items.ctypes.data, count) == count
    dev = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=gpu)
    d_sys = torch.tensor(np.frombuffer(bytes(host), dtype=np.uint8), device=gpu)
    d_items = dev(items, torch.int32)
    d_bands = dev(np.concatenate(bands), torch.float32)
    d_scales = dev(np.concatenate(scales), torch.float32)
    d_windows = dev(np.array(windows, dtype=np.int32).ravel(), torch.int32)
    b0 = np.concatenate([b.ravel() for b in rhs64]).astype(np.float32)
    stream = torch.cuda.current_stream().cuda_stream
    solve = _lib.lib().sl3dgpu_band_solve_batch_f32

    def run(modes):
        x = dev(b0, torch.float32)
        for mode in modes:
            st = solve(d_sys.data_ptr(), host, len(systems), d_items.data_ptr(), count, d_bands.data_ptr(),
                       x.data_ptr(), d_scales.data_ptr(), d_windows.data_ptr() if mode else None, mode, stream)
            assert st == _lib.OK
        torch.cuda.synchronize()
        return x.cpu().numpy()

    full = run([0])
    windowed = run([1, 2])
    partial = run([1])
    at = 0
    for k, (n, kd, nrhs, _) in enumerate(shapes):
        lo = windows[k][0]
        f = full[at:at + n * nrhs].reshape(n, nrhs)
        w = windowed[at:at + n * nrhs].reshape(n, nrhs)
        p = partial[at:at + n * nrhs].reshape(n, nrhs)
        assert np.array_equal(p[lo:], f[lo:]), k
        assert np.array_equal(w[lo:], f[lo:]), k
        if scaled and np.any(f):
            assert rel(w, f) < 1e-5, k
        else:
            assert np.array_equal(w, f), k
        # the FP32 solve against the FP64 oracle (scaling: D^-1 A^-1 D^-1 b as
        # the scaled systems solve, x = D (U^T U)^-1 D b)
        d = scales[k] if scaled else np.ones(n)
        want = (rhs64[k] * d[:, None]).T.copy().ravel()
        o.oracle_band_cholesky_solve(_oracle.ptr(bands[k]), n, kd, _oracle.ptr(want), nrhs)
        want = want.reshape(nrhs, n).T * d[:, None]
        if np.any(want):
            assert rel(f.astype(np.float64), want) < 1e-4, k
        else:
            assert not np.any(f), k
        at += n * nrhs
