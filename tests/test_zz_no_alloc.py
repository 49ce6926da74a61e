"""The banded Cholesky solve that allocates no device memory, for callers
that cannot call cudaMalloc (their device memory belongs to another
allocator or a fixed arena, or a driver allocation is not acceptable on their
loop). It must give the allocating entry point's solution, call after call,
on buffers the caller owns, and refuse sizes beyond its static scratch."""

import ctypes

import numpy as np
import pytest

from tests.test_band import rel, symmetric_band, uniform

TOL = 1e-12


def _entry():
    from sl3dpp_gb300 import _lib

    fn = _lib.lib().sl3dgpu_band_cholesky_solve_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    return fn


def dense_upper(ab, n, kd):
    """The symmetric matrix whose upper band LAPACK stores in ab."""
    a = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - kd), j + 1):
            a[i, j] = a[j, i] = ab[j * (kd + 1) + kd + i - j]
    return a


@pytest.mark.gpu
def test_no_alloc_solve_matches_the_allocating_solve(gpu):
    import torch

    from sl3dpp_gb300 import _lib
    from sl3dpp_gb300.band import BandCholeskyFactor, BandCholeskySolve

    solve = _entry()
    n, kd = 1803, 17  # the largest degree system's shape at lmax 256
    ab = symmetric_band(n, kd, 2.0 * kd + 1.0, 21)
    dense = dense_upper(ab, n, kd)
    assert BandCholeskyFactor(ab, n, kd) == 0
    d_ab = torch.tensor(ab, device=gpu)
    stream = torch.cuda.current_stream().cuda_stream
    for nrhs, seed in [(66, 5), (130, 6)]:  # two calls in a row, different shapes
        b = uniform(n * nrhs, seed)
        want = b.copy()
        BandCholeskySolve(ab, n, kd, want, nrhs)  # the existing, allocating entry point
        d_b = torch.tensor(b, device=gpu)
        assert solve(d_ab.data_ptr(), n, kd, d_b.data_ptr(), nrhs, stream) == _lib.OK
        torch.cuda.synchronize()
        got = d_b.cpu().numpy()
        assert rel(got, want) < TOL
        # and against a dense solve of the same system (numpy's LAPACK), so
        # that the entry point's own packing is checked by other arithmetic
        exact = np.linalg.solve(dense, b.reshape(nrhs, n).T).T.reshape(-1)
        assert rel(got, exact) < 1e-11


@pytest.mark.gpu
def test_no_alloc_solve_single_column_small_system(gpu):
    """One right-hand side (not a multiple of the 64-column work item) on a
    small system, against a dense solve."""
    import torch

    from sl3dpp_gb300 import _lib
    from sl3dpp_gb300.band import BandCholeskyFactor

    solve = _entry()
    stream = torch.cuda.current_stream().cuda_stream
    for n, kd, nrhs, seed in [(40, 5, 1, 31), (97, 14, 3, 32)]:
        ab = symmetric_band(n, kd, 2.0 * kd + 1.0, seed)
        dense = dense_upper(ab, n, kd)
        assert BandCholeskyFactor(ab, n, kd) == 0
        b = uniform(n * nrhs, seed + 100)
        d_ab = torch.tensor(ab, device=gpu)
        d_b = torch.tensor(b, device=gpu)
        assert solve(d_ab.data_ptr(), n, kd, d_b.data_ptr(), nrhs, stream) == _lib.OK
        torch.cuda.synchronize()
        exact = np.linalg.solve(dense, b.reshape(nrhs, n).T).T.reshape(-1)
        assert rel(d_b.cpu().numpy(), exact) < 1e-12


@pytest.mark.gpu
def test_no_alloc_solve_refuses_sizes_beyond_its_scratch(gpu):
    import torch

    from sl3dpp_gb300 import _lib

    solve = _entry()
    n, kd, nrhs = 1803, 17, 400  # 721200 values > 2^19
    d_ab = torch.zeros((kd + 1) * n, dtype=torch.float64, device=gpu)
    d_b = torch.zeros(n * nrhs, dtype=torch.float64, device=gpu)
    st = solve(d_ab.data_ptr(), n, kd, d_b.data_ptr(), nrhs, torch.cuda.current_stream().cuda_stream)
    assert st == _lib.ERR_ARGUMENT
    assert b"static scratch" in _lib.lib().sl3dgpu_last_error()
