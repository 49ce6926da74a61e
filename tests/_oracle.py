"""ctypes access to the oracle (oracle/_build/liboracle.so), the CPU FP64
restatement the tests check the GPU path against. Test infrastructure."""

from __future__ import annotations

import ctypes
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent.parent
P_double = ctypes.POINTER(ctypes.c_double)
P_int = ctypes.POINTER(ctypes.c_int)

_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    sys.path.insert(0, str(ROOT))
    from oracle import build as oracle_build

    path = oracle_build.build()
    L = ctypes.CDLL(str(path))
    i, d, v = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    sig = {
        "oracle_band_cholesky_factor": (i, [P_double, i, i]),
        "oracle_band_cholesky_solve": (None, [P_double, i, i, P_double, i]),
        "oracle_band_lu_factor": (i, [P_double, i, i, i, P_int]),
        "oracle_band_lu_solve": (None, [P_double, i, i, i, P_int, P_double, i]),
        "oracle_gauss_legendre": (None, [i, P_double, P_double]),
        "oracle_wigner_column": (None, [i, i, i, i, P_double, P_double]),
        "oracle_synthesise_spin": (None, [i, i, i, i, P_double, P_double, P_double]),
        "oracle_expand_spin": (None, [i, i, i, i, P_double, P_double, P_double, P_double]),
        "oracle_synthesise_real": (None, [i, i, i, P_double, P_double, P_double]),
        "oracle_expand_real": (None, [i, i, i, P_double, P_double, P_double, P_double]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def ptr(a: np.ndarray):
    if a.dtype == np.int32:
        return a.ctypes.data_as(P_int)
    return a.ctypes.data_as(P_double)


# -- convenience wrappers ---------------------------------------------------------

def gauss_legendre(n: int):
    x = np.empty(n)
    w = np.empty(n)
    load().oracle_gauss_legendre(n, ptr(x), ptr(w))
    return x, w


def fft_friendly(n: int) -> int:
    m = max(n, 1)
    while True:
        r = m
        for p in (2, 3, 5):
            while r % p == 0:
                r //= p
        if r == 1:
            return m
        m += 1


def grid_shape(lmax: int, oversampling: float = 1.0):
    band = int(np.ceil(oversampling * lmax - 1e-12))
    return band + 1, fft_friendly(2 * band + 1)


def grid(lmax: int, oversampling: float = 1.0):
    nt, nph = grid_shape(lmax, oversampling)
    x, w = gauss_legendre(nt)
    return np.arccos(x), w, nph


def wigner_column(lmax: int, N: int, m: int, theta: np.ndarray) -> np.ndarray:
    l0 = max(abs(m), abs(N))
    out = np.zeros((lmax - l0 + 1, theta.size))
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    load().oracle_wigner_column(lmax, N, m, theta.size, ptr(theta), ptr(out))
    return out


def synthesise_spin(lmax, N, theta, nphi, coeffs):
    coeffs = np.ascontiguousarray(coeffs, dtype=np.complex128)
    field = np.zeros(theta.size * nphi, dtype=np.complex128)
    load().oracle_synthesise_spin(lmax, N, theta.size, nphi, ptr(theta), coeffs.ctypes.data_as(P_double),
                                  field.ctypes.data_as(P_double))
    return field


def expand_spin(lmax, N, theta, weights, nphi, field):
    field = np.ascontiguousarray(field, dtype=np.complex128)
    coeffs = np.zeros((lmax + 1) ** 2 - N * N, dtype=np.complex128)
    load().oracle_expand_spin(lmax, N, theta.size, nphi, ptr(theta), ptr(weights),
                              field.ctypes.data_as(P_double), coeffs.ctypes.data_as(P_double))
    return coeffs


def synthesise_real(lmax, theta, nphi, coeffs):
    coeffs = np.ascontiguousarray(coeffs, dtype=np.complex128)
    field = np.zeros(theta.size * nphi)
    load().oracle_synthesise_real(lmax, theta.size, nphi, ptr(theta), coeffs.ctypes.data_as(P_double), ptr(field))
    return field


def expand_real(lmax, theta, weights, nphi, field):
    field = np.ascontiguousarray(field, dtype=np.float64)
    coeffs = np.zeros((lmax + 1) * (lmax + 2) // 2, dtype=np.complex128)
    load().oracle_expand_real(lmax, theta.size, nphi, ptr(theta), ptr(weights), ptr(field),
                              coeffs.ctypes.data_as(P_double))
    return coeffs
