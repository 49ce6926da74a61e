"""One degree's system through the C ABI: DegreeOperator (toroidal=False) or
ToroidalOperator (toroidal=True) of degree l on the unrelaxed material of a
layered earth (include/sl3dpp/DegreeOperator.hpp:94-384): DofCount, Dof,
SurfaceDof, Load, Tide, Apply (host) and Solve (GPU band solves of the
factorised scaled band), UsedCholesky. Vectors are float64 numpy arrays of
DofCount() values; several right-hand sides are columns of (ndof, nrhs)
stored column after column, as the reference passes them."""

from __future__ import annotations

import ctypes

import numpy as np

from ._lib import P_double, check, lib
from .viscoelastic3d import Layer

_SIGNED = False


def _signatures():
    global _SIGNED
    if _SIGNED:
        return
    L, v, i, d = lib(), ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    for name, res, args in (
            ("sl3dgpu_degree_create", i, [ctypes.POINTER(Layer), i, i, i, d, i, ctypes.POINTER(v)]),
            ("sl3dgpu_degree_destroy", None, [v]),
            ("sl3dgpu_degree_dof_count", i, [v]),
            ("sl3dgpu_degree_bandwidth", i, [v]),
            ("sl3dgpu_degree_used_cholesky", i, [v]),
            ("sl3dgpu_degree_dof", i, [v, i, i]),
            ("sl3dgpu_degree_surface_dof", i, [v, i]),
            ("sl3dgpu_degree_load", i, [v, P_double]),
            ("sl3dgpu_degree_tide", i, [v, i, P_double]),
            ("sl3dgpu_degree_apply", i, [v, P_double, i, P_double]),
            ("sl3dgpu_degree_band", i, [v, P_double]),
            ("sl3dgpu_degree_solve", i, [v, P_double, i])):
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    _SIGNED = True


def _p(a: np.ndarray):
    return a.ctypes.data_as(P_double)


class DegreeOperator:
    def __init__(self, layers, ngll: int, l: int, eps: float = 1e-8, toroidal: bool = False):
        _signatures()
        self.l, self.toroidal = l, toroidal
        h = ctypes.c_void_p()
        check(lib().sl3dgpu_degree_create(layers, len(layers), ngll, l, eps, int(toroidal), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        try:
            lib().sl3dgpu_degree_destroy(self._h)
        except Exception:
            pass

    def DofCount(self) -> int:
        return check(lib().sl3dgpu_degree_dof_count(self._h))

    def Bandwidth(self) -> int:
        return check(lib().sl3dgpu_degree_bandwidth(self._h))

    def UsedCholesky(self) -> bool:
        return check(lib().sl3dgpu_degree_used_cholesky(self._h)) == 1

    def Dof(self, node: int, component: int = 0) -> int:
        out = lib().sl3dgpu_degree_dof(self._h, node, component)
        return out if out >= -1 else check(out)

    def SurfaceDof(self, component: int = 0) -> int:
        out = lib().sl3dgpu_degree_surface_dof(self._h, component)
        return out if out >= -1 else check(out)

    def Band(self) -> np.ndarray:
        """The assembled, unscaled upper band as a (ndof, kd + 1) array (LAPACK
        storage, one stored column per row)."""
        out = np.empty((self.DofCount(), self.Bandwidth() + 1))
        check(lib().sl3dgpu_degree_band(self._h, _p(out)))
        return out

    def Load(self) -> np.ndarray:
        out = np.zeros(self.DofCount())
        check(lib().sl3dgpu_degree_load(self._h, _p(out)))
        return out

    def Tide(self, power: int = -1) -> np.ndarray:
        out = np.zeros(self.DofCount())
        check(lib().sl3dgpu_degree_tide(self._h, power, _p(out)))
        return out

    def Apply(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        nrhs = x.size // self.DofCount()
        y = np.zeros_like(x)
        check(lib().sl3dgpu_degree_apply(self._h, _p(x), nrhs, _p(y)))
        return y

    def Solve(self, b: np.ndarray) -> np.ndarray:
        x = np.array(b, dtype=np.float64, copy=True, order="C")
        nrhs = x.size // self.DofCount()
        check(lib().sl3dgpu_degree_solve(self._h, _p(x), nrhs))
        return x
