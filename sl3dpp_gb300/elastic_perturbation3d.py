"""ElasticPerturbation3D on the GPU (include/sl3dpp/ElasticPerturbation3D.hpp:
77-225): the static gravitating elastic problem under lateral perturbations of
the shear and bulk moduli, through the sl3dgpu C ABI.

The names follow the reference class: SolveLoad (the reference response),
Respond (the first-order, Born response of the held solution), SolveLateral
(the full solve by preconditioned conjugate gradients), Surface."""

from __future__ import annotations

import ctypes
from ctypes import c_void_p

import numpy as np

from ._lib import P_double, P_int, check, lib
from .viscoelastic3d import COMPONENTS, Layer, StepInfo, _signatures as _v3d_signatures


class EpOptions(ctypes.Structure):
    """sl3dgpu_ep3d_options (ElasticPerturbation3D::Options)."""

    _fields_ = [("lmax", ctypes.c_int), ("ngll", ctypes.c_int), ("eps", ctypes.c_double),
                ("oversampling", ctypes.c_double)]


_SIGNED = False


def _signatures():
    global _SIGNED
    if _SIGNED:
        return
    _v3d_signatures()
    v, i, d = c_void_p, ctypes.c_int, ctypes.c_double
    sig = {
        "sl3dgpu_ep3d_create": (i, [ctypes.POINTER(Layer), i, ctypes.POINTER(EpOptions), ctypes.POINTER(v)]),
        "sl3dgpu_ep3d_destroy": (None, [v]),
        "sl3dgpu_ep3d_shape": (i, [v, P_int, P_int, P_int]),
        "sl3dgpu_ep3d_nodes": (i, [v, P_double, P_int]),
        "sl3dgpu_ep3d_colatitudes": (i, [v, P_double, P_double]),
        "sl3dgpu_ep3d_scales": (i, [v, P_double, P_double, P_double]),
        "sl3dgpu_ep3d_set_moduli": (i, [v, v, v, i]),
        "sl3dgpu_ep3d_solve_load": (i, [v, v]),
        "sl3dgpu_ep3d_respond": (i, [v]),
        "sl3dgpu_ep3d_solve_lateral": (i, [v, v, d, i, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_ep3d_surface": (i, [v, i, v]),
        "sl3dgpu_ep3d_residual_history": (i, [v, P_double, i]),
        "sl3dgpu_ep3d_layout": (i, [v, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
        "sl3dgpu_ep3d_force": (i, [v, v, v]),
        "sl3dgpu_ep3d_apply": (i, [v, v, v]),
        "sl3dgpu_ep3d_load_forces": (i, [v, v, v]),
        "sl3dgpu_ep3d_solution": (i, [v, v]),
    }
    L = lib()
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _SIGNED = True


class ElasticPerturbation3D:
    """The static problem on the GPU; moduli directions over the coupling's
    grid values (node-major, colatitude, longitude) in the model's modulus
    unit (`modulus_scale` Pa)."""

    def __init__(self, layers, lmax: int, ngll: int = 5, eps: float = 1e-8, oversampling: float = 1.5):
        _signatures()
        h = c_void_p()
        check(lib().sl3dgpu_ep3d_create(layers, len(layers), ctypes.byref(EpOptions(lmax, ngll, eps, oversampling)),
                                        ctypes.byref(h)))
        self._h = h
        self.lmax = lmax
        P, nt, nph = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().sl3dgpu_ep3d_shape(h, ctypes.byref(P), ctypes.byref(nt), ctypes.byref(nph)))
        self.node_count, self.ntheta, self.nphi = P.value, nt.value, nph.value
        self.radius = np.empty(self.node_count)
        self.element = np.empty(self.node_count, dtype=np.int32)
        check(lib().sl3dgpu_ep3d_nodes(h, self.radius.ctypes.data_as(P_double), self.element.ctypes.data_as(P_int)))
        self.theta = np.empty(self.ntheta)
        self.weights = np.empty(self.ntheta)
        check(lib().sl3dgpu_ep3d_colatitudes(h, self.theta.ctypes.data_as(P_double),
                                             self.weights.ctypes.data_as(P_double)))
        length, modulus, sigma = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib().sl3dgpu_ep3d_scales(h, ctypes.byref(length), ctypes.byref(modulus), ctypes.byref(sigma)))
        self.length_scale, self.modulus_scale, self.surface_density_scale = length.value, modulus.value, sigma.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().sl3dgpu_ep3d_destroy(h)
            self._h = None

    @property
    def values(self) -> int:
        return self.node_count * self.ntheta * self.nphi

    def set_moduli(self, d_mu=None, d_kappa=None) -> None:
        """The directions (numpy arrays, or torch CUDA tensors), None for none."""
        on_device = 0
        ptrs = []
        self._keep = []
        for a in (d_mu, d_kappa):
            if a is None:
                ptrs.append(None)
                continue
            if hasattr(a, "data_ptr"):
                if a.numel() != self.values:
                    raise ValueError("a moduli direction lives on the grid values")
                on_device = 1
                ptrs.append(a.data_ptr())
            else:
                arr = np.ascontiguousarray(a, dtype=np.float64)
                if arr.size != self.values:
                    raise ValueError("a moduli direction lives on the grid values")
                self._keep.append(arr)
                ptrs.append(arr.ctypes.data)
        check(lib().sl3dgpu_ep3d_set_moduli(self._h, ptrs[0], ptrs[1], on_device))

    def _load(self, load):
        load = np.ascontiguousarray(load, dtype=np.complex128)
        if load.size != (self.lmax + 1) * (self.lmax + 2) // 2:
            raise ValueError("a load lives on the lmax grid (l(l+1)/2 + m)")
        return load

    def SolveLoad(self, load) -> None:
        load = self._load(load)
        check(lib().sl3dgpu_ep3d_solve_load(self._h, load.ctypes.data))

    def Respond(self) -> None:
        check(lib().sl3dgpu_ep3d_respond(self._h))

    def SolveLateral(self, load, rtol: float = 1e-10, max_iterations: int = 200) -> StepInfo:
        load = self._load(load)
        info = StepInfo()
        check(lib().sl3dgpu_ep3d_solve_lateral(self._h, load.ctypes.data, rtol, max_iterations, ctypes.byref(info)))
        return info

    def Surface(self, component="U") -> np.ndarray:
        code = COMPONENTS[component] if isinstance(component, str) else int(component)
        out = np.zeros((self.lmax + 1) * (self.lmax + 2) // 2, dtype=np.complex128)
        check(lib().sl3dgpu_ep3d_surface(self._h, code, out.ctypes.data))
        return out

    # -- Force / Apply / LoadForces on device solutions (CUDA complex128
    # tensors in the spheroidal-then-toroidal layout)

    def _solutions(self):
        import torch

        s, tor = ctypes.c_longlong(), ctypes.c_longlong()
        check(lib().sl3dgpu_ep3d_layout(self._h, ctypes.byref(s), ctypes.byref(tor)))
        return torch.zeros(s.value + max(tor.value, 1), dtype=torch.complex128, device="cuda")

    def Solution(self):
        """The held solution (SolveLoad's, Respond's or SolveLateral's)."""
        out = self._solutions()
        check(lib().sl3dgpu_ep3d_solution(self._h, out.data_ptr()))
        return out

    def Force(self, x):
        """ElasticPerturbation3D::Force: (dK) x under the set directions."""
        out = self._solutions()
        check(lib().sl3dgpu_ep3d_force(self._h, x.data_ptr(), out.data_ptr()))
        return out

    def Apply(self, x):
        """ElasticPerturbation3D::Apply: (K_ref + dK) x."""
        out = self._solutions()
        check(lib().sl3dgpu_ep3d_apply(self._h, x.data_ptr(), out.data_ptr()))
        return out

    def LoadForces(self, load):
        out = self._solutions()
        load = self._load(load)
        check(lib().sl3dgpu_ep3d_load_forces(self._h, load.ctypes.data, out.data_ptr()))
        return out

    def residual_history(self) -> np.ndarray:
        n = lib().sl3dgpu_ep3d_residual_history(self._h, None, 0)
        out = np.zeros(max(n, 0))
        if n > 0:
            lib().sl3dgpu_ep3d_residual_history(self._h, out.ctypes.data_as(P_double), n)
        return out
