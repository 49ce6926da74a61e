"""The surface grid and its spin-weighted transforms, on the GPU.

Mirrors include/sl3dpp/SurfaceGrid.hpp:58-287: a Gauss-Legendre grid for
degrees to lmax and spins to nmax, oversampled for pointwise products, with
the batched synthesis and analysis of spin-N complex fields and real spin-0
fields in the reference's coefficient layouts. Fields and coefficients are
torch CUDA tensors (device memory only: torch is the allocator here).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import P_double, P_int, c_void_p, check, lib


def _ptr(t: torch.Tensor) -> int:
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return t.data_ptr()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


class SurfaceGrid:
    """A device grid handle (SurfaceGrid's shared Wigner table, on the GPU)."""

    def __init__(self, lmax: int, nmax: int = 0, oversampling: float = 1.0, fp64_emulation: bool = False):
        """fp64_emulation: the Legendre contractions emulated on the tensor
        cores (BF16 slices, exact products, FP64 joins) rather than run on the
        FP64 units."""
        handle = c_void_p()
        check(lib().sl3dgpu_grid_create(lmax, nmax, float(oversampling), ctypes.byref(handle)))
        self._handle = handle
        if fp64_emulation:
            check(lib().sl3dgpu_grid_set_fp64_emulation(handle, 1))
        self.lmax = lmax
        self.nmax = nmax
        nt, nph = ctypes.c_int(), ctypes.c_int()
        check(lib().sl3dgpu_grid_shape(handle, ctypes.byref(nt), ctypes.byref(nph)))
        self.ntheta, self.nphi = nt.value, nph.value
        theta = np.empty(self.ntheta)
        weights = np.empty(self.ntheta)
        check(lib().sl3dgpu_grid_colatitudes(handle, theta.ctypes.data_as(P_double),
                                             weights.ctypes.data_as(P_double)))
        self.theta, self.weights = theta, weights
        self.phi = 2.0 * np.pi * np.arange(self.nphi) / self.nphi

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle is not None and handle.value:
            lib().sl3dgpu_grid_destroy(handle)
            self._handle = None

    # sizes, as SurfaceGrid's
    def FieldSize(self) -> int:
        return self.ntheta * self.nphi

    def CoefficientSize(self) -> int:
        return (self.lmax + 1) * (self.lmax + 2) // 2

    def SpinCoefficientSize(self, N: int) -> int:
        return (self.lmax + 1) ** 2 - N * N

    @staticmethod
    def Index(l: int, m: int) -> int:
        return l * (l + 1) // 2 + m

    @staticmethod
    def SpinIndex(N: int, l: int, m: int) -> int:
        return l * l - N * N + (m + l)

    # batched transforms: complex128 / float64 CUDA tensors
    def SynthesiseSpinBatch(self, N: int, coefficients: torch.Tensor, count: int) -> torch.Tensor:
        assert coefficients.dtype == torch.complex128 and coefficients.numel() == count * self.SpinCoefficientSize(N)
        out = torch.empty(count * self.FieldSize(), dtype=torch.complex128, device=coefficients.device)
        check(lib().sl3dgpu_synthesise_spin_batch(self._handle, N, _ptr(coefficients), count, _ptr(out), _stream()))
        return out

    def ExpandSpinBatch(self, N: int, fields: torch.Tensor, count: int) -> torch.Tensor:
        assert fields.dtype == torch.complex128 and fields.numel() == count * self.FieldSize()
        out = torch.empty(count * self.SpinCoefficientSize(N), dtype=torch.complex128, device=fields.device)
        check(lib().sl3dgpu_expand_spin_batch(self._handle, N, _ptr(fields), count, _ptr(out), _stream()))
        return out

    def SynthesiseBatch(self, coefficients: torch.Tensor, count: int) -> torch.Tensor:
        assert coefficients.dtype == torch.complex128 and coefficients.numel() == count * self.CoefficientSize()
        out = torch.empty(count * self.FieldSize(), dtype=torch.float64, device=coefficients.device)
        check(lib().sl3dgpu_synthesise_batch(self._handle, _ptr(coefficients), count, _ptr(out), _stream()))
        return out

    def ExpandBatch(self, fields: torch.Tensor, count: int) -> torch.Tensor:
        assert fields.dtype == torch.float64 and fields.numel() == count * self.FieldSize()
        out = torch.empty(count * self.CoefficientSize(), dtype=torch.complex128, device=fields.device)
        check(lib().sl3dgpu_expand_batch(self._handle, _ptr(fields), count, _ptr(out), _stream()))
        return out
