"""ctypes binding of the sl3dgpu C ABI (include/sl3dgpu.h).

The library is the in-tree libsl3dgpu.so next to this file. It is built by
__graft_entry__.build() or sl3dpp_gb300.build; loading fails loudly when it is
missing -- there is no CPU fallback behind this package.
"""

from __future__ import annotations

import ctypes
import pathlib

_HERE = pathlib.Path(__file__).resolve().parent
LIBRARY_PATH = _HERE / "libsl3dgpu.so"

c_int = ctypes.c_int
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
c_longlong = ctypes.c_longlong
P_double = ctypes.POINTER(ctypes.c_double)
P_int = ctypes.POINTER(ctypes.c_int)

OK = 0
ERR_ARGUMENT = -1
ERR_CUDA = -2
ERR_RUNTIME = -3
ERR_UNCONVERGED = -4
ERR_WAIT = -5


class BandSystem(ctypes.Structure):
    """sl3dgpu_band_system."""

    _fields_ = [
        ("n", c_int),
        ("kl", c_int),
        ("ku", c_int),
        ("nrhs", c_int),
        ("band", c_longlong),
        ("pivots", c_longlong),
        ("rhs", c_longlong),
        ("scale", c_longlong),
        ("pinned0", c_int),
        ("pinned1", c_int),
    ]


class SleBody(ctypes.Structure):
    """sl3dgpu_sle_body: the solver's Love numbers (host arrays) and constants."""
    _fields_ = [("h", P_double), ("k", P_double), ("l", P_double), ("ht", P_double), ("kt", P_double),
                ("lt", P_double), ("g", ctypes.c_double), ("water_density", ctypes.c_double),
                ("radius", ctypes.c_double), ("rotation", ctypes.c_int), ("omega", ctypes.c_double),
                ("polar_moment", ctypes.c_double), ("equatorial_moment", ctypes.c_double),
                ("gravitational_constant", ctypes.c_double), ("hc", ctypes.c_double), ("kc", ctypes.c_double),
                ("m_u", ctypes.c_double), ("m_phi", ctypes.c_double), ("m_c", ctypes.c_double)] + [
                (name, P_double) for name in ("h_u", "k_u", "l_u", "h_phi", "k_phi", "l_phi", "h_v", "k_v", "l_v")]


class SleForcing(ctypes.Structure):
    """sl3dgpu_sle_forcing: GeneralisedForcing's channels (device pointers or null)."""
    _fields_ = [(name, ctypes.c_void_p) for name in
                ("direct_load", "direct_load_outside", "solid_surface_change", "displacement_response",
                 "potential_response", "tangential_response", "toroidal_response", "tide")] + [
                ("inertia_moment_change", ctypes.c_double), ("angular_momentum_change", ctypes.c_double * 3)] + [
                (name, ctypes.c_void_p) for name in ("displacement_load", "potential_load", "tangential_traction")]


class SleState(ctypes.Structure):
    """sl3dgpu_sle_state: GRDSolver::State's fields (device pointers; the land mask may be null)."""
    _fields_ = [(name, ctypes.c_void_p) for name in ("ice_thickness", "sea_level", "ocean_function",
                                                     "forced_land")]


class SleNonlinearForcing(ctypes.Structure):
    """sl3dgpu_sle_nonlinear_forcing: NonlinearForcing's channels (device pointers or null)."""
    _fields_ = [(name, ctypes.c_void_p) for name in
                ("ice_thickness_change", "direct_load", "direct_load_outside", "solid_surface_change",
                 "dynamic_sea_level_change", "displacement_response", "potential_response", "tangential_response",
                 "toroidal_response", "tide")] + [
                ("inertia_moment_change", ctypes.c_double), ("hold_land", ctypes.c_int),
                ("forced_land", ctypes.c_void_p)]


class SleResult(ctypes.Structure):
    """sl3dgpu_sle_result: GRDSolver::Response's scalars."""
    _fields_ = [("uniform_shift", ctypes.c_double), ("error", ctypes.c_double), ("iterations", ctypes.c_int),
                ("converged", ctypes.c_int), ("angular_velocity", ctypes.c_double * 3)]


class Sl3dgpuError(RuntimeError):
    """A failed sl3dgpu call (the reference's std::runtime_error and friends)."""

    def __init__(self, status: int, text: str):
        super().__init__(f"sl3dgpu status {status}: {text}")
        self.status = status


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIBRARY_PATH.exists():
        raise ImportError(
            f"{LIBRARY_PATH} is missing: build it with __graft_entry__.build() "
            "(the CUDA path is the only path; nothing falls back to the CPU)")
    L = ctypes.CDLL(str(LIBRARY_PATH))
    sig = {
        "sl3dgpu_last_error": (ctypes.c_char_p, []),
        "sl3dgpu_version": (ctypes.c_char_p, []),
        "sl3dgpu_band_cholesky_factor": (c_int, [P_double, c_int, c_int]),
        "sl3dgpu_band_cholesky_solve": (c_int, [P_double, c_int, c_int, P_double, c_int]),
        "sl3dgpu_band_lu_factor": (c_int, [P_double, c_int, c_int, c_int, P_int]),
        "sl3dgpu_band_lu_solve": (c_int, [P_double, c_int, c_int, c_int, P_int, P_double, c_int]),
        "sl3dgpu_band_factor_batch": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                                              c_int, c_void_p]),
        "sl3dgpu_band_work_items": (c_int, [c_void_p, c_int, c_void_p, c_int]),
        "sl3dgpu_band_solve_batch": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p,
                                             c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
        "sl3dgpu_band_solve_batch_f32": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p,
                                                 c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
        "sl3dgpu_grid_create": (c_int, [c_int, c_int, c_double, ctypes.POINTER(c_void_p)]),
        "sl3dgpu_grid_destroy": (None, [c_void_p]),
        "sl3dgpu_grid_shape": (c_int, [c_void_p, P_int, P_int]),
        "sl3dgpu_grid_lmax": (c_int, [c_void_p]),
        "sl3dgpu_sle_solve": (c_int, [c_void_p, ctypes.POINTER(SleBody), c_void_p, ctypes.POINTER(SleForcing),
                                      c_double, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      ctypes.POINTER(SleResult), c_void_p]),
        "sl3dgpu_sle_solve_nonlinear": (c_int, [c_void_p, ctypes.POINTER(SleBody), c_double,
                                                ctypes.POINTER(SleState), ctypes.POINTER(SleNonlinearForcing),
                                                c_double, c_int] + [c_void_p] * 8 + [ctypes.POINTER(SleResult),
                                                                                      c_void_p]),
        "sl3dgpu_sle_flotation": (c_int, [ctypes.c_longlong, c_double, c_double, c_void_p, c_void_p, c_void_p,
                                          c_void_p, c_void_p]),
        "sl3dgpu_grid_set_fp64_emulation": (c_int, [c_void_p, c_int]),
        "sl3dgpu_grid_colatitudes": (c_int, [c_void_p, P_double, P_double]),
        "sl3dgpu_synthesise_spin_batch": (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p]),
        "sl3dgpu_legendre_device": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_int, c_void_p,
                                            c_void_p]),
        "sl3dgpu_expand_spin_batch": (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p]),
        "sl3dgpu_synthesise_batch": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
        "sl3dgpu_expand_batch": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
        "sl3dgpu_launch_count": (ctypes.c_longlong, []),
        "sl3dgpu_profile_enable": (c_int, [c_int]),
        "sl3dgpu_profile_reset": (c_int, []),
        "sl3dgpu_profile_read": (c_int, [c_int, P_double, ctypes.POINTER(ctypes.c_longlong), P_double, P_double]),
        "sl3dgpu_fp64_fma_peak": (c_int, [P_double]),
        "sl3dgpu_fp32_fma_peak": (c_int, [P_double]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def exported_symbols() -> list[str]:
    """Every function include/sl3dgpu.h declares (parsed from the header)."""
    import re

    header = (_HERE.parent / "include" / "sl3dgpu.h").read_text()
    return sorted(set(re.findall(r"\b(sl3dgpu_[a-z0-9_]+)\s*\(", header)))


def check(status: int) -> int:
    """Raise on a negative status; return non-negative ones (LAPACK info)."""
    if status < 0:
        text = lib().sl3dgpu_last_error().decode(errors="replace")
        raise Sl3dgpuError(status, text)
    return status
