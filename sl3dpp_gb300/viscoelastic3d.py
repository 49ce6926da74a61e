"""The 3D quasi-static step on the GPU, mirroring Viscoelastic3D.

Mirrors include/sl3dpp/Viscoelastic3D.hpp:79-837 for the fixed-point step
(Picard, then Anderson when a pass contracts too slowly): construction over a
layered Earth with the log-viscosity perturbation delta sampled on every
memory node's grid, ZeroState, Step (ExponentialTrapezoid, BackwardEuler or
Sdirk2) under a surface-load channel, Surface. All compute runs in
libsl3dgpu.so (the C ABI of include/sl3dgpu.h); this class holds the handles.
"""

from __future__ import annotations

import ctypes

import numpy as np

from ._lib import P_double, P_int, c_void_p, check, lib

SCHEMES = {"exponential_trapezoid": 0, "backward_euler": 1, "sdirk2": 2}
COMPONENTS = {"U": 0, "V": 1, "phi": 2, "W": 3}


class Layer(ctypes.Structure):
    """sl3dgpu_layer."""

    _fields_ = [("r0", ctypes.c_double), ("r1", ctypes.c_double), ("fluid", ctypes.c_int),
                ("elements", ctypes.c_int), ("rho0", ctypes.c_double), ("rho1", ctypes.c_double),
                ("kappa0", ctypes.c_double), ("kappa1", ctypes.c_double), ("mu0", ctypes.c_double),
                ("mu1", ctypes.c_double), ("viscosity", ctypes.c_double),
                ("kelvin_fraction", ctypes.c_double), ("kelvin_viscosity", ctypes.c_double)]


class Options(ctypes.Structure):
    """sl3dgpu_v3d_options (Viscoelastic3D::Options)."""

    _fields_ = [("lmax", ctypes.c_int), ("ngll", ctypes.c_int), ("eps", ctypes.c_double),
                ("oversampling", ctypes.c_double), ("max_iterations", ctypes.c_int),
                ("rtol", ctypes.c_double), ("damping", ctypes.c_double), ("anderson_memory", ctypes.c_int),
                ("anderson_rate", ctypes.c_double), ("precision", ctypes.c_int),
                ("correction_rtol", ctypes.c_double), ("solver", ctypes.c_int),
                ("solve_rtol", ctypes.c_double), ("solve_max_iterations", ctypes.c_int),
                ("warm_start", ctypes.c_int),
                ("fp64_emulation", ctypes.c_int), ("correction_memory", ctypes.c_int)]

    @classmethod
    def defaults(cls, lmax: int, ngll: int = 5, **kw) -> "Options":
        o = cls(lmax=lmax, ngll=ngll, eps=1e-8, oversampling=1.5, max_iterations=40, rtol=1e-11,
                damping=1.0, anderson_memory=5, anderson_rate=0.5, precision=0, correction_rtol=1e-5,
                solver=0, solve_rtol=1e-11, solve_max_iterations=200, warm_start=0,
                fp64_emulation=0, correction_memory=0)
        for k, v in kw.items():
            setattr(o, k, v)
        return o


class OceanOptions(ctypes.Structure):
    """sl3dgpu_v3d_ocean: the ocean of the coupled step (SI), SeaLevelParameters'
    defaults (include/sl3dpp/SeaLevel.hpp:54-68) for the body's constants."""

    _fields_ = [("ocean_function", c_void_p), ("rotation", ctypes.c_int), ("water_density", ctypes.c_double),
                ("rotation_frequency", ctypes.c_double), ("polar_moment", ctypes.c_double),
                ("equatorial_moment", ctypes.c_double), ("rtol", ctypes.c_double),
                ("max_iterations", ctypes.c_int), ("anderson_memory", ctypes.c_int),
                ("migrating", ctypes.c_int), ("ice_density", ctypes.c_double), ("ice_thickness", c_void_p),
                ("sea_level", c_void_p), ("forced_land", c_void_p), ("max_nonlinear_iterations", ctypes.c_int)]


class SleResult(ctypes.Structure):
    """sl3dgpu_sle_result."""

    _fields_ = [("uniform_shift", ctypes.c_double), ("error", ctypes.c_double), ("iterations", ctypes.c_int),
                ("converged", ctypes.c_int), ("angular_velocity", ctypes.c_double * 3)]


class StepInfo(ctypes.Structure):
    """sl3dgpu_step_info (Viscoelastic3D::StepInfo)."""

    _fields_ = [("iterations", ctypes.c_int), ("residual", ctypes.c_double), ("converged", ctypes.c_int),
                ("mixed_passes", ctypes.c_int), ("correction_passes", ctypes.c_int),
                ("solve_iterations", ctypes.c_int)]


_SIGNED = False


def _signatures():
    global _SIGNED
    if _SIGNED:
        return
    L = lib()
    v, i, d = c_void_p, ctypes.c_int, ctypes.c_double
    sig = {
        "sl3dgpu_standard_earth": (i, [i, d, d, ctypes.POINTER(Layer)]),
        "sl3dgpu_v3d_create": (i, [ctypes.POINTER(Layer), i, ctypes.POINTER(Options), ctypes.POINTER(v)]),
        "sl3dgpu_v3d_destroy": (None, [v]),
        "sl3dgpu_v3d_shape": (i, [v, P_int, P_int, P_int]),
        "sl3dgpu_v3d_nodes": (i, [v, P_double, P_int]),
        "sl3dgpu_v3d_colatitudes": (i, [v, P_double, P_double]),
        "sl3dgpu_v3d_scales": (i, [v, P_double, P_double, P_double]),
        "sl3dgpu_v3d_set_delta": (i, [v, v, i]),
        "sl3dgpu_v3d_zero_state": (i, [v, ctypes.POINTER(v)]),
        "sl3dgpu_v3d_free_state": (None, [v]),
        "sl3dgpu_v3d_step": (i, [v, v, d, i, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_surface": (i, [v, i, v]),
        "sl3dgpu_v3d_inertia_moment": (i, [v, P_double]),
        "sl3dgpu_v3d_state_strain": (i, [v, v, v]),
        "sl3dgpu_v3d_residual_history": (i, [v, P_double, i]),
        "sl3dgpu_v3d_correction_history": (i, [v, P_double, i]),
        "sl3dgpu_v3d_step_device": (i, [v, v, d, i, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_step_tide": (i, [v, v, d, i, v, v, v, v, i, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_stream": (v, [v]),
        "sl3dgpu_v3d_set_start": (i, [v, v, i]),
        "sl3dgpu_v3d_start_taken": (i, [v]),
        "sl3dgpu_v3d_state_coefficients": (i, [v, v, ctypes.POINTER(c_void_p), ctypes.POINTER(ctypes.c_longlong)]),
        "sl3dgpu_v3d_run": (i, [v, v, P_double, i, i, v, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_adjoint_run": (i, [v, P_double, i, i, i, v, v, v, v, v, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_sample_volumes": (i, [v, v]),
        "sl3dgpu_v3d_tangent_run": (i, [v, P_double, i, i, v, v, v, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_run_many": (i, [i, v, v, v, v, i, v, v, v, v, i, v]),
        "sl3dgpu_v3d_state_coefficients_host": (i, [v, v, v]),
        "sl3dgpu_v3d_assembled_band": (i, [v, i, d, i, i, P_double, ctypes.c_longlong, P_int, P_int]),
        "sl3dgpu_v3d_surface_device": (i, [v, i, v]),
        "sl3dgpu_v3d_set_ocean": (i, [v, ctypes.POINTER(OceanOptions)]),
        "sl3dgpu_v3d_ocean_grid": (i, [v, P_int, P_int, P_double, P_double]),
        "sl3dgpu_v3d_step_ocean": (i, [v, v, d, i, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_run_ocean": (i, [v, v, P_double, i, i, v, v, v, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_sea_level": (i, [v, v, v, ctypes.POINTER(SleResult)]),
        "sl3dgpu_v3d_step_migrating": (i, [v, v, d, i, v, v, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_run_migrating": (i, [v, v, P_double, i, i, v, v, v, v, v, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_ocean_function": (i, [v, v]),
        "sl3dgpu_v3d_effective_love": (i, [v, i, d, P_double]),
        "sl3dgpu_v3d_start_step": (i, [v, v, d, i, v]),
        "sl3dgpu_v3d_step_start_strain": (i, [v, v]),
        "sl3dgpu_v3d_step_respond": (i, [v, v]),
        "sl3dgpu_v3d_step_add_channels": (i, [v, v, v]),
        "sl3dgpu_v3d_step_strain_of": (i, [v, v]),
        "sl3dgpu_v3d_step_converge": (i, [v, v, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_step_finish": (i, [v, v]),
        "sl3dgpu_v3d_step_forces": (i, [v, v, v, v]),
        "sl3dgpu_v3d_step_apply": (i, [v, v, v]),
        "sl3dgpu_v3d_step_solve": (i, [v, v, v, ctypes.POINTER(StepInfo)]),
        "sl3dgpu_v3d_relative_change": (i, [v, v, v, P_double]),
        "sl3dgpu_v3d_layout": (i, [v] + [ctypes.POINTER(ctypes.c_longlong)] * 4),
        "sl3dgpu_v3d_solution_layout": (i, [v, i, ctypes.POINTER(ctypes.c_longlong), P_int,
                                            ctypes.POINTER(ctypes.c_longlong), P_int]),
        "sl3dgpu_v3d_synthesise_tensor": (i, [v, v, v, v, v]),
        "sl3dgpu_v3d_analyse_tensor": (i, [v, v, v, v, v]),
        "sl3dgpu_v3d_degree_forces": (i, [v, v, v, v]),
        "sl3dgpu_v3d_strain_of_solutions": (i, [v, v, v, v]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _SIGNED = True


def standard_earth(elements: int, kelvin_fraction: float = 0.0, kelvin_div: float = 10.0):
    """The measured configurations' layered Earth (four layers)."""
    _signatures()
    layers = (Layer * 4)()
    check(lib().sl3dgpu_standard_earth(elements, kelvin_fraction, kelvin_div, layers))
    return layers


class State:
    """Viscoelastic3D::State: the memory tensors and the strain cache, on the GPU."""

    def __init__(self, op: "Viscoelastic3D"):
        self._op = op
        h = c_void_p()
        check(lib().sl3dgpu_v3d_zero_state(op._h, ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().sl3dgpu_v3d_free_state(h)
            self._h = None

    def device_coefficients(self):
        """(device address, count of doubles) of the strain coefficients in
        the device layout (address 0 before the first step)."""
        ptr, count = c_void_p(), ctypes.c_longlong()
        check(lib().sl3dgpu_v3d_state_coefficients(self._op._h, self._h, ctypes.byref(ptr), ctypes.byref(count)))
        return ptr.value or 0, count.value

    def device_layout_coefficients(self) -> np.ndarray:
        """A host copy of the strain coefficients in the device layout (what
        Viscoelastic3D.set_start takes)."""
        _, count = self.device_coefficients()
        out = np.zeros(count, dtype=np.float64)
        check(lib().sl3dgpu_v3d_state_coefficients_host(self._op._h, self._h, out.ctypes.data))
        return out

    def strain_coefficients(self) -> np.ndarray:
        """The strain coefficients, reference layouts (node-major spin -2, -1, 0 blocks)."""
        out = np.zeros(self._op.spectral_size, dtype=np.complex128)
        check(lib().sl3dgpu_v3d_state_strain(self._op._h, self._h, out.ctypes.data))
        return out


class Viscoelastic3D:
    """The GPU 3D viscoelastic operator (Viscoelastic3D)."""

    def __init__(self, layers, options: Options):
        _signatures()
        h = c_void_p()
        check(lib().sl3dgpu_v3d_create(layers, len(layers), ctypes.byref(options), ctypes.byref(h)))
        self._h = h
        self.options = options
        self.lmax = options.lmax
        P, nt, nph = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().sl3dgpu_v3d_shape(h, ctypes.byref(P), ctypes.byref(nt), ctypes.byref(nph)))
        self.node_count, self.ntheta, self.nphi = P.value, nt.value, nph.value
        self.radius = np.empty(self.node_count)
        self.element = np.empty(self.node_count, dtype=np.int32)
        check(lib().sl3dgpu_v3d_nodes(h, self.radius.ctypes.data_as(P_double), self.element.ctypes.data_as(P_int)))
        self.theta = np.empty(self.ntheta)
        self.weights = np.empty(self.ntheta)
        check(lib().sl3dgpu_v3d_colatitudes(h, self.theta.ctypes.data_as(P_double),
                                            self.weights.ctypes.data_as(P_double)))
        length, time, sigma = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib().sl3dgpu_v3d_scales(h, ctypes.byref(length), ctypes.byref(time), ctypes.byref(sigma)))
        self.length_scale, self.time_scale, self.surface_density_scale = length.value, time.value, sigma.value
        L = self.lmax
        self.spectral_size = ((L + 1) ** 2 - 4 + (L + 1) ** 2 - 1 + (L + 1) * (L + 2) // 2) * self.node_count

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().sl3dgpu_v3d_destroy(h)
            self._h = None

    @property
    def values(self) -> int:
        return self.node_count * self.ntheta * self.nphi

    def set_delta(self, samples) -> None:
        """delta over every node's grid: a host numpy array or a CUDA torch tensor."""
        if isinstance(samples, np.ndarray):
            a = np.ascontiguousarray(samples, dtype=np.float64).ravel()
            assert a.size == self.values
            check(lib().sl3dgpu_v3d_set_delta(self._h, a.ctypes.data, 0))
        else:
            assert samples.is_cuda and samples.numel() == self.values and samples.is_contiguous()
            check(lib().sl3dgpu_v3d_set_delta(self._h, samples.data_ptr(), 1))

    def ZeroState(self) -> State:
        return State(self)

    def Step(self, state: State, dt: float, scheme="sdirk2", load0=None, load1=None, tide0=None,
             tide1=None) -> StepInfo:
        """One step of length dt (non-dimensional) under the load channel and,
        given, the tide channel (Viscoelastic3D::Step's load and tide: (l, m >= 0)
        coefficients at the step's start and end; a tide has no degree-0 or
        degree-1 part beyond its degree-0 centrifugal mean)."""
        code = SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        info = StepInfo()
        a = None if load0 is None else np.ascontiguousarray(load0, dtype=np.complex128)
        b = None if load1 is None else np.ascontiguousarray(load1, dtype=np.complex128)
        if tide0 is None and tide1 is None:
            check(lib().sl3dgpu_v3d_step(self._h, state._h, float(dt), code,
                                         None if a is None else a.ctypes.data,
                                         None if b is None else b.ctypes.data, ctypes.byref(info)))
            return info
        c = None if tide0 is None else np.ascontiguousarray(tide0, dtype=np.complex128)
        e = None if tide1 is None else np.ascontiguousarray(tide1, dtype=np.complex128)
        ptr = lambda x: None if x is None else x.ctypes.data
        check(lib().sl3dgpu_v3d_step_tide(self._h, state._h, float(dt), code, ptr(a), ptr(b), ptr(c), ptr(e), 0,
                                          ctypes.byref(info)))
        return info

    def StepDevice(self, state: State, dt: float, scheme, load0, load1) -> StepInfo:
        """Step with the load coefficients already in device memory (CUDA torch tensors)."""
        code = SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        info = StepInfo()
        check(lib().sl3dgpu_v3d_step_device(self._h, state._h, float(dt), code,
                                            None if load0 is None else load0.data_ptr(),
                                            None if load1 is None else load1.data_ptr(), ctypes.byref(info)))
        return info

    def set_start(self, coefficients) -> None:
        """The warm start of the next step (Converge's start): coefficients in
        the device layout (a CUDA torch tensor of doubles, or a numpy array),
        None to disarm. Kept only if its first residual beats the plain start's."""
        if coefficients is None:
            check(lib().sl3dgpu_v3d_set_start(self._h, None, 0))
        elif hasattr(coefficients, "data_ptr"):
            check(lib().sl3dgpu_v3d_set_start(self._h, coefficients.data_ptr(), 1))
        else:
            arr = np.ascontiguousarray(coefficients, dtype=np.float64)
            check(lib().sl3dgpu_v3d_set_start(self._h, arr.ctypes.data, 0))

    @property
    def start_taken(self) -> bool:
        return bool(lib().sl3dgpu_v3d_start_taken(self._h))

    @property
    def stream(self) -> int:
        """The CUDA stream (cudaStream_t) the operator's kernels run on."""
        return lib().sl3dgpu_v3d_stream(self._h) or 0

    def residual_history(self) -> np.ndarray:
        """The last step's pass residuals, the stages in turn."""
        n = lib().sl3dgpu_v3d_residual_history(self._h, None, 0)
        out = np.zeros(max(n, 0))
        if n > 0:
            lib().sl3dgpu_v3d_residual_history(self._h, out.ctypes.data_as(P_double), n)
        return out

    def correction_history(self) -> np.ndarray:
        """The mixed form's last step: every FP32 correction pass's relative change."""
        n = lib().sl3dgpu_v3d_correction_history(self._h, None, 0)
        out = np.zeros(max(n, 0))
        if n > 0:
            lib().sl3dgpu_v3d_correction_history(self._h, out.ctypes.data_as(P_double), n)
        return out

    def sample_volumes(self) -> np.ndarray:
        """The volume each grid sample stands for (jac w_q r^2 of its memory
        node times 2 pi w_theta / nphi of its colatitude), node-major."""
        out = np.zeros(self.values)
        check(lib().sl3dgpu_v3d_sample_volumes(self._h, out.ctypes.data))
        return out

    def Surface(self, component="U") -> np.ndarray:
        code = COMPONENTS[component] if isinstance(component, str) else int(component)
        out = np.zeros((self.lmax + 1) * (self.lmax + 2) // 2, dtype=np.complex128)
        check(lib().sl3dgpu_v3d_surface(self._h, code, out.ctypes.data))
        return out

    def SurfaceDevice(self, component, out) -> None:
        """The surface coefficients into a CUDA complex128 tensor of (lmax + 1)(lmax + 2) / 2
        values, stream-ordered on the operator's stream, without waiting."""
        code = COMPONENTS[component] if isinstance(component, str) else int(component)
        assert out.is_cuda and out.numel() == (self.lmax + 1) * (self.lmax + 2) // 2 and out.is_contiguous()
        check(lib().sl3dgpu_v3d_surface_device(self._h, code, out.data_ptr()))

    def SurfaceToroidal(self) -> np.ndarray:
        """Viscoelastic3D::SurfaceToroidal: the surface W per (l, m >= 0)."""
        return self.Surface(3)

    def assembled_band(self, l: int, toroidal: bool = False, scheme: int = 1, dt: float = 0.0) -> np.ndarray:
        """Degree l's assembled, unscaled upper band ((kd + 1) x ndof, LAPACK
        storage, column-major as a (ndof, kd + 1) array) in the flavour of
        `scheme` (0 exponential trapezoid, 1 backward Euler) and `dt` (0: the
        elastic flavour), as the GPU assembled it."""
        n, kd = ctypes.c_int(), ctypes.c_int()
        check(lib().sl3dgpu_v3d_assembled_band(self._h, scheme, dt, int(toroidal), l, None, 0, ctypes.byref(n),
                                                ctypes.byref(kd)))
        out = np.empty((n.value, kd.value + 1))
        check(lib().sl3dgpu_v3d_assembled_band(self._h, scheme, dt, int(toroidal), l,
                                                out.ctypes.data_as(P_double), out.size, None, None))
        return out

    def InertiaMoment(self) -> float:
        """Viscoelastic3D::InertiaMoment of the last step's solutions."""
        out = ctypes.c_double()
        check(lib().sl3dgpu_v3d_inertia_moment(self._h, ctypes.byref(out)))
        return out.value

    def StartStep(self, state: State, dt: float, scheme=1, load0=None) -> OpenStep:
        """Viscoelastic3D::StartStep: one stage opened for a driver's own iteration."""
        return OpenStep(self, state, dt, scheme, load0)

    def layout(self) -> dict:
        """The device layouts' sizes: complex spectral coefficients, grid values
        (every node), spheroidal and toroidal solution values."""
        vals = [ctypes.c_longlong() for _ in range(4)]
        check(lib().sl3dgpu_v3d_layout(self._h, *(ctypes.byref(x) for x in vals)))
        return dict(zip(("spectral", "grid", "spheroidal", "toroidal"), (x.value for x in vals)))

    def solution_layout(self, l: int) -> dict:
        so, to = ctypes.c_longlong(), ctypes.c_longlong()
        sn, tn = ctypes.c_int(), ctypes.c_int()
        check(lib().sl3dgpu_v3d_solution_layout(self._h, l, ctypes.byref(so), ctypes.byref(sn), ctypes.byref(to),
                                                ctypes.byref(tn)))
        return {"sph_offset": so.value, "sph_dofs": sn.value, "tor_offset": to.value, "tor_dofs": tn.value}

    # -- GridCoupling's maps (CUDA tensors in the device layouts)

    def SynthesiseTensor(self, spectral):
        import torch

        n = self.layout()["grid"]
        c0 = torch.empty(n, dtype=torch.complex128, device="cuda")
        c1 = torch.empty(n, dtype=torch.complex128, device="cuda")
        r = torch.empty(n, dtype=torch.float64, device="cuda")
        check(lib().sl3dgpu_v3d_synthesise_tensor(self._h, spectral.data_ptr(), c0.data_ptr(), c1.data_ptr(),
                                                  r.data_ptr()))
        return c0, c1, r

    def AnalyseTensor(self, c0, c1, r):
        import torch

        out = torch.empty(self.layout()["spectral"], dtype=torch.complex128, device="cuda")
        check(lib().sl3dgpu_v3d_analyse_tensor(self._h, c0.data_ptr(), c1.data_ptr(), r.data_ptr(), out.data_ptr()))
        return out

    def DegreeForces(self, spectral):
        import torch

        lay = self.layout()
        sph = torch.empty(lay["spheroidal"], dtype=torch.complex128, device="cuda")
        tor = torch.empty(max(lay["toroidal"], 1), dtype=torch.complex128, device="cuda")
        check(lib().sl3dgpu_v3d_degree_forces(self._h, spectral.data_ptr(), sph.data_ptr(), tor.data_ptr()))
        return sph, tor

    def StrainOfSolutions(self, sph, tor):
        import torch

        out = torch.empty(self.layout()["spectral"], dtype=torch.complex128, device="cuda")
        check(lib().sl3dgpu_v3d_strain_of_solutions(self._h, sph.data_ptr(), tor.data_ptr(), out.data_ptr()))
        return out

    # -- the ocean closure (Evolution3D's Coupled::Closure, frozen shorelines)

    def ocean_grid(self):
        """The sea-level grid: (colatitudes, quadrature weights, longitudes)."""
        nt, nph = ctypes.c_int(), ctypes.c_int()
        check(lib().sl3dgpu_v3d_ocean_grid(self._h, ctypes.byref(nt), ctypes.byref(nph), None, None))
        theta, w = np.empty(nt.value), np.empty(nt.value)
        check(lib().sl3dgpu_v3d_ocean_grid(self._h, None, None, theta.ctypes.data_as(P_double),
                                           w.ctypes.data_as(P_double)))
        return theta, w, nph.value

    def set_ocean(self, ocean_function, rotation: int = 1, water_density: float = 1000.0,
                  rotation_frequency: float = 7.27220521664304e-05, polar_moment: float = 8.0359e37,
                  equatorial_moment: float = 8.0096e37, rtol: float = 1e-10, max_iterations: int = 200,
                  anderson_memory: int = 5) -> None:
        """The ocean of the coupled steps (None removes it): its function on
        the sea-level grid, the rotational feedback (0 None, 1 Axial, 2 Full)
        and the sea-level solve's tolerance, budget and mixer."""
        if ocean_function is None:
            check(lib().sl3dgpu_v3d_set_ocean(self._h, None))
            return
        theta, _, nphi = self.ocean_grid()
        f = np.ascontiguousarray(ocean_function, dtype=np.float64).ravel()
        if f.size != theta.size * nphi:
            raise ValueError("the ocean function lives on the sea-level grid")
        o = OceanOptions(f.ctypes.data, int(rotation), float(water_density), float(rotation_frequency),
                         float(polar_moment), float(equatorial_moment), float(rtol), int(max_iterations),
                         int(anderson_memory))
        check(lib().sl3dgpu_v3d_set_ocean(self._h, ctypes.byref(o)))

    def set_migrating_ocean(self, ice_thickness, sea_level, forced_land=None, rotation: int = 1,
                            water_density: float = 1000.0, ice_density: float = 917.0,
                            rotation_frequency: float = 7.27220521664304e-05, polar_moment: float = 8.0359e37,
                            equatorial_moment: float = 8.0096e37, rtol: float = 1e-10,
                            max_nonlinear_iterations: int = 50, ocean_function=None) -> None:
        """An ocean whose shorelines migrate (Evolution3D::RunMigrating): the
        background state's ice thickness and sea level (fields on the
        sea-level grid, model length unit) and the land held (a mask, None:
        none); its ocean function is flotation's (a given one must equal
        it). Every pass solves the nonlinear sea-level equation from it."""
        theta, _, nphi = self.ocean_grid()
        n = theta.size * nphi
        ice = np.ascontiguousarray(ice_thickness, dtype=np.float64).ravel()
        sea = np.ascontiguousarray(sea_level, dtype=np.float64).ravel()
        land = None if forced_land is None else np.ascontiguousarray(forced_land, dtype=np.uint8).ravel()
        given = None if ocean_function is None else np.ascontiguousarray(ocean_function, dtype=np.float64).ravel()
        if ice.size != n or sea.size != n or (land is not None and land.size != n) or \
                (given is not None and given.size != n):
            raise ValueError("the background's fields live on the sea-level grid")
        o = OceanOptions(None if given is None else given.ctypes.data, int(rotation), float(water_density),
                         float(rotation_frequency), float(polar_moment), float(equatorial_moment), float(rtol), 1,
                         0, 1, float(ice_density), ice.ctypes.data, sea.ctypes.data,
                         None if land is None else land.ctypes.data, int(max_nonlinear_iterations))
        check(lib().sl3dgpu_v3d_set_ocean(self._h, ctypes.byref(o)))

    def StepMigrating(self, state: State, dt: float, scheme="sdirk2", ice0=None, ice1=None, load0=None,
                      load1=None) -> StepInfo:
        """One coupled step under migrating shorelines: the ice thickness at
        the step's two ends and the direct loads beside it (None: none)."""
        code = SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        arrays = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (ice0, ice1, load0, load1)]
        info = StepInfo()
        check(lib().sl3dgpu_v3d_step_migrating(self._h, state._h, float(dt), code,
                                               *(None if a is None else a.ctypes.data for a in arrays),
                                               ctypes.byref(info)))
        return info

    def OceanFunction(self):
        """The last closure's ocean function (a field on the sea-level grid)."""
        theta, _, nphi = self.ocean_grid()
        out = np.zeros(theta.size * nphi)
        check(lib().sl3dgpu_v3d_ocean_function(self._h, out.ctypes.data))
        return out

    def StepOcean(self, state: State, dt: float, scheme="sdirk2", load0=None, load1=None) -> StepInfo:
        """One coupled step under the direct (non-ocean) load fields on the
        sea-level grid at the step's start and end (non-dimensional)."""
        code = SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        info = StepInfo()
        a = None if load0 is None else np.ascontiguousarray(load0, dtype=np.float64)
        b = None if load1 is None else np.ascontiguousarray(load1, dtype=np.float64)
        check(lib().sl3dgpu_v3d_step_ocean(self._h, state._h, float(dt), code, None if a is None else a.ctypes.data,
                                           None if b is None else b.ctypes.data, ctypes.byref(info)))
        return info

    def SeaLevel(self):
        """The last closure's relative sea level change ((l, m >= 0)
        coefficients, model length unit), angular velocity and solve scalars."""
        out = np.zeros((self.lmax + 1) * (self.lmax + 2) // 2, dtype=np.complex128)
        omega = np.zeros(3)
        res = SleResult()
        check(lib().sl3dgpu_v3d_sea_level(self._h, out.ctypes.data, omega.ctypes.data, ctypes.byref(res)))
        return out, omega, res

    def effective_love(self, scheme: int, dt: float) -> dict:
        """A one-stage flavour's effective Love numbers (model units)."""
        L = self.lmax
        out = np.zeros(6 * (L + 1) + 4)
        check(lib().sl3dgpu_v3d_effective_love(self._h, int(scheme), float(dt), out.ctypes.data_as(P_double)))
        names = ("h", "k", "l", "ht", "kt", "lt")
        love = {n: out[i * (L + 1):(i + 1) * (L + 1)].copy() for i, n in enumerate(names)}
        love.update(hc=out[6 * (L + 1)], kc=out[6 * (L + 1) + 1], m=out[6 * (L + 1) + 2], mc=out[6 * (L + 1) + 3])
        return love


class OpenStep:
    """Viscoelastic3D::OpenStep (include/sl3dpp/Viscoelastic3D.hpp:440-640): one
    stage opened on the operator's buffers for a driver's own within-step
    iteration. Strain coefficients are CUDA complex128 tensors in the device
    layout; the solutions stay in the operator (Surface, InertiaMoment read
    them)."""

    def __init__(self, op: "Viscoelastic3D", state: State, dt: float, scheme=1, load0=None):
        import torch

        self.op, self.state = op, state
        code = SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
        a = None if load0 is None else np.ascontiguousarray(load0, dtype=np.complex128)
        check(lib().sl3dgpu_v3d_start_step(op._h, state._h, float(dt), code, None if a is None else a.ctypes.data))
        self.size = op.layout()["spectral"]
        self._torch = torch

    def _new(self):
        return self._torch.empty(self.size, dtype=self._torch.complex128, device="cuda")

    def StartStrain(self):
        out = self._new()
        check(lib().sl3dgpu_v3d_step_start_strain(self.op._h, out.data_ptr()))
        return out

    def Respond(self, strain=None) -> None:
        """The channel-free solutions of a strain (None: the start strain)."""
        check(lib().sl3dgpu_v3d_step_respond(self.op._h, None if strain is None else strain.data_ptr()))

    def AddChannels(self, load=None, tide=None) -> None:
        a = None if load is None else np.ascontiguousarray(load, dtype=np.complex128)
        b = None if tide is None else np.ascontiguousarray(tide, dtype=np.complex128)
        check(lib().sl3dgpu_v3d_step_add_channels(self.op._h, None if a is None else a.ctypes.data,
                                                  None if b is None else b.ctypes.data))

    def StrainOf(self):
        out = self._new()
        check(lib().sl3dgpu_v3d_step_strain_of(self.op._h, out.data_ptr()))
        return out

    def RelativeChange(self, next_, now) -> float:
        out = ctypes.c_double()
        check(lib().sl3dgpu_v3d_relative_change(self.op._h, next_.data_ptr(), now.data_ptr(), ctypes.byref(out)))
        return out.value

    def Close(self, load=None, tide=None):
        """The stage under known channels by the operator's own iteration."""
        a = None if load is None else np.ascontiguousarray(load, dtype=np.complex128)
        b = None if tide is None else np.ascontiguousarray(tide, dtype=np.complex128)
        out = self._new()
        info = StepInfo()
        check(lib().sl3dgpu_v3d_step_converge(self.op._h, None if a is None else a.ctypes.data,
                                              None if b is None else b.ctypes.data, out.data_ptr(),
                                              ctypes.byref(info)))
        return out, info

    def Finish(self, strain=None) -> None:
        check(lib().sl3dgpu_v3d_step_finish(self.op._h, None if strain is None else strain.data_ptr()))

    # the conjugate-gradient close's pieces (Options solver = 1)

    def _columns(self):
        lay = self.op.layout()
        return self._torch.zeros(lay["spheroidal"] + max(lay["toroidal"], 1), dtype=self._torch.complex128,
                                 device="cuda")

    def Forces(self, load=None, tide=None):
        a = None if load is None else np.ascontiguousarray(load, dtype=np.complex128)
        b = None if tide is None else np.ascontiguousarray(tide, dtype=np.complex128)
        out = self._columns()
        check(lib().sl3dgpu_v3d_step_forces(self.op._h, None if a is None else a.ctypes.data,
                                            None if b is None else b.ctypes.data, out.data_ptr()))
        return out

    def Apply(self, x):
        out = self._columns()
        check(lib().sl3dgpu_v3d_step_apply(self.op._h, x.data_ptr(), out.data_ptr()))
        return out

    def Solve(self, forces):
        out = self._columns()
        info = StepInfo()
        check(lib().sl3dgpu_v3d_step_solve(self.op._h, forces.data_ptr(), out.data_ptr(), ctypes.byref(info)))
        return out, info


class Evolution3D:
    """Evolution3D::Run for a body without an ocean and without rotational
    feedback (GRDSolver::NoOceanState): node 0 is the instantaneous elastic
    response, each later node one step of the operator under the direct
    loads at its two ends. Snapshots carry the surface U and phi
    coefficients (l, m >= 0) and the node's step info."""

    def __init__(self, op: Viscoelastic3D, scheme="sdirk2"):
        self.op = op
        self.scheme = SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)

    def Run(self, times, loads, state: State | None = None):
        times = np.ascontiguousarray(times, dtype=np.float64)
        loads = np.ascontiguousarray(loads, dtype=np.complex128)
        n = times.size
        lm = (self.op.lmax + 1) * (self.op.lmax + 2) // 2
        if loads.shape != (n, lm):
            raise ValueError("one load (l(l+1)/2 + m coefficients) per node")
        state = state if state is not None else self.op.ZeroState()
        U = np.zeros((n, lm), dtype=np.complex128)
        phi = np.zeros((n, lm), dtype=np.complex128)
        infos = (StepInfo * max(n, 1))()
        check(lib().sl3dgpu_v3d_run(self.op._h, state._h, times.ctypes.data_as(P_double), n, self.scheme,
                                    loads.ctypes.data, U.ctypes.data, phi.ctypes.data, infos))
        return {"U": U, "phi": phi, "infos": [infos[k] for k in range(n)], "state": state}

    def Adjoint(self, times, loads, u_dual=None, phi_dual=None, gradient=True, stride=1):
        """The discrete adjoint of Run from a zero state (AdjointSolver3D::
        FirstOrderKernels under AdjointMethod::Discrete, include/sl3dpp/
        Adjoint3D.hpp:241-322): for J = sum_n <u_dual_n, U_n> +
        <phi_dual_n, phi_n> (the surface pairing of real fields, m > 0 twice),
        the load and tide kernels per node (dJ = sum_n <kernel_n, dL_n>), dJ/d delta at
        every grid sample (node-major, as set_delta's samples) and J itself.
        stride: the forward run's states kept every stride-th node, the gaps
        rebuilt by its own steps during the sweep."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        loads = np.ascontiguousarray(loads, dtype=np.complex128)
        n = times.size
        lm = (self.op.lmax + 1) * (self.op.lmax + 2) // 2
        if loads.shape != (n, lm):
            raise ValueError("one load (l(l+1)/2 + m coefficients) per node")
        duals = []
        for g in (u_dual, phi_dual):
            if g is None:
                duals.append(None)
                continue
            g = np.ascontiguousarray(g, dtype=np.complex128)
            if g.shape != (n, lm):
                raise ValueError("one dual (l(l+1)/2 + m coefficients) per node")
            duals.append(g)
        kernels = np.zeros((n, lm), dtype=np.complex128)
        tides = np.zeros((n, lm), dtype=np.complex128)
        grad = np.zeros(self.op.values) if gradient else None
        objective = ctypes.c_double()
        infos = (StepInfo * max(n, 1))()
        check(lib().sl3dgpu_v3d_adjoint_run(
            self.op._h, times.ctypes.data_as(P_double), n, self.scheme, int(stride), loads.ctypes.data,
            None if duals[0] is None else duals[0].ctypes.data, None if duals[1] is None else duals[1].ctypes.data,
            kernels.ctypes.data, tides.ctypes.data, None if grad is None else grad.ctypes.data,
            ctypes.byref(objective), infos))
        return {"objective": objective.value, "load_kernels": kernels, "tide_kernels": tides, "delta_gradient": grad,
                "infos": [infos[k] for k in range(n)]}

    def Tangent(self, times, loads, delta_direction=None, load_directions=None):
        """The discrete tangent-linear run beside Run from a zero state
        (TangentLinearSolver3D's discrete method): the derivative of U and
        phi at every node along a log-viscosity direction over every grid
        sample and along per-node load directions (either None)."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        loads = np.ascontiguousarray(loads, dtype=np.complex128)
        n = times.size
        lm = (self.op.lmax + 1) * (self.op.lmax + 2) // 2
        if loads.shape != (n, lm):
            raise ValueError("one load (l(l+1)/2 + m coefficients) per node")
        p = None if delta_direction is None else np.ascontiguousarray(delta_direction, dtype=np.float64).ravel()
        if p is not None and p.size != self.op.values:
            raise ValueError("one direction value per grid sample")
        dl = None if load_directions is None else np.ascontiguousarray(load_directions, dtype=np.complex128)
        if dl is not None and dl.shape != (n, lm):
            raise ValueError("one load direction per node")
        U = np.zeros((n, lm), dtype=np.complex128)
        phi = np.zeros((n, lm), dtype=np.complex128)
        infos = (StepInfo * max(n, 1))()
        check(lib().sl3dgpu_v3d_tangent_run(self.op._h, times.ctypes.data_as(P_double), n, self.scheme,
                                            loads.ctypes.data, None if p is None else p.ctypes.data,
                                            None if dl is None else dl.ctypes.data, U.ctypes.data, phi.ctypes.data,
                                            infos))
        return {"U": U, "phi": phi, "infos": [infos[k] for k in range(n)]}

    def Instantaneous(self, load):
        out = self.Run(np.zeros(1), np.asarray(load)[None, :])
        return {"U": out["U"][0], "phi": out["phi"][0]}

    def RunOcean(self, times, loads, state: State | None = None):
        """Evolution3D::Run with the operator's ocean (set_ocean): loads are
        the direct (non-ocean) load fields on the sea-level grid per node;
        snapshots carry U, phi and the relative sea level change as
        coefficients and the angular velocity."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        theta, _, nphi = self.op.ocean_grid()
        n = times.size
        loads = np.ascontiguousarray(loads, dtype=np.float64).reshape(n, theta.size * nphi)
        lm = (self.op.lmax + 1) * (self.op.lmax + 2) // 2
        state = state if state is not None else self.op.ZeroState()
        U, phi, slc = (np.zeros((n, lm), dtype=np.complex128) for _ in range(3))
        omega = np.zeros((n, 3))
        infos = (StepInfo * max(n, 1))()
        check(lib().sl3dgpu_v3d_run_ocean(self.op._h, state._h, times.ctypes.data_as(P_double), n, self.scheme,
                                          loads.ctypes.data, U.ctypes.data, phi.ctypes.data, slc.ctypes.data,
                                          omega.ctypes.data, infos))
        return {"U": U, "phi": phi, "sea_level": slc, "omega": omega, "infos": [infos[k] for k in range(n)],
                "state": state}

    def RunMigrating(self, times, ice, loads=None, state: State | None = None):
        """Evolution3D::RunMigrating with the operator's migrating ocean
        (set_migrating_ocean): the ice thickness per node (and direct loads,
        None: none) on the sea-level grid; snapshots carry U, phi, the
        relative sea level change, the angular velocity and each node's
        ocean function."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        theta, _, nphi = self.op.ocean_grid()
        n, size = times.size, theta.size * nphi
        ice = np.ascontiguousarray(ice, dtype=np.float64).reshape(n, size)
        loads = None if loads is None else np.ascontiguousarray(loads, dtype=np.float64).reshape(n, size)
        lm = (self.op.lmax + 1) * (self.op.lmax + 2) // 2
        state = state if state is not None else self.op.ZeroState()
        U, phi, slc = (np.zeros((n, lm), dtype=np.complex128) for _ in range(3))
        omega = np.zeros((n, 3))
        oceans = np.zeros((n, size))
        infos = (StepInfo * max(n, 1))()
        check(lib().sl3dgpu_v3d_run_migrating(self.op._h, state._h, times.ctypes.data_as(P_double), n, self.scheme,
                                              ice.ctypes.data, None if loads is None else loads.ctypes.data,
                                              U.ctypes.data, phi.ctypes.data, slc.ctypes.data, omega.ctypes.data,
                                              oceans.ctypes.data, infos))
        return {"U": U, "phi": phi, "sea_level": slc, "omega": omega, "ocean": oceans,
                "infos": [infos[k] for k in range(n)], "state": state}
