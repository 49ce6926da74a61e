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
        "oracle_degree_band": (i, [v, i, i, d, i, i, d, i, i, P_double, P_int, P_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def degree_band(layers, ngll: int, l: int, toroidal: bool = False, relaxed: bool = True, scheme: int = 1,
                dt: float = 0.0, eps: float = 1e-8) -> np.ndarray:
    """The oracle's assembled, unscaled upper band of one degree, (ndof, kd + 1):
    relaxed, the 3D step's flavour (long-term material, the point shear of a
    step of `scheme` and model-unit length `dt`, 0 the elastic one); else the
    unrelaxed material without point shear."""
    L = load()
    n, kd = ctypes.c_int(), ctypes.c_int()
    args = (ctypes.cast(layers, ctypes.c_void_p), len(layers), ngll, eps, int(relaxed), scheme, dt, int(toroidal), l)
    assert L.oracle_degree_band(*args, None, ctypes.byref(n), ctypes.byref(kd)) == 0
    out = np.empty((n.value, kd.value + 1))
    assert L.oracle_degree_band(*args, ptr(out), ctypes.byref(n), ctypes.byref(kd)) == 0
    return out


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


# -- the 3D step --------------------------------------------------------------------------

import ctypes as _ct


class Layer(_ct.Structure):
    """sl3dgpu_layer (include/sl3dgpu.h)."""
    _fields_ = [("r0", _ct.c_double), ("r1", _ct.c_double), ("fluid", _ct.c_int), ("elements", _ct.c_int),
                ("rho0", _ct.c_double), ("rho1", _ct.c_double), ("kappa0", _ct.c_double), ("kappa1", _ct.c_double),
                ("mu0", _ct.c_double), ("mu1", _ct.c_double), ("viscosity", _ct.c_double),
                ("kelvin_fraction", _ct.c_double), ("kelvin_viscosity", _ct.c_double)]


class Options(_ct.Structure):
    """sl3dgpu_v3d_options (include/sl3dgpu.h)."""
    _fields_ = [("lmax", _ct.c_int), ("ngll", _ct.c_int), ("eps", _ct.c_double), ("oversampling", _ct.c_double),
                ("max_iterations", _ct.c_int), ("rtol", _ct.c_double), ("damping", _ct.c_double),
                ("anderson_memory", _ct.c_int), ("anderson_rate", _ct.c_double), ("precision", _ct.c_int),
                ("correction_rtol", _ct.c_double), ("solver", _ct.c_int),
                ("solve_rtol", _ct.c_double), ("solve_max_iterations", _ct.c_int),
                ("warm_start", _ct.c_int), ("fp64_emulation", _ct.c_int), ("correction_memory", _ct.c_int)]


class StepInfo(_ct.Structure):
    _fields_ = [("iterations", _ct.c_int), ("residual", _ct.c_double), ("converged", _ct.c_int),
                ("mixed_passes", _ct.c_int), ("correction_passes", _ct.c_int),
                ("solve_iterations", _ct.c_int)]


def default_options(lmax, ngll=5, **kw):
    o = Options(lmax=lmax, ngll=ngll, eps=1e-8, oversampling=1.5, max_iterations=40, rtol=1e-11, damping=1.0,
                anderson_memory=5, anderson_rate=0.5, precision=0, correction_rtol=1e-5,
                solver=0, solve_rtol=1e-11, solve_max_iterations=200, warm_start=0, fp64_emulation=0,
                correction_memory=0)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class EpOptions(_ct.Structure):
    """sl3dgpu_ep3d_options (include/sl3dgpu.h)."""
    _fields_ = [("lmax", _ct.c_int), ("ngll", _ct.c_int), ("eps", _ct.c_double), ("oversampling", _ct.c_double)]


# oracle_closure_fn (oracle_step.cpp)
_CLOSURE = _ct.CFUNCTYPE(None, _ct.c_void_p, _ct.c_double, _ct.POINTER(_ct.c_double), _ct.c_int,
                         _ct.POINTER(_ct.c_double), _ct.POINTER(_ct.c_double), _ct.POINTER(_ct.c_double),
                         _ct.c_double, _ct.POINTER(_ct.c_double), _ct.POINTER(_ct.c_double))


def _v3d_sigs(L):
    v, i, d = _ct.c_void_p, _ct.c_int, _ct.c_double
    sig = {
        "oracle_standard_earth": (i, [i, d, d, _ct.POINTER(Layer)]),
        "oracle_v3d_create": (v, [_ct.POINTER(Layer), i, _ct.POINTER(Options)]),
        "oracle_v3d_destroy": (None, [v]),
        "oracle_v3d_node_count": (i, [v]),
        "oracle_v3d_nodes": (None, [v, P_double, P_int]),
        "oracle_v3d_grid": (None, [v, P_int, P_int, P_double, P_double]),
        "oracle_v3d_time_scale": (d, [v]),
        "oracle_v3d_surface_density_scale": (d, [v]),
        "oracle_v3d_set_delta": (None, [v, P_double]),
        "oracle_v3d_zero_state": (v, [v]),
        "oracle_v3d_free_state": (None, [v]),
        "oracle_v3d_step": (i, [v, v, d, i, v, v, _ct.POINTER(StepInfo)]),
        "oracle_v3d_step_tide": (i, [v, v, d, i, v, v, v, v, _ct.POINTER(StepInfo)]),
        "oracle_v3d_surface": (None, [v, i, v]),
        "oracle_v3d_inertia_moment": (d, [v]),
        "oracle_v3d_state_strain": (i, [v, v]),
        "oracle_v3d_residual_history": (i, [v, P_double, i]),
        "oracle_v3d_sample": (i, [v, v, d, v, v, i, P_double, P_double]),
        "oracle_threads": (i, []),
        "oracle_ep3d_create": (v, [_ct.POINTER(Layer), i, _ct.POINTER(EpOptions)]),
        "oracle_v3d_modulus_scale": (d, [v]),
        "oracle_ep3d_set_moduli": (None, [v, v, v]),
        "oracle_ep3d_solve_load": (None, [v, v]),
        "oracle_ep3d_respond": (None, [v]),
        "oracle_ep3d_solve_lateral": (i, [v, v, d, i, _ct.POINTER(StepInfo)]),
        "oracle_v3d_set_closure": (None, [v, _CLOSURE, v]),
        "oracle_v3d_effective_love": (None, [v, i, d, P_double]),
        "oracle_v3d_body": (None, [v, P_double]),
        "oracle_v3d_adjoint_run": (i, [v, P_double, i, i, v, v, v, v, v, P_double, v]),
        "oracle_v3d_tangent_run": (i, [v, P_double, i, i, v, v, v, v, v]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def standard_earth(elements, kelvin_fraction=0.0, kelvin_div=10.0):
    L = load()
    _v3d_sigs(L)
    layers = (Layer * 4)()
    L.oracle_standard_earth(elements, kelvin_fraction, kelvin_div, layers)
    return layers


class OracleStep:
    """The oracle's Viscoelastic3D (CPU FP64), for parity checks."""

    def __init__(self, layers, options):
        self.L = load()
        _v3d_sigs(self.L)
        self.options = options
        self.h = self.L.oracle_v3d_create(layers, len(layers), _ct.byref(options))
        self.P = self.L.oracle_v3d_node_count(self.h)
        nt, nph = _ct.c_int(), _ct.c_int()
        self.L.oracle_v3d_grid(self.h, _ct.byref(nt), _ct.byref(nph), None, None)
        self.ntheta, self.nphi = nt.value, nph.value
        self.theta = np.empty(self.ntheta)
        self.weights = np.empty(self.ntheta)
        self.L.oracle_v3d_grid(self.h, None, None, ptr(self.theta), ptr(self.weights))
        self.radius = np.empty(self.P)
        self.element = np.empty(self.P, dtype=np.int32)
        self.L.oracle_v3d_nodes(self.h, ptr(self.radius), ptr(self.element))
        self.time_scale = self.L.oracle_v3d_time_scale(self.h)
        self.sigma_scale = self.L.oracle_v3d_surface_density_scale(self.h)
        self.state = self.L.oracle_v3d_zero_state(self.h)

    def __del__(self):
        try:
            self.L.oracle_v3d_free_state(self.state)
            self.L.oracle_v3d_destroy(self.h)
        except Exception:
            pass

    def set_delta(self, samples):
        samples = np.ascontiguousarray(samples, dtype=np.float64)
        assert samples.size == self.P * self.ntheta * self.nphi
        self.L.oracle_v3d_set_delta(self.h, ptr(samples))

    def step(self, dt, scheme=2, load0=None, load1=None, tide0=None, tide1=None):
        info = StepInfo()
        cols = [None if c is None else np.ascontiguousarray(c, dtype=np.complex128)
                for c in (load0, load1, tide0, tide1)]
        p = [None if c is None else c.ctypes.data for c in cols]
        if tide0 is None and tide1 is None:
            st = self.L.oracle_v3d_step(self.h, self.state, dt, scheme, p[0], p[1], _ct.byref(info))
        else:
            st = self.L.oracle_v3d_step_tide(self.h, self.state, dt, scheme, *p, _ct.byref(info))
        assert st == 0
        return info

    def adjoint(self, times, scheme, loads, u_dual=None, phi_dual=None):
        """The oracle's discrete adjoint of the run from a zero state: the
        objective, the load and tide kernels per node and dJ/d delta per
        sample."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        loads = np.ascontiguousarray(loads, dtype=np.complex128)
        n = times.size
        duals = [None if g is None else np.ascontiguousarray(g, dtype=np.complex128) for g in (u_dual, phi_dual)]
        kernels = np.zeros_like(loads)
        tides = np.zeros_like(loads)
        grad = np.zeros(self.P * self.ntheta * self.nphi)
        J = _ct.c_double()
        st = self.L.oracle_v3d_adjoint_run(self.h, ptr(times), n, scheme, loads.ctypes.data,
                                           None if duals[0] is None else duals[0].ctypes.data,
                                           None if duals[1] is None else duals[1].ctypes.data,
                                           kernels.ctypes.data, ptr(grad), _ct.byref(J), tides.ctypes.data)
        assert st == 0
        return {"objective": J.value, "load_kernels": kernels, "tide_kernels": tides, "delta_gradient": grad}

    def tangent(self, times, scheme, loads, direction=None, load_directions=None):
        """The oracle's tangent-linear run beside the run from a zero state:
        the derivatives of U and phi per node."""
        times = np.ascontiguousarray(times, dtype=np.float64)
        loads = np.ascontiguousarray(loads, dtype=np.complex128)
        p = None if direction is None else np.ascontiguousarray(direction, dtype=np.float64)
        d = None if load_directions is None else np.ascontiguousarray(load_directions, dtype=np.complex128)
        U, phi = np.zeros_like(loads), np.zeros_like(loads)
        st = self.L.oracle_v3d_tangent_run(self.h, ptr(times), times.size, scheme, loads.ctypes.data,
                                           None if p is None else p.ctypes.data, None if d is None else d.ctypes.data,
                                           U.ctypes.data, phi.ctypes.data)
        assert st == 0
        return {"U": U, "phi": phi}

    def sample(self, dt, passes, load0=None, load1=None):
        """Seconds of a backward Euler stage's start, and of each of `passes`
        passes after it (an array)."""
        a = None if load0 is None else np.ascontiguousarray(load0, dtype=np.complex128)
        b = None if load1 is None else np.ascontiguousarray(load1, dtype=np.complex128)
        t0 = _ct.c_double()
        each = np.zeros(max(passes, 1))
        st = self.L.oracle_v3d_sample(self.h, self.state, dt, None if a is None else a.ctypes.data,
                                      None if b is None else b.ctypes.data, passes, _ct.byref(t0), ptr(each))
        assert st == 0
        return t0.value, each[:passes]

    def residual_history(self):
        n = self.L.oracle_v3d_residual_history(self.h, None, 0)
        out = np.zeros(max(n, 0))
        if n > 0:
            self.L.oracle_v3d_residual_history(self.h, ptr(out), n)
        return out

    def surface(self, component):
        L = self.options.lmax
        out = np.zeros((L + 1) * (L + 2) // 2, dtype=np.complex128)
        self.L.oracle_v3d_surface(self.h, component, out.ctypes.data)
        return out

    # -- the ocean closure (oracle/coupled.py)

    def body(self):
        out = np.zeros(6)
        self.L.oracle_v3d_body(self.h, ptr(out))
        return dict(radius=out[0], g=out[1], G=out[2], length=out[3], mass=out[4], time=out[5])

    def effective_love(self, scheme, dt):
        L = self.options.lmax
        out = np.zeros(6 * (L + 1) + 4)
        self.L.oracle_v3d_effective_love(self.h, scheme, dt, ptr(out))
        return out

    def set_ocean(self, ocean, **kw):
        """Closes every pass with the sea-level equation over `ocean` (a
        field on the sea-level grid, lmax at oversampling 1), the closure of
        oracle/coupled.py; kw: OceanClosure's constants."""
        from oracle.coupled import OceanClosure

        lmax = self.options.lmax
        theta, w, nphi = grid(lmax, 1.0)
        self.sle_grid = (theta, w, nphi)
        transforms = (lambda c: synthesise_real(lmax, theta, nphi, c),
                      lambda f: expand_real(lmax, theta, w, nphi, f),
                      lambda f: float(np.sum(w * f.reshape(theta.size, nphi).sum(axis=1)) * 2 * np.pi / nphi))
        self.closure = OceanClosure(lmax, transforms, self.body(), ocean, **kw)
        size = (lmax + 1) * (lmax + 2) // 2

        def callback(user, t, love, count, u, v, phi, inertia, sigma, psi):
            love_a = np.ctypeslib.as_array(love, (count,)).copy()
            cx = lambda q: np.ctypeslib.as_array(q, (2 * size,)).view(np.complex128).copy()
            s, p = self.closure(t, love_a, cx(u), cx(v), cx(phi), inertia)
            np.ctypeslib.as_array(sigma, (2 * size,))[:] = s.view(np.float64)
            np.ctypeslib.as_array(psi, (2 * size,))[:] = p.view(np.float64)

        self._callback = _CLOSURE(callback)
        self.L.oracle_v3d_set_closure(self.h, self._callback, None)
        self.t = 0.0

    def set_migrating(self, ice, sea_level, forced_land=None, **kw):
        """Closes every pass with the nonlinear sea-level equation from the
        background (ice, sea_level, forced_land on the sea-level grid, model
        length), oracle/coupled.py's MigratingClosure; kw: its constants."""
        from oracle.coupled import MigratingClosure

        lmax = self.options.lmax
        theta, w, nphi = grid(lmax, 1.0)
        self.sle_grid = (theta, w, nphi)
        transforms = (lambda c: synthesise_real(lmax, theta, nphi, c),
                      lambda f: expand_real(lmax, theta, w, nphi, f),
                      lambda f: float(np.sum(w * f.reshape(theta.size, nphi).sum(axis=1)) * 2 * np.pi / nphi))
        state = dict(ice=ice, sea_level=sea_level, forced_land=forced_land)
        self.closure = MigratingClosure(lmax, transforms, self.body(), state, **kw)
        size = (lmax + 1) * (lmax + 2) // 2

        def callback(user, t, love, count, u, v, phi, inertia, sigma, psi):
            love_a = np.ctypeslib.as_array(love, (count,)).copy()
            cx = lambda q: np.ctypeslib.as_array(q, (2 * size,)).view(np.complex128).copy()
            s, p = self.closure(t, love_a, cx(u), cx(v), cx(phi), inertia)
            np.ctypeslib.as_array(sigma, (2 * size,))[:] = s.view(np.float64)
            np.ctypeslib.as_array(psi, (2 * size,))[:] = p.view(np.float64)

        self._callback = _CLOSURE(callback)
        self.L.oracle_v3d_set_closure(self.h, self._callback, None)
        self.t = 0.0

    def step_migrating(self, dt, scheme, ice0, ice1, load0=None, load1=None):
        """One coupled step under migrating shorelines: the ice at its two
        ends and the direct loads beside it (None: none)."""
        self.closure.set_step_ice(self.t, ice0, self.t + dt, ice1)
        if load0 is None and load1 is None:
            self.closure.loads = None
        else:
            n = self.sle_grid[0].size * self.sle_grid[2]
            zero = np.zeros(n)
            self.closure.set_step_loads(self.t, zero if load0 is None else load0, self.t + dt,
                                        zero if load1 is None else load1)
        info = self.step(dt, scheme)
        self.t += dt
        return info

    def step_ocean(self, dt, scheme=2, load0=None, load1=None):
        """One coupled step under the direct load fields at its two ends."""
        n = self.sle_grid[0].size * self.sle_grid[2]
        zero = np.zeros(n)
        self.closure.set_step_loads(self.t, zero if load0 is None else load0, self.t + dt,
                                    zero if load1 is None else load1)
        info = self.step(dt, scheme)
        self.t += dt
        return info

    def sea_level(self):
        """The last closure's relative sea level change (coefficients) and angular velocity."""
        lmax = self.options.lmax
        theta, w, nphi = self.sle_grid
        last = self.closure.last
        return expand_real(lmax, theta, w, nphi, last["sea_level_change"]), np.asarray(last["angular_velocity"])


class OraclePerturbation(OracleStep):
    """The oracle's ElasticPerturbation3D (CPU FP64): the static problem under
    lateral moduli perturbations on the GLL nodes of the solid elements."""

    def __init__(self, layers, lmax, ngll=5, eps=1e-8, oversampling=1.5):
        self.L = load()
        _v3d_sigs(self.L)
        self.options = default_options(lmax, ngll)
        self.h = self.L.oracle_ep3d_create(layers, len(layers), _ct.byref(EpOptions(lmax, ngll, eps, oversampling)))
        self.P = self.L.oracle_v3d_node_count(self.h)
        nt, nph = _ct.c_int(), _ct.c_int()
        self.L.oracle_v3d_grid(self.h, _ct.byref(nt), _ct.byref(nph), None, None)
        self.ntheta, self.nphi = nt.value, nph.value
        self.theta = np.empty(self.ntheta)
        self.weights = np.empty(self.ntheta)
        self.L.oracle_v3d_grid(self.h, None, None, ptr(self.theta), ptr(self.weights))
        self.radius = np.empty(self.P)
        self.element = np.empty(self.P, dtype=np.int32)
        self.L.oracle_v3d_nodes(self.h, ptr(self.radius), ptr(self.element))
        self.sigma_scale = self.L.oracle_v3d_surface_density_scale(self.h)
        self.modulus_scale = self.L.oracle_v3d_modulus_scale(self.h)
        self.state = self.L.oracle_v3d_zero_state(self.h)
        self._keep = []

    def set_moduli(self, d_mu=None, d_kappa=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (d_mu, d_kappa)]
        self._keep = arrs
        self.L.oracle_ep3d_set_moduli(self.h, *(None if a is None else a.ctypes.data for a in arrs))

    def solve_load(self, load):
        load = np.ascontiguousarray(load, dtype=np.complex128)
        self.L.oracle_ep3d_solve_load(self.h, load.ctypes.data)

    def respond(self):
        self.L.oracle_ep3d_respond(self.h)

    def solve_lateral(self, load, rtol=1e-10, max_iterations=200):
        load = np.ascontiguousarray(load, dtype=np.complex128)
        info = StepInfo()
        self.L.oracle_ep3d_solve_lateral(self.h, load.ctypes.data, rtol, max_iterations, _ct.byref(info))
        return info
