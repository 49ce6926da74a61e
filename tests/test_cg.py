"""The step closed by preconditioned conjugate gradients (Options::solver =
ConjugateGradients; Viscoelastic3D.cpp:2008-2015, detail/LateralSolve.hpp:
112-181).

The reference's gate re-expressed (tests/TestViscoelastic3D.cpp:664-726): at
a 10x contrast, delta = 0.5 ln 10 sin(theta) cos(phi), over two exponential
trapezoid steps of about two relaxation times, the conjugate-gradient step
lands where the fixed point does (1e-9) with no mixed passes. The GPU path
follows the oracle's conjugate gradients residual for residual."""

import numpy as np
import pytest

from tests import _oracle as O
from tests.test_step import cap_load, rel
from sl3dpp_gb300 import configs

TOL = 1e-10


def _contrast(o):
    """0.5 ln 10 sin(theta) cos(phi) at every memory node (a 10x contrast)."""
    amp = 0.5 * np.log(10.0)
    phi = 2.0 * np.pi * np.arange(o.nphi) / o.nphi
    pattern = amp * np.sin(o.theta)[:, None] * np.cos(phi)[None, :]
    return np.ascontiguousarray(np.broadcast_to(pattern, (o.P, o.ntheta, o.nphi)).reshape(-1))


def _oracle(lmax, solver, **kw):
    o = O.OracleStep(O.standard_earth(20), O.default_options(lmax, 5, solver=solver, rtol=1e-12, solve_rtol=1e-12,
                                                              max_iterations=200, **kw))
    o.set_delta(_contrast(o))
    return o


def _run(op, steps, dt, load, step):
    infos = []
    for n in range(steps):
        infos.append(step(op, dt, 0, load * n / 2, load * (n + 1) / 2))
    return infos


def test_oracle_conjugate_gradients_step_matches_the_fixed_point():
    lmax = 8
    fixed, cg = _oracle(lmax, 0), _oracle(lmax, 1)
    load = cap_load(lmax, fixed.sigma_scale, 2000.0)
    dt = 300 * configs.SECONDS_PER_YEAR / fixed.time_scale
    for n in range(2):
        i_f = fixed.step(dt, 0, load * n / 2, load * (n + 1) / 2)
        i_c = cg.step(dt, 0, load * n / 2, load * (n + 1) / 2)
        assert i_f.converged == 1 and i_c.converged == 1
        assert i_c.mixed_passes == 0 and i_c.solve_iterations == i_c.iterations > 0
        assert i_c.solve_iterations < i_f.iterations  # fewer iterations than passes
        for comp in (0, 2):
            assert rel(cg.surface(comp), fixed.surface(comp)) < 1e-9, (n, comp)
    h = cg.residual_history()
    assert h[-1] <= 1e-12 and h[0] > h[-1]


def test_oracle_conjugate_gradients_without_contrast_converge_at_once():
    lmax = 6
    o = O.OracleStep(O.standard_earth(20), O.default_options(lmax, 5, solver=1))
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    info = o.step(dt, 2, 0 * load, load)
    assert info.converged == 1 and info.solve_iterations == 0


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [0, 2])
def test_gpu_conjugate_gradients_match_the_oracle(gpu, scheme):
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    lmax = 8
    o = _oracle(lmax, 1)
    g = Viscoelastic3D(standard_earth(20), Options.defaults(lmax, 5, solver=1, rtol=1e-12, solve_rtol=1e-12,
                                                           max_iterations=200))
    g.set_delta(_contrast(o))
    state = g.ZeroState()
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 300 * configs.SECONDS_PER_YEAR / o.time_scale
    for n in range(2):
        io = o.step(dt, scheme, load * n / 2, load * (n + 1) / 2)
        ig = g.Step(state, dt, scheme, load * n / 2, load * (n + 1) / 2)
        assert ig.converged == io.converged == 1
        assert ig.solve_iterations == io.solve_iterations
        ho, hg = o.residual_history(), g.residual_history()
        assert ho.size == hg.size
        big = ho > 1e-9
        assert np.max(np.abs(hg[big] - ho[big]) / ho[big]) < 1e-6
        for comp in (0, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < TOL, (n, comp)
    want = np.zeros(g.spectral_size, dtype=np.complex128)
    o.L.oracle_v3d_state_strain(o.state, want.ctypes.data)
    assert rel(state.strain_coefficients(), want) < TOL


@pytest.mark.gpu
def test_gpu_conjugate_gradients_match_the_gpu_fixed_point(gpu):
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    lmax = 12
    results = {}
    for solver in (0, 1):
        g = Viscoelastic3D(standard_earth(24), Options.defaults(lmax, 5, solver=solver, rtol=1e-12, solve_rtol=1e-12,
                                                               max_iterations=200))
        d = np.zeros(g.node_count * g.ntheta * g.nphi)
        amp = 0.5 * np.log(10.0)
        phi = 2.0 * np.pi * np.arange(g.nphi) / g.nphi
        d[:] = np.broadcast_to(amp * np.sin(g.theta)[:, None] * np.cos(phi)[None, :],
                               (g.node_count, g.ntheta, g.nphi)).reshape(-1)
        g.set_delta(d)
        state = g.ZeroState()
        exact_theta, w, nphi = O.grid(lmax, 1.0)
        cap = configs.cap_field(exact_theta, nphi, 15.0, 2000.0)
        load = O.expand_real(lmax, exact_theta, w, nphi, cap) / g.surface_density_scale
        dt = 300 * configs.SECONDS_PER_YEAR / g.time_scale
        iters = []
        for n in range(2):
            info = g.Step(state, dt, 0, load * n / 2, load * (n + 1) / 2)
            assert info.converged == 1
            iters.append(info.iterations)
        results[solver] = (g.Surface(0), g.Surface(2), iters)
    for comp in (0, 1):
        assert rel(results[1][comp], results[0][comp]) < 1e-9
    assert results[1][2][-1] < results[0][2][-1]
