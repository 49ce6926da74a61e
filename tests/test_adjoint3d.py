"""The discrete adjoint of the 3D run without an ocean (AdjointSolver3D::
FirstOrderKernels under AdjointMethod::Discrete, include/sl3dpp/
Adjoint3D.hpp:241-322, src/AdjointDiscrete3D.cpp), checked as the
reference's own gates check it (tests/TestDiscreteAdjoint3D.cpp): the
pairing identity and the gradient against differences of the forward run.

With delta fixed the run is linear in its loads, so the load kernels must
pair with any loads to the objective of the forward run under them:
sum_n <kernel_n, L_n> = J(L) = sum_n <g_n, U_n(L)> + <h_n, phi_n(L)> -- against
the library's forward run and against the oracle's march of the same nodes
(1e-8: both runs and the transposed solves converge to rtol 1e-11). The
log-viscosity gradient must give the derivative of J along a direction p
over every node (the sweep forms it at nodes outside delta's range too):
Richardson-extrapolated central differences of the forward run, 1e-6. Each
for the three schemes, and the mixed form for Sdirk2. A record stride (the
forward states kept every stride-th node, the gaps rebuilt) changes nothing
but the memory held. The tangent-linear run (TangentLinearSolver3D's
discrete method) pairs with the adjoint to 1e-8 along a direction in the
log-viscosity and the loads together. On the CPU, the oracle's own
restatement of the transposed sweep (oracle_step.cpp, AdjointRun) meets the
pairing identity with the oracle's run (1e-12), its tide kernels a run under
tides (1e-12), its gradient the differences of that run (1e-6) and the
oracle's tangent-linear run (1e-10)."""

import numpy as np
import pytest

from sl3dpp_gb300 import configs
from tests import _oracle as O
from tests.test_step import _pair, cap_load, rel


def real_coefficients(lmax, rng, count):
    """Random coefficients (l, m >= 0) of real fields: m = 0 parts real."""
    lm = (lmax + 1) * (lmax + 2) // 2
    c = rng.standard_normal((count, lm)) + 1j * rng.standard_normal((count, lm))
    for l in range(lmax + 1):
        c[:, l * (l + 1) // 2] = c[:, l * (l + 1) // 2].real
    return c


def pairing(lmax, a, b):
    """sum over (l, m >= 0) of w_m Re(a conj b), w_m = 1 at m = 0 and 2 above."""
    w = np.concatenate([[1.0] + [2.0] * l for l in range(lmax + 1)])
    return float(np.sum(w * (a * np.conj(b)).real))


def _run(lmax, scheme, nodes, precision=0, seed=3):
    o, g = _pair(lmax, 20, 5, rms=0.8, rtol=1e-11, max_iterations=120, precision=precision)
    rng = np.random.default_rng(seed)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    times = dt * np.arange(nodes)
    full = cap_load(lmax, o.sigma_scale, 2000.0)
    loads = np.stack([full * (k + 1) / nodes for k in range(nodes)]) + 0.05 * np.max(np.abs(full)) * \
        real_coefficients(lmax, rng, nodes)
    gU = real_coefficients(lmax, rng, nodes)
    gPhi = real_coefficients(lmax, rng, nodes)
    return o, g, times, loads, gU, gPhi


def _objective(lmax, out, gU, gPhi):
    return sum(pairing(lmax, gU[k], out["U"][k]) + pairing(lmax, gPhi[k], out["phi"][k])
               for k in range(len(gU)))


CASES = [(2, 0), (0, 0), (1, 0), (2, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,precision", CASES)
def test_gpu_load_kernels_pair_with_the_forward_run(gpu, scheme, precision):
    from sl3dpp_gb300.viscoelastic3d import Evolution3D

    lmax, nodes = 8, 4
    o, g, times, loads, gU, gPhi = _run(lmax, scheme, nodes, precision)
    adj = Evolution3D(g, scheme).Adjoint(times, loads, gU, gPhi, gradient=False)
    assert all(i.converged for i in adj["infos"])
    paired = sum(pairing(lmax, adj["load_kernels"][k], loads[k]) for k in range(nodes))
    forward = Evolution3D(g, scheme).Run(times, loads)
    J = _objective(lmax, forward, gU, gPhi)
    assert abs(adj["objective"] - J) < 1e-10 * abs(J)
    assert abs(paired - J) < 1e-8 * abs(J), (paired, J)
    # the oracle's march of the same nodes
    U, phi = [], []
    for k in range(nodes):
        step_dt = 0.0 if k == 0 else times[k] - times[k - 1]
        assert o.step(step_dt, scheme, loads[max(k - 1, 0)], loads[k]).converged
        U.append(o.surface(0))
        phi.append(o.surface(2))
    Jo = _objective(lmax, {"U": U, "phi": phi}, gU, gPhi)
    assert abs(paired - Jo) < 1e-8 * abs(Jo), (paired, Jo)
    # one node's kernel alone: the response at the last node to a load at node 1
    one = np.zeros_like(loads)
    one[1] = loads[1]
    single = Evolution3D(g, scheme).Run(times, one)
    assert abs(pairing(lmax, adj["load_kernels"][1], loads[1]) - _objective(lmax, single, gU, gPhi)) < \
        1e-8 * abs(J)


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,precision", CASES)
def test_gpu_delta_gradient_matches_differences_of_the_run(gpu, scheme, precision):
    from sl3dpp_gb300.viscoelastic3d import Evolution3D

    lmax, nodes = 8, 4
    o, g, times, loads, gU, gPhi = _run(lmax, scheme, nodes, precision, seed=5)
    delta = np.asarray(_delta(o, lmax))
    adj = Evolution3D(g, scheme).Adjoint(times, loads, gU, gPhi)
    grad = adj["delta_gradient"]
    assert grad.shape == (g.values,)
    # a smooth direction over every node, delta's range and beyond
    rng = np.random.default_rng(17)
    pattern = O.synthesise_real(lmax, o.theta, o.nphi, real_coefficients(lmax, rng, 1)[0] / (lmax + 1))
    radial = 1.0 + 0.5 * np.sin(7.0 * np.asarray(o.radius))
    p = (radial[:, None] * np.asarray(pattern).ravel()[None, :]).ravel()
    predicted = float(grad @ p)

    def J(h):
        g.set_delta(delta + h * p)
        return _objective(lmax, Evolution3D(g, scheme).Run(times, loads), gU, gPhi)

    h = 1e-2
    d1 = (J(h) - J(-h)) / (2 * h)
    d2 = (J(h / 2) - J(-h / 2)) / h
    richardson = (4 * d2 - d1) / 3
    g.set_delta(delta)
    assert abs(predicted - richardson) < 1e-6 * abs(richardson), (predicted, richardson, d1, d2)
    # nodes outside delta's range carry gradient too
    outside = np.ones(g.node_count, dtype=bool)
    per_node = delta.reshape(g.node_count, -1)
    outside[np.any(per_node != 0.0, axis=1)] = False
    assert outside.any()
    assert np.max(np.abs(grad.reshape(g.node_count, -1)[outside])) > 0.0


def _delta(o, lmax):
    from tests.test_step import delta_for

    return delta_for(o, lmax, 4, 0.8, 11)



@pytest.mark.gpu
@pytest.mark.parametrize("stride", [2, 3])
def test_gpu_record_stride_gives_the_kernels_of_every_node_kept(gpu, stride):
    """ForwardTrajectory3D's stride: the sweep rebuilds a gap's states by the
    run's own steps from the kept state below; the kernels are those of the
    run with every node kept (1e-9: the rebuilt steps converge afresh)."""
    from sl3dpp_gb300.viscoelastic3d import Evolution3D

    lmax, nodes = 8, 7
    o, g, times, loads, gU, gPhi = _run(lmax, 2, nodes, 0, seed=9)
    every = Evolution3D(g, 2).Adjoint(times, loads, gU, gPhi)
    sparse = Evolution3D(g, 2).Adjoint(times, loads, gU, gPhi, stride=stride)
    assert abs(sparse["objective"] - every["objective"]) < 1e-12 * abs(every["objective"])
    assert rel(sparse["load_kernels"], every["load_kernels"]) < 1e-9
    assert rel(sparse["delta_gradient"], every["delta_gradient"]) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,precision", CASES)
def test_gpu_adjoint_pairs_with_the_tangent_linear_run(gpu, scheme, precision):
    """The reference's tight gate (TestDiscreteAdjoint3D): the adjoint's
    gradient and load kernels paired with a direction -- in the log-viscosity
    over every node and in the loads, together -- equal the objective's
    derivative from the tangent-linear run along it (1e-8); along loads
    alone the tangent run is the forward run under them."""
    from sl3dpp_gb300.viscoelastic3d import Evolution3D

    lmax, nodes = 8, 4
    o, g, times, loads, gU, gPhi = _run(lmax, scheme, nodes, precision, seed=21)
    ev = Evolution3D(g, scheme)
    adj = ev.Adjoint(times, loads, gU, gPhi)
    rng = np.random.default_rng(23)
    pattern = O.synthesise_real(lmax, o.theta, o.nphi, real_coefficients(lmax, rng, 1)[0] / (lmax + 1))
    radial = 1.0 + 0.5 * np.cos(5.0 * np.asarray(o.radius))
    p = (radial[:, None] * np.asarray(pattern).ravel()[None, :]).ravel()
    dL = 0.1 * np.max(np.abs(loads)) * real_coefficients(lmax, rng, nodes)
    tl = ev.Tangent(times, loads, p, dL)
    assert all(i.converged for i in tl["infos"])
    lhs = _objective(lmax, tl, gU, gPhi)
    rhs = float(adj["delta_gradient"] @ p) + sum(pairing(lmax, adj["load_kernels"][k], dL[k]) for k in range(nodes))
    assert abs(lhs - rhs) < 1e-8 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    # along loads alone: the forward run under them
    alone = ev.Tangent(times, loads, None, dL)
    run = ev.Run(times, dL)
    assert rel(alone["U"], run["U"]) < 1e-9 and rel(alone["phi"], run["phi"]) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [2, 0])
def test_gpu_tide_kernels_pair_with_a_tide_run(gpu, scheme):
    """Kernels::tideKernels: the run is linear in a tide added to its tide
    channel, so the tide kernels pair with any tides (no degree-1 part) to
    the objective of the run under those tides alone (1e-8)."""
    from sl3dpp_gb300.viscoelastic3d import Evolution3D

    lmax, nodes = 8, 4
    o, g, times, loads, gU, gPhi = _run(lmax, scheme, nodes, 0, seed=31)
    adj = Evolution3D(g, scheme).Adjoint(times, loads, gU, gPhi, gradient=False)
    tides = 1e-3 * real_coefficients(lmax, np.random.default_rng(33), nodes)
    tides[:, 1:3] = 0.0  # no degree-1 tide
    zero = np.zeros_like(tides[0])
    state = g.ZeroState()
    U, phi = [], []
    for k in range(nodes):
        dt = 0.0 if k == 0 else times[k] - times[k - 1]
        assert g.Step(state, dt, scheme, zero, zero, tides[max(k - 1, 0)], tides[k]).converged
        U.append(g.Surface("U"))
        phi.append(g.Surface("phi"))
    J = _objective(lmax, {"U": U, "phi": phi}, gU, gPhi)
    paired = sum(pairing(lmax, adj["tide_kernels"][k], tides[k]) for k in range(nodes))
    assert abs(paired - J) < 1e-8 * abs(J), (paired, J)
    assert np.all(adj["tide_kernels"][:, 1:3] == 0.0)


# -- the oracle's restatement (CPU) ---------------------------------------------------------------

def _oracle_case(lmax=6, nodes=4, seed=3):
    def make():
        o = O.OracleStep(O.standard_earth(20, 0.0, 10.0), O.default_options(lmax, 5, rtol=1e-11, max_iterations=80))
        o.set_delta(_delta_of(o, lmax))
        return o

    o = make()
    rng = np.random.default_rng(seed)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    times = dt * np.arange(nodes)
    full = cap_load(lmax, o.sigma_scale, 2000.0, alpha=40.0)
    loads = np.stack([full * (k + 1) / nodes for k in range(nodes)]) + 0.05 * np.max(np.abs(full)) * \
        real_coefficients(lmax, rng, nodes)
    return make, times, loads, real_coefficients(lmax, rng, nodes), real_coefficients(lmax, rng, nodes)


def _delta_of(o, lmax):
    from tests.test_step import delta_for

    return delta_for(o, lmax, 3, 0.8, 11)


def _oracle_objective(make, lmax, scheme, times, loads, gU, gPhi, delta=None):
    o = make()
    if delta is not None:
        o.set_delta(delta)
    J = 0.0
    for k in range(len(times)):
        dt = 0.0 if k == 0 else times[k] - times[k - 1]
        assert o.step(dt, scheme, loads[max(k - 1, 0)], loads[k]).converged
        J += pairing(o.options.lmax, gU[k], o.surface(0)) + pairing(o.options.lmax, gPhi[k], o.surface(2))
    return J


@pytest.mark.parametrize("scheme", [2, 0, 1])
def test_oracle_adjoint_pairs_with_the_oracle_run(scheme):
    """The oracle's own transpose of its step (the restatement the GPU sweep
    is compared with): its load kernels pair with the loads to its forward
    run's objective (1e-12)."""
    lmax = 6
    make, times, loads, gU, gPhi = _oracle_case(lmax)
    adj = make().adjoint(times, scheme, loads, gU, gPhi)
    J = _oracle_objective(make, lmax, scheme, times, loads, gU, gPhi)
    paired = sum(pairing(lmax, adj["load_kernels"][k], loads[k]) for k in range(len(times)))
    assert abs(adj["objective"] - J) < 1e-13 * abs(J)
    assert abs(paired - J) < 1e-12 * abs(J), (paired, J)


def test_oracle_delta_gradient_matches_differences():
    """The oracle's gradient in delta along a direction over every node
    against Richardson-extrapolated central differences of its run (1e-6)."""
    lmax, scheme = 6, 2
    make, times, loads, gU, gPhi = _oracle_case(lmax, seed=5)
    o = make()
    delta = np.asarray(_delta_of(o, lmax))
    adj = o.adjoint(times, scheme, loads, gU, gPhi)
    rng = np.random.default_rng(17)
    pattern = O.synthesise_real(lmax, o.theta, o.nphi, real_coefficients(lmax, rng, 1)[0] / (lmax + 1))
    radial = 1.0 + 0.5 * np.sin(7.0 * np.asarray(o.radius))
    p = (radial[:, None] * np.asarray(pattern).ravel()[None, :]).ravel()
    J = lambda h: _oracle_objective(make, lmax, scheme, times, loads, gU, gPhi, delta + h * p)
    h = 1e-2
    d1 = (J(h) - J(-h)) / (2 * h)
    d2 = (J(h / 2) - J(-h / 2)) / h
    richardson = (4 * d2 - d1) / 3
    predicted = float(adj["delta_gradient"] @ p)
    assert abs(predicted - richardson) < 1e-6 * abs(richardson), (predicted, richardson)



@pytest.mark.parametrize("scheme", [2, 0])
def test_oracle_tangent_pairs_with_the_oracle_adjoint(scheme):
    """The oracle's tangent-linear run against its adjoint along a direction
    in the log-viscosity over every node and in the loads (1e-10)."""
    lmax = 6
    make, times, loads, gU, gPhi = _oracle_case(lmax, seed=7)
    adj = make().adjoint(times, scheme, loads, gU, gPhi)
    o = make()
    rng = np.random.default_rng(29)
    pattern = O.synthesise_real(lmax, o.theta, o.nphi, real_coefficients(lmax, rng, 1)[0] / (lmax + 1))
    radial = 1.0 + 0.5 * np.cos(5.0 * np.asarray(o.radius))
    p = (radial[:, None] * np.asarray(pattern).ravel()[None, :]).ravel()
    dL = 0.1 * np.max(np.abs(loads)) * real_coefficients(lmax, rng, len(times))
    tl = o.tangent(times, scheme, loads, p, dL)
    lhs = _objective(lmax, tl, gU, gPhi)
    rhs = float(adj["delta_gradient"] @ p) + sum(pairing(lmax, adj["load_kernels"][k], dL[k])
                                                 for k in range(len(times)))
    assert abs(lhs - rhs) < 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_oracle_tide_kernels_pair_with_a_tide_run():
    """The oracle's tide kernels pair with tides (no degree-1 part) to its
    run under those tides alone (1e-12)."""
    lmax, scheme = 6, 2
    make, times, loads, gU, gPhi = _oracle_case(lmax, seed=9)
    adj = make().adjoint(times, scheme, loads, gU, gPhi)
    tides = 1e-3 * real_coefficients(lmax, np.random.default_rng(33), len(times))
    tides[:, 1:3] = 0.0
    zero = np.zeros_like(tides[0])
    o = make()
    J = 0.0
    for k in range(len(times)):
        dt = 0.0 if k == 0 else times[k] - times[k - 1]
        assert o.step(dt, scheme, zero, zero, tides[max(k - 1, 0)], tides[k]).converged
        J += pairing(lmax, gU[k], o.surface(0)) + pairing(lmax, gPhi[k], o.surface(2))
    paired = sum(pairing(lmax, adj["tide_kernels"][k], tides[k]) for k in range(len(times)))
    assert abs(paired - J) < 1e-12 * abs(J), (paired, J)
