"""ElasticPerturbation3D: the static problem under lateral moduli
perturbations (src/ElasticPerturbation3D.cpp), in the oracle and on the GPU.

The reference's gates re-expressed (tests/TestElasticPerturbation3D.cpp):
  - an angle-uniform 10% shift of mu and kappa solved laterally equals the
    plain solve on the shifted material (:440-492, 1e-9);
  - the lateral solve departs from reference + Born response at second
    order: halving the contrast quarters the departure (:353-438, 4 +- 0.3).
The GPU path follows the oracle: SolveLoad, Respond (deviatoric and
dilatation parts) and SolveLateral residual for residual, 1e-10."""

import numpy as np
import pytest

from tests import _oracle as O
from tests.test_step import rel

TOL = 1e-10
ELEMENTS = 16


def _layers(shift=0.0, product=False):
    if product:
        from sl3dpp_gb300.viscoelastic3d import standard_earth

        layers = standard_earth(ELEMENTS)
    else:
        layers = O.standard_earth(ELEMENTS)
    for layer in layers:
        if not layer.fluid:
            layer.mu0 *= 1.0 + shift
            layer.mu1 *= 1.0 + shift
            layer.kappa0 *= 1.0 + shift
            layer.kappa1 *= 1.0 + shift
    return layers


def _nodal(o, field):
    """A layer field (mu or kappa, SI) at every node, in the model's modulus unit."""
    layers = _layers()
    length = 6371e3
    out = np.empty(o.P)
    for p in range(o.P):
        e = o.element[p]
        mid = 0.5 * (o.radius[o.element == e].min() + o.radius[o.element == e].max()) * length
        r = o.radius[p] * length
        for layer in layers:
            if layer.r0 <= mid <= layer.r1:
                v0, v1 = getattr(layer, field + "0"), getattr(layer, field + "1")
                out[p] = v0 + (v1 - v0) * (r - layer.r0) / (layer.r1 - layer.r0)
                break
    return out / o.modulus_scale


def _load(lmax, scale):
    load = np.zeros((lmax + 1) * (lmax + 2) // 2, dtype=np.complex128)
    for l in range(lmax + 1):
        for m in range(l + 1):
            load[l * (l + 1) // 2 + m] = complex(1.0 / (1.0 + l), 0.0 if m == 0 else 0.3 * m)
    return load * scale


def _lateral(o, radial, angular):
    """radial(r) x angular(theta, phi) on every grid value."""
    phi = 2.0 * np.pi * np.arange(o.nphi) / o.nphi
    ang = angular(o.theta[:, None], phi[None, :])
    return np.ascontiguousarray((radial[:, None, None] * ang[None, :, :]).reshape(-1))


def test_oracle_angle_uniform_solve_matches_the_shifted_material():
    lmax = 6
    born = O.OraclePerturbation(_layers(), lmax)
    exact = O.OraclePerturbation(_layers(0.1), lmax)
    uniform = lambda t, p: np.ones(np.broadcast(t, p).shape)
    d_mu = _lateral(born, 0.1 * _nodal(born, "mu"), uniform)
    d_kappa = _lateral(born, 0.1 * _nodal(born, "kappa"), uniform)
    born.set_moduli(d_mu, d_kappa)
    load = _load(lmax, 1.0 / born.sigma_scale * 1e3)
    info = born.solve_lateral(load, rtol=1e-13)
    assert info.converged == 1 and info.solve_iterations > 0
    exact.solve_load(load)
    for comp in (0, 1, 2):
        assert rel(born.surface(comp), exact.surface(comp)) < 1e-9, comp


def _born_departure(o, load, d_mu, d_kappa, factor):
    o.set_moduli(d_mu * factor, d_kappa * factor)
    o.solve_load(load)
    u0 = [o.surface(c) for c in (0, 2)]
    o.respond()
    du = [o.surface(c) for c in (0, 2)]
    info = o.solve_lateral(load, rtol=1e-13)
    assert info.converged == 1 and info.solve_iterations < 40
    u = [o.surface(c) for c in (0, 2)]
    departure = max(np.max(np.abs(u[i] - u0[i] - du[i])) for i in range(2))
    first = max(np.max(np.abs(du[i])) for i in range(2))
    return departure, first


def test_oracle_lateral_solve_is_born_to_first_order():
    lmax = 6
    o = O.OraclePerturbation(_layers(), lmax)
    mu = _nodal(o, "mu")
    r = o.radius
    d_mu = _lateral(o, 0.1 * mu.max() * (0.5 + r * r),
                    lambda t, p: np.sin(t) * np.cos(t) * np.cos(p) + 0.3 * np.cos(2 * p) * np.sin(t) ** 2)
    d_kappa = _lateral(o, 0.1 * mu.max() * (1.0 - 0.5 * r), lambda t, p: np.cos(t) + 0 * p)
    load = np.zeros((lmax + 1) * (lmax + 2) // 2, dtype=np.complex128)
    load[2 * 3 // 2 + 0] = 1.0
    load[3 * 4 // 2 + 1] = 0.5 + 0.25j
    load *= 1e3 / o.sigma_scale
    s1, f1 = _born_departure(o, load, d_mu, d_kappa, 1.0)
    s2, f2 = _born_departure(o, load, d_mu, d_kappa, 0.5)
    assert s1 < 0.2 * f1
    assert abs(s1 / s2 - 4.0) < 0.3, s1 / s2


@pytest.mark.gpu
def test_gpu_static_perturbation_matches_the_oracle(gpu):
    from sl3dpp_gb300.elastic_perturbation3d import ElasticPerturbation3D

    lmax = 8
    o = O.OraclePerturbation(_layers(), lmax)
    g = ElasticPerturbation3D(_layers(product=True), lmax)
    assert (g.node_count, g.ntheta, g.nphi) == (o.P, o.ntheta, o.nphi)
    assert np.max(np.abs(g.radius - o.radius)) < 1e-14  # separate setups, the same nodes to rounding
    mu = _nodal(o, "mu")
    r = o.radius
    d_mu = _lateral(o, 0.1 * mu.max() * (0.5 + r * r),
                    lambda t, p: np.sin(t) * np.cos(t) * np.cos(p) + 0.3 * np.cos(2 * p) * np.sin(t) ** 2)
    d_kappa = _lateral(o, 0.1 * mu.max() * (1.0 - 0.5 * r), lambda t, p: np.cos(t) * np.sin(p) + 0.2)
    load = _load(lmax, 1e3 / o.sigma_scale)
    for mu_dir, kappa_dir in ((d_mu, None), (None, d_kappa), (d_mu, d_kappa)):
        o.set_moduli(mu_dir, kappa_dir)
        g.set_moduli(mu_dir, kappa_dir)
        o.solve_load(load)
        g.SolveLoad(load)
        for comp in (0, 1, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < TOL
        o.respond()
        g.Respond()
        for comp in (0, 1, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < 1e-9, (comp, mu_dir is None, kappa_dir is None)
        io = o.solve_lateral(load, rtol=1e-12)
        ig = g.SolveLateral(load, rtol=1e-12)
        assert ig.converged == io.converged == 1
        assert ig.solve_iterations == io.solve_iterations
        ho, hg = o.residual_history(), g.residual_history()
        assert ho.size == hg.size
        big = ho > 1e-9
        assert np.max(np.abs(hg[big] - ho[big]) / ho[big]) < 1e-6
        for comp in (0, 1, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < TOL


@pytest.mark.gpu
def test_gpu_force_and_apply_are_the_solves_operators(gpu):
    """Force and Apply through the C ABI (ElasticPerturbation3D.hpp:98-130)
    agree with the solves: SolveLoad's solution x has K_ref x = LoadForces,
    so Apply(x) - Force(x) is the load's forces; SolveLateral's solution
    satisfies Apply(x) = LoadForces to its tolerance; Force is linear and
    vanishes without directions."""
    import torch

    from sl3dpp_gb300.elastic_perturbation3d import ElasticPerturbation3D

    lmax = 8
    o = O.OraclePerturbation(_layers(), lmax)
    g = ElasticPerturbation3D(_layers(product=True), lmax)
    mu = _nodal(o, "mu")
    r = o.radius
    d_mu = _lateral(o, 0.1 * mu.max() * (0.5 + r * r),
                    lambda t, p: np.sin(t) * np.cos(t) * np.cos(p) + 0.3 * np.cos(2 * p) * np.sin(t) ** 2)
    load = _load(lmax, 1e3 / o.sigma_scale)
    g.set_moduli(d_mu, None)
    g.SolveLoad(load)
    x = g.Solution()
    f = g.LoadForces(load)
    scale = torch.max(torch.abs(f)).item()
    assert (torch.max(torch.abs(g.Apply(x) - g.Force(x) - f)) / scale).item() < 1e-10
    assert (torch.max(torch.abs(g.Force(2.0 * x) - 2.0 * g.Force(x))) / scale).item() < 1e-13
    g.SolveLateral(load, rtol=1e-12)
    y = g.Solution()
    assert (torch.max(torch.abs(g.Apply(y) - f)) / scale).item() < 1e-9
    g.set_moduli(None, None)
    assert torch.max(torch.abs(g.Force(y))).item() == 0.0
