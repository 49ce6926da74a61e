"""The degree systems: the library assembles every degree's band on the GPU
(one thread per stored entry); the oracle assembles each on the CPU from
element matrices F^T M F. The two are separate code written from the same
weak form (reference src/DegreeOperator.cpp:253-474, src/ToroidalOperator.cpp),
so they must agree to rounding at every degree of the measured
configurations' meshes: 1e-13 of the band's largest entry."""

import numpy as np
import pytest

from tests import _oracle as O

TOL = 1e-13
SECONDS_PER_YEAR = 3.15576e7


def rel_band(got, want):
    return np.max(np.abs(got - want)) / np.max(np.abs(want))


# -- the oracle's assembly on its own ----------------------------------------------------------

def test_oracle_bands_are_definite_where_the_reference_factorises_by_cholesky():
    """The toroidal systems and the solid degrees >= 2 are positive definite
    (Cholesky succeeds on the scaled band), as DegreeOperator::Factorise
    expects; the layouts have the reference's sizes (3 unknowns a solid node,
    phi alone in the fluid core, the centre's U and degree 1's surface phi
    removed)."""
    layers = O.standard_earth(20)
    o = O.load()
    for l, tor in [(2, False), (5, False), (1, True), (6, True)]:
        band = O.degree_band(layers, 5, l, toroidal=tor)
        n, ld = band.shape
        d = band[:, -1]
        assert np.all(d > 0)
        s = 1.0 / np.sqrt(d)
        scaled = band.copy()
        for j in range(n):
            for t in range(ld):
                i = j - (ld - 1) + t
                if i >= 0:
                    scaled[j, t] *= s[i] * s[j]
        if tor and l == 1:
            continue  # the rigid rotation: singular until its gauge row is pinned
        assert o.oracle_band_cholesky_factor(O.ptr(np.ascontiguousarray(scaled.reshape(-1))), n, ld - 1) == 0
    # 20 elements of order 4; below the core-mantle boundary node the core's
    # nodes carry phi alone for l > 0
    nodes = 20 * 4 + 1
    fluid = layers[0].elements * 4
    assert O.degree_band(layers, 5, 2).shape[0] == 3 * (nodes - fluid) + fluid
    assert O.degree_band(layers, 5, 1).shape[0] == 3 * (nodes - fluid) + fluid - 1
    assert O.degree_band(layers, 5, 0).shape[0] == 2 * nodes - 1


def test_oracle_band_softens_as_the_step_relaxes():
    """A longer step leaves less of the branches' shear unrelaxed: every
    diagonal entry falls (or stays, where nothing relaxes) from the elastic
    flavour towards the long-term material's."""
    layers = O.standard_earth(20)
    tau = 3e7  # about the lower mantle's Maxwell time in model units
    d = [O.degree_band(layers, 5, 4, dt=t)[:, -1] for t in (0.0, 0.1 * tau, tau, 100 * tau)]
    for a, b in zip(d, d[1:]):
        assert np.all(b <= a * (1 + 1e-15))
        assert np.any(b < a * (1 - 1e-6))


# -- the GPU's assembly against the oracle's ------------------------------------------------------

CONFIGS = [
    # (elements, ngll, lmax, kelvin fraction, step length in years)
    pytest.param(40, 5, 32, 0.0, 500.0, id="lmax32-40el-ngll5-maxwell"),
    pytest.param(80, 6, 128, 0.5, 250.0, id="lmax128-80el-ngll6-burgers"),
    pytest.param(120, 6, 256, 0.0, 500.0, id="lmax256-120el-ngll6-maxwell"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("elements,ngll,lmax,kelvin,years", CONFIGS)
def test_gpu_bands_match_the_oracle_at_every_degree(gpu, elements, ngll, lmax, kelvin, years):
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    layers = standard_earth(elements, kelvin)
    op = Viscoelastic3D(layers, Options.defaults(lmax, ngll))
    olayers = O.standard_earth(elements, kelvin)
    dt = years * SECONDS_PER_YEAR / op.time_scale
    worst = 0.0
    # the elastic flavour, a backward Euler flavour (Sdirk2's first stage) and
    # an exponential trapezoid one
    for scheme, length in [(1, 0.0), (1, 0.29289321881345247560 * dt), (0, dt)]:
        for tor in (False, True):
            for l in range(1 if tor else 0, lmax + 1):
                got = op.assembled_band(l, toroidal=tor, scheme=scheme, dt=length)
                want = O.degree_band(olayers, ngll, l, toroidal=tor, scheme=scheme, dt=length)
                assert got.shape == want.shape, (scheme, tor, l)
                err = rel_band(got, want)
                worst = max(worst, err)
                assert err < TOL, (scheme, length, tor, l, err)
    print(f"worst band difference {worst:.2e}")


@pytest.mark.gpu
def test_gpu_single_degree_band_matches_the_oracle_unrelaxed(gpu):
    """The one-degree drop-in (DegreeOperator on the unrelaxed material)."""
    from sl3dpp_gb300.degree import DegreeOperator
    from sl3dpp_gb300.viscoelastic3d import standard_earth

    layers = standard_earth(40)
    olayers = O.standard_earth(40)
    for l, tor in [(0, False), (1, False), (2, False), (17, False), (1, True), (9, True)]:
        got = DegreeOperator(layers, 5, l, toroidal=tor).Band()
        want = O.degree_band(olayers, 5, l, toroidal=tor, relaxed=False)
        assert rel_band(got, want) < TOL, (l, tor)
