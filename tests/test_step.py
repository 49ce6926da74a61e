"""The 3D quasi-static step: the oracle's physics checks on the CPU, and the GPU
step against the oracle on the same inputs (tolerance 1e-10 relative, the FP64
form's bar).

The reference's gates re-expressed here (tests/TestViscoelastic3D.cpp):
zero-lateral steps decouple the degrees and converge in two passes a stage
(:90-196); a lateral contrast couples orders and toroidal motion (:293-322);
both Prony bodies (Maxwell, Burgers); every scheme."""

import numpy as np
import pytest

from tests import _oracle as O
from sl3dpp_gb300 import configs

TOL = 1e-10


def cap_load(op_lmax, sigma_scale, thickness, alpha=15.0):
    theta, w, nphi = O.grid(op_lmax, 1.0)
    field = configs.cap_field(theta, nphi, alpha, thickness)
    return O.expand_real(op_lmax, theta, w, nphi, field) / sigma_scale


def delta_for(oracle_step, lmax, ldelta, rms, seed):
    c = configs.delta_coefficients(lmax, ldelta, rms, seed)
    pattern = O.synthesise_real(lmax, oracle_step.theta, oracle_step.nphi, c)
    return configs.delta_samples(pattern, oracle_step.radius)


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


# -- the oracle's physics ---------------------------------------------------------------------

def test_zero_lateral_step_decouples_and_converges_in_two_passes():
    lmax = 8
    st = O.OracleStep(O.standard_earth(20), O.default_options(lmax))
    load = cap_load(lmax, st.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / st.time_scale
    for n in range(2):
        info = st.step(dt, 2, load * n / 10, load * (n + 1) / 10)
        assert info.converged and info.iterations == 4  # two passes in each Sdirk2 stage
        U = st.surface(0)
        zonal = np.array([configs.real_index(l, 0) for l in range(lmax + 1)])
        rest = np.setdiff1d(np.arange(U.size), zonal)
        assert np.max(np.abs(U[rest])) < 1e-12 * np.max(np.abs(U[zonal]))
        assert U[configs.real_index(2, 0)].real < 0.0  # the load depresses the surface
        # no lateral contrast: no toroidal motion beyond the transforms' rounding
        assert np.max(np.abs(st.surface(3))) < 1e-12 * np.max(np.abs(U))
    # the degree-0 inertia moment is linear in the load's degree-0 part
    moment = st.L.oracle_v3d_inertia_moment(st.h)
    assert moment != 0.0
    st2 = O.OracleStep(O.standard_earth(20), O.default_options(lmax))
    for n in range(2):
        st2.step(dt, 2, 2 * load * n / 10, 2 * load * (n + 1) / 10)
    assert abs(st2.L.oracle_v3d_inertia_moment(st2.h) - 2 * moment) < 1e-12 * abs(moment)


def test_lateral_viscosity_couples_orders():
    lmax = 8
    st = O.OracleStep(O.standard_earth(20), O.default_options(lmax))
    st.set_delta(delta_for(st, lmax, 4, 0.5, seed=7))
    load = cap_load(lmax, st.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / st.time_scale
    for n in range(2):
        info = st.step(dt, 2, load * n / 10, load * (n + 1) / 10)
        assert info.converged and info.residual <= 1e-11
    U = st.surface(0)
    zonal = np.array([configs.real_index(l, 0) for l in range(lmax + 1)])
    rest = np.setdiff1d(np.arange(U.size), zonal)
    assert np.max(np.abs(U[rest])) > 1e-6 * np.max(np.abs(U[zonal]))


def tide_columns(lmax, scale=1e-4):
    """A degree-2 tide (orders 0 and 2) with a degree-0 centrifugal mean."""
    t = np.zeros((lmax + 1) * (lmax + 2) // 2, dtype=np.complex128)
    t[configs.real_index(0, 0)] = 0.3 * scale
    t[configs.real_index(2, 0)] = scale
    t[configs.real_index(2, 2)] = (0.5 - 0.25j) * scale
    return t


def test_tide_channel_is_degree_local_and_superposes_with_the_load():
    # zero lateral contrast: the tide moves only its own degrees and orders,
    # and a step under load and tide is the sum of the two steps apart
    # (AddUnitChannels adds both columns to the same right-hand side)
    lmax = 8
    dt = None
    out = []
    for use_load, use_tide in ((True, False), (False, True), (True, True)):
        st = O.OracleStep(O.standard_earth(20), O.default_options(lmax))
        load = cap_load(lmax, st.sigma_scale, 2000.0)
        tide = tide_columns(lmax)
        dt = 500 * configs.SECONDS_PER_YEAR / st.time_scale
        for n in range(2):
            info = st.step(dt, 2, load * n / 10 if use_load else None, load * (n + 1) / 10 if use_load else None,
                           tide * n if use_tide else None, tide * (n + 1) if use_tide else None)
            assert info.converged
        out.append(st.surface(0))
    U_load, U_tide, U_both = out
    touched = [configs.real_index(l, m) for l, m in ((0, 0), (2, 0), (2, 2))]
    rest = np.setdiff1d(np.arange(U_tide.size), touched)
    assert np.max(np.abs(U_tide[rest])) < 1e-14 * np.max(np.abs(U_tide))
    assert abs(U_tide[configs.real_index(2, 2)] / U_tide[configs.real_index(2, 0)] - (0.5 - 0.25j)) < 1e-12
    assert rel(U_both, U_load + U_tide) < 1e-12


# -- the GPU step against the oracle ------------------------------------------------------------

def _pair(lmax, elements, ngll, kelvin=0.0, rms=0.5, ldelta=4, seed=11, **opt):
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    layers_o = O.standard_earth(elements, kelvin, 10.0)
    o = O.OracleStep(layers_o, O.default_options(lmax, ngll, **opt))
    g = Viscoelastic3D(standard_earth(elements, kelvin, 10.0), Options.defaults(lmax, ngll, **opt))
    assert (g.node_count, g.ntheta, g.nphi) == (o.P, o.ntheta, o.nphi)
    assert np.max(np.abs(g.radius - o.radius)) < 1e-14  # separate setups, the same nodes to rounding
    assert np.max(np.abs(g.theta - o.theta)) < 1e-15
    if rms > 0:
        d = delta_for(o, lmax, ldelta, rms, seed)
        o.set_delta(d)
        g.set_delta(d)
    return o, g


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [2, 0, 1])
def test_gpu_step_matches_oracle(gpu, scheme):
    lmax = 8
    o, g = _pair(lmax, 20, 5)
    state = g.ZeroState()
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    for n in range(3):
        l0, l1 = load * n / 10, load * (n + 1) / 10
        io = o.step(dt, scheme, l0, l1)
        ig = g.Step(state, dt, scheme, l0, l1)
        assert ig.converged == io.converged == 1
        assert abs(ig.iterations - io.iterations) <= 1
        for comp in (0, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < TOL, (n, comp)
        # SurfaceToroidal: W from the lateral coupling alone, on U's scale
        W, Wo, U = g.SurfaceToroidal(), o.surface(3), o.surface(0)
        assert np.max(np.abs(Wo)) > 1e-8 * np.max(np.abs(U))
        assert np.max(np.abs(W - Wo)) < TOL * np.max(np.abs(U)), n
        assert abs(g.InertiaMoment() - o.L.oracle_v3d_inertia_moment(o.h)) <= TOL * abs(
            o.L.oracle_v3d_inertia_moment(o.h)), n
    want = np.zeros(g.spectral_size, dtype=np.complex128)
    o.L.oracle_v3d_state_strain(o.state, want.ctypes.data)
    assert rel(state.strain_coefficients(), want) < TOL


@pytest.mark.gpu
def test_gpu_step_matches_oracle_burgers_ngll6_lmax16(gpu):
    lmax = 16
    o, g = _pair(lmax, 24, 6, kelvin=0.5, rms=1.0, ldelta=6, seed=3)
    state = g.ZeroState()
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 250 * configs.SECONDS_PER_YEAR / o.time_scale
    for n in range(2):
        l0, l1 = load * n / 10, load * (n + 1) / 10
        io = o.step(dt, 2, l0, l1)
        ig = g.Step(state, dt, 2, l0, l1)
        assert ig.converged == io.converged == 1
        for comp in (0, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < TOL, (n, comp)


@pytest.mark.gpu
def test_gpu_step_with_anderson_from_the_first_pass(gpu):
    # anderson_rate 0: the mixer engages from the first pass (IterationControl);
    # the pass residuals follow the oracle's pass for pass
    lmax = 8
    o, g = _pair(lmax, 20, 5, rms=0.8, anderson_rate=0.0, max_iterations=60)
    state = g.ZeroState()
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    io = o.step(dt, 2, 0 * load, load)
    ig = g.Step(state, dt, 2, 0 * load, load)
    assert ig.mixed_passes > 0 and ig.mixed_passes == io.mixed_passes
    assert ig.iterations == io.iterations
    ho, hg = o.residual_history(), g.residual_history()
    assert ho.size == hg.size
    big = ho > 1e-8
    assert np.max(np.abs(hg[big] - ho[big]) / ho[big]) < 1e-6
    assert ig.converged == io.converged
    assert rel(g.Surface(0), o.surface(0)) < TOL


@pytest.mark.gpu
def test_gpu_residual_history_matches_oracle_at_high_contrast(gpu):
    # a contrast the fixed point does not close in 40 passes: unconverged
    # alike, the same residual after every pass
    lmax = 8
    o, g = _pair(lmax, 20, 5, rms=1.5, anderson_rate=0.0)
    state = g.ZeroState()
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 2000 * configs.SECONDS_PER_YEAR / o.time_scale
    io = o.step(dt, 2, 0 * load, load)
    ig = g.Step(state, dt, 2, 0 * load, load)
    assert ig.converged == io.converged == 0
    ho, hg = o.residual_history(), g.residual_history()
    assert ho.size == hg.size == 80
    assert np.max(np.abs(hg - ho) / ho) < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [2, 0])
def test_gpu_step_with_tide_matches_oracle(gpu, scheme):
    # the tide channel beside the load under a lateral contrast: the tide's
    # columns enter every pass's right-hand side (and, in Sdirk2, its blend
    # at the inner stage time) as in the oracle
    lmax = 8
    o, g = _pair(lmax, 20, 5)
    state = g.ZeroState()
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    tide = tide_columns(lmax)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    for n in range(2):
        l0, l1 = load * n / 10, load * (n + 1) / 10
        t0, t1 = tide * np.cos(n), tide * np.cos(n + 1)
        io = o.step(dt, scheme, l0, l1, t0, t1)
        ig = g.Step(state, dt, scheme, l0, l1, t0, t1)
        assert ig.converged == io.converged == 1
        for comp in (0, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < TOL, (n, comp)


@pytest.mark.gpu
def test_gpu_step_refuses_a_degree_one_tide(gpu):
    from sl3dpp_gb300._lib import Sl3dgpuError

    lmax = 8
    o, g = _pair(lmax, 20, 5, rms=0.0)
    state = g.ZeroState()
    tide = tide_columns(lmax)
    tide[configs.real_index(1, 1)] = 1e-6
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    with pytest.raises(Sl3dgpuError, match="degree-1"):
        g.Step(state, dt, 2, None, None, None, tide)


@pytest.mark.gpu
@pytest.mark.parametrize("l,toroidal", [(0, False), (2, False), (17, False), (1, True), (5, True)])
def test_gpu_degree_operator_solves_its_own_system(gpu, l, toroidal):
    # DegreeOperator / ToroidalOperator through the C ABI: Solve inverts
    # Apply (K K^-1 b = b off the pinned rows), the load and tide vectors
    # sit on the surface dofs, and the dof map agrees with the operator's
    from sl3dpp_gb300.degree import DegreeOperator
    from sl3dpp_gb300.viscoelastic3d import standard_earth

    op = DegreeOperator(standard_earth(20), 5, l, toroidal=toroidal)
    n = op.DofCount()
    assert n > 0 and op.Bandwidth() == (4 if toroidal else 14)
    rng = np.random.default_rng(l)
    b = rng.standard_normal((3, n))
    x = op.Solve(b.ravel()).reshape(3, n)
    r = op.Apply(x.ravel()).reshape(3, n)
    keep = np.ones(n, bool)
    if toroidal:
        keep[np.abs(x).max(axis=0) == 0.0] = False  # the pinned rotation rows
    assert rel(r[:, keep], b[:, keep]) < 1e-9
    surf = op.SurfaceDof(0)
    assert 0 <= surf < n
    if not toroidal:
        load = op.Load()
        assert np.count_nonzero(load) >= 1 and load[surf] != 0.0
        assert np.any(op.Tide(2 if l == 0 else -1))
