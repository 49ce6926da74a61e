"""The coupled step under an ocean with frozen shorelines (Evolution3D's
Coupled / Closure, src/Evolution3D.cpp:184-394): every pass of the strain
fixed point closes the sea-level equation on the pass flavour's effective
Love numbers, and its total load and centrifugal potential become the
pass's load and tide channels.

On the CPU the oracle's closure (oracle/coupled.py around the oracle's 3D
step) is checked on what must hold whatever the implementation: without an
ocean and without rotation the closure is the plain load channel; the ocean
loses the mass the growing ice takes; the effective Love numbers keep the
axial reciprocity between the inertia and centrifugal numbers. On the
GPU the library's coupled step (sl3dgpu_v3d_step_ocean) is compared with
the oracle pass for pass at 1e-10 (the FP64 form's bar): a small Earth over
several Sdirk2 and trapezoid steps, and config 2's shape (lmax 128, 80
elements of order 5, Burgers, delta to degree 32 at RMS 1, an ocean over
70% of a seeded mask, axial rotation) over the first passes of a stage; the
mixed form under the closure, frozen or migrating, against the FP64 form."""

import numpy as np
import pytest

from sl3dpp_gb300 import configs
from tests import _oracle as O
from tests.test_step import delta_for, rel

GAMMA = 0.29289321881345247560


def ocean_mask(lmax, land_fraction=0.3, seed=11):
    """The ocean of config 2's kind: land where a seeded smooth field is
    highest, over the given fraction of the area."""
    theta, w, nphi = O.grid(lmax, 1.0)
    field = O.synthesise_real(lmax, theta, nphi, configs.land_field_coefficients(lmax, seed))
    return configs.ocean_from_field(field, w, nphi, land_fraction)


def cap_field(lmax, sigma_scale, thickness, alpha=15.0):
    """The ice cap's surface density on the sea-level grid (non-dimensional)."""
    theta, w, nphi = O.grid(lmax, 1.0)
    return configs.cap_field(theta, nphi, alpha, thickness) / sigma_scale


def _oracle_pair(lmax, elements, ngll=5, kelvin=0.0, rtol=1e-10, max_iterations=60):
    layers = O.standard_earth(elements, kelvin, 10.0)
    opts = O.default_options(lmax, ngll, rtol=rtol, max_iterations=max_iterations)
    return O.OracleStep(layers, opts), O.OracleStep(layers, opts)


def test_oracle_closure_without_ocean_or_rotation_is_the_plain_load():
    lmax = 8
    coupled, plain = _oracle_pair(lmax, 20)
    theta, w, nphi = O.grid(lmax, 1.0)
    coupled.set_ocean(np.zeros(theta.size * nphi), rotation=0)
    load = cap_field(lmax, coupled.sigma_scale, 1000.0)
    coefficients = O.expand_real(lmax, theta, w, nphi, load)
    dt = 500 * configs.SECONDS_PER_YEAR / coupled.time_scale
    for n in range(2):
        ic = coupled.step_ocean(dt, 2, load * n / 2, load * (n + 1) / 2)
        ip = plain.step(dt, 2, coefficients * n / 2, coefficients * (n + 1) / 2)
        assert ic.converged and ip.converged and ic.iterations == ip.iterations
        for comp in (0, 2):
            assert rel(coupled.surface(comp), plain.surface(comp)) < 1e-12


def test_oracle_ocean_gives_what_the_ice_takes():
    lmax = 10
    o, _ = _oracle_pair(lmax, 20)
    theta, w, nphi = O.grid(lmax, 1.0)
    ocean = ocean_mask(lmax)
    o.set_ocean(ocean, rotation=1)
    ice = cap_field(lmax, o.sigma_scale, 1000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    info = o.step_ocean(dt, 2, 0.5 * ice, ice)
    assert info.converged
    integ = lambda f: float(np.sum(w * f.reshape(theta.size, nphi).sum(axis=1)) * 2 * np.pi / nphi)
    slc = o.closure.last["sea_level_change"]
    rho_w = o.closure.water_density
    taken = integ(ice)
    assert abs(integ(rho_w * ocean * slc) + taken) < 1e-10 * abs(taken)
    # the growing ice draws the ocean down, and the axial rotation answers the zonal load
    assert integ(ocean * slc) < 0.0
    assert o.closure.last["angular_velocity"][2] != 0.0


def test_oracle_effective_love_numbers_keep_the_axial_reciprocity():
    """The inertia-trace numbers of a flavour against its centrifugal ones:
    m_u + m_phi = sqrt(4 pi) a^4 (g h_c + k_c) / 2, the reciprocity the
    reference checks on every Love table (LoveNumbers::ReciprocityResidual,
    src/LoveNumbers.cpp:52-90), here for the elastic flavour and a relaxed
    one; and loads depress the surface and the potential at degrees >= 2."""
    lmax = 6
    o, _ = _oracle_pair(lmax, 20)
    body = o.body()
    n = lmax + 1
    dt = 5000 * configs.SECONDS_PER_YEAR / o.time_scale
    for scheme, length in [(1, 0.0), (1, dt), (0, dt)]:
        love = o.effective_love(scheme, length)
        h, k = love[:n], love[n:2 * n]
        assert np.all(h[2:] < 0.0) and np.all(k[2:] < 0.0)
        hc, kc, m = love[6 * n], love[6 * n + 1], love[6 * n + 2]
        want = np.sqrt(4 * np.pi) * body["radius"] ** 4 * (body["g"] * hc + kc) / 2
        assert abs(m - want) < 1e-8 * abs(want), (scheme, length, m, want)


def _gpu_pair(lmax, elements, ngll, kelvin, ldelta, rms, seed, rotation, **opt):
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    o = O.OracleStep(O.standard_earth(elements, kelvin, 10.0), O.default_options(lmax, ngll, **opt))
    g = Viscoelastic3D(standard_earth(elements, kelvin, 10.0), Options.defaults(lmax, ngll, **opt))
    if ldelta:
        d = delta_for(o, lmax, ldelta, rms, seed)
        o.set_delta(d)
        g.set_delta(d)
    ocean = ocean_mask(lmax)
    theta, _, nphi = g.ocean_grid()
    assert theta.size * nphi == ocean.size
    o.set_ocean(ocean, rotation=rotation)
    g.set_ocean(ocean, rotation=rotation)
    return o, g


@pytest.mark.gpu
def test_gpu_effective_love_numbers_match_the_oracle(gpu):
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    lmax = 16
    o = O.OracleStep(O.standard_earth(24, 0.5, 10.0), O.default_options(lmax, 5))
    g = Viscoelastic3D(standard_earth(24, 0.5, 10.0), Options.defaults(lmax, 5))
    dt = 250 * configs.SECONDS_PER_YEAR / o.time_scale
    for scheme, length in [(1, 0.0), (1, GAMMA * dt), (0, dt)]:
        want = o.effective_love(scheme, length)
        got = g.effective_love(scheme, length)
        n = lmax + 1
        # each number family against its own largest value (k_c vanishes to
        # rounding: a degree-0 mass redistribution leaves the outer potential)
        for i, name in enumerate(("h", "k", "l", "ht", "kt", "lt")):
            assert rel(got[name], want[i * n:(i + 1) * n]) < 1e-10, (scheme, length, name)
        axial = np.array([got["hc"], got["kc"], got["m"], got["mc"]])
        assert rel(axial, want[6 * n:]) < 1e-10, (scheme, length, axial, want[6 * n:])


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,rotation", [(2, 1), (0, 2), (2, 0)])
def test_gpu_coupled_steps_match_the_oracle(gpu, scheme, rotation):
    lmax = 12
    o, g = _gpu_pair(lmax, 24, 5, 0.5 if scheme == 2 else 0.0, 4, 0.5, 3, rotation, rtol=1e-11,
                     max_iterations=80)
    ice = cap_field(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    state = g.ZeroState()
    # node 0: the instantaneous response, then four steps of a growing cap
    schedule = [(0.0, 0.1, 0.1)] + [(dt, 0.1 * n, 0.1 * (n + 1)) for n in range(1, 5)]
    for length, a, b in schedule:
        io = o.step_ocean(length, scheme, a * ice, b * ice)
        ig = g.StepOcean(state, length, scheme, a * ice, b * ice)
        assert io.converged and ig.converged, (length, a)
        assert abs(ig.iterations - io.iterations) <= 1, (ig.iterations, io.iterations)
        for comp in (0, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < 1e-10, (a, comp)
        slc_g, omega_g, res = g.SeaLevel()
        slc_o, omega_o = o.sea_level()
        assert res.converged
        assert rel(slc_g, slc_o) < 1e-10, a
        if rotation:
            assert np.max(np.abs(omega_g - omega_o)) < 1e-10 * np.max(np.abs(omega_o)), (omega_g, omega_o)


@pytest.mark.gpu
def test_gpu_config2_coupled_stage_passes_match_the_oracle(gpu):
    """Config 2's shape: the first passes of a Sdirk2 first stage, pass for
    pass (a stage cut at its pass budget, both sides)."""
    lmax, passes = 128, 3
    o, g = _gpu_pair(lmax, 80, 6, 0.5, 32, 1.0, 2, 1, rtol=1e-10, max_iterations=passes)
    ice = cap_field(lmax, o.sigma_scale, 2000.0)
    h = GAMMA * 250 * configs.SECONDS_PER_YEAR / o.time_scale
    io = o.step_ocean(h, 1, 0.5 * ice, 0.6 * ice)
    ig = g.StepOcean(g.ZeroState(), h, 1, 0.5 * ice, 0.6 * ice)
    assert ig.iterations == io.iterations == passes
    ro, rg = o.residual_history(), g.residual_history()
    assert np.max(np.abs(rg - ro) / ro) < 1e-8, (rg, ro)
    for comp in (0, 2):
        assert rel(g.Surface(comp), o.surface(comp)) < 1e-10, comp
    slc_g, omega_g, _ = g.SeaLevel()
    slc_o, omega_o = o.sea_level()
    assert rel(slc_g, slc_o) < 1e-10
    assert abs(omega_g[2] - omega_o[2]) < 1e-10 * abs(omega_o[2])


@pytest.mark.gpu
@pytest.mark.parametrize("migrating", [False, True])
def test_gpu_mixed_form_closes_the_ocean(gpu, migrating):
    """The mixed form under the ocean closure: its FP64 passes close the
    sea-level equation (frozen or migrating shorelines), its FP32
    corrections leave the ocean's feedback out, and the FP64 passes refine
    the difference away -- the same steps as the FP64 form to its bar's
    neighbourhood (1e-8), in fewer FP64 passes."""
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth
    from tests.test_migrating import basin

    lmax = 12
    o = O.OracleStep(O.standard_earth(24, 0.5, 10.0), O.default_options(lmax, 5))
    d = delta_for(o, lmax, 4, 0.8, 3)
    forms = {}
    for name, kw in (("fp64", {}), ("mixed", dict(precision=1, correction_rtol=3e-6, correction_memory=8,
                                                   warm_start=1))):
        g = Viscoelastic3D(standard_earth(24, 0.5, 10.0), Options.defaults(lmax, 5, rtol=1e-11, max_iterations=80,
                                                                            **kw))
        g.set_delta(d)
        dt = 500 * configs.SECONDS_PER_YEAR / g.time_scale
        state = g.ZeroState()
        surfaces, passes = [], []
        if migrating:
            sea, ice = basin(o, lmax)
            g.set_migrating_ocean(ice, sea, rotation=1, rtol=1e-11, max_nonlinear_iterations=300)
            for n in range(1, 4):
                info = g.StepMigrating(state, dt, "sdirk2", ice * (1 - 0.15 * (n - 1)), ice * (1 - 0.15 * n))
                assert info.converged
                surfaces.append((g.Surface(0), g.SeaLevel()[0], g.OceanFunction()))
                passes.append(info.iterations)
        else:
            g.set_ocean(ocean_mask(lmax), rotation=1, rtol=1e-11)
            load = cap_field(lmax, g.surface_density_scale, 2000.0)
            g.StepOcean(state, 0.0, 2, 0.1 * load, 0.1 * load)
            for n in range(1, 4):
                info = g.StepOcean(state, dt, 2, 0.1 * n * load, 0.1 * (n + 1) * load)
                assert info.converged
                surfaces.append((g.Surface(0), g.SeaLevel()[0], None))
                passes.append(info.iterations)
        forms[name] = (surfaces, passes)
    for (u64, s64, c64), (umx, smx, cmx) in zip(forms["fp64"][0], forms["mixed"][0]):
        assert rel(umx, u64) < 1e-8 and rel(smx, s64) < 1e-8
        if migrating:
            np.testing.assert_array_equal(cmx, c64)
    assert sum(forms["mixed"][1]) < sum(forms["fp64"][1])
