"""Migrating shorelines: the nonlinear sea-level equation (GRDSolver::
SolveNonlinear, src/SeaLevel.cpp:970-1289) and the coupled step that closes
every pass with it (Evolution3D::RunMigrating, src/Evolution3D.cpp:117-133,
Coupled::Closure's nonlinear branch :308-319).

On the CPU the oracle's restatement (oracle/sealevel.py solve_nonlinear) is
checked on what must hold whatever the implementation: the water the ice
loses is the ocean's (the carried load has no mass); where no shoreline moves
the nonlinear solve is the linear one under the grounded ice change; a
thinning marine ice cap floats and the shorelines move; the land held stays
land. The coupled oracle step under still ice is the frozen run (the
reference's own check, tests/TestEvolution3D.cpp:486-507). On the GPU the
library's solve (sl3dgpu_sle_solve_nonlinear) and coupled steps
(sl3dgpu_v3d_run_migrating) are compared with the oracle: fields at 1e-10,
the ocean functions exactly (flotation's 0/1 on cells away from the
threshold); and under still ice the GPU's migrating run is its frozen run.
Synthetic Love numbers, states and ice histories; non-dimensional."""

import numpy as np
import pytest

from oracle import sealevel as S
from sl3dpp_gb300 import configs
from tests import _oracle as O
from tests.test_sealevel import ROTATION, channel_forcing
from tests.test_step import delta_for, rel

RHO_I = 0.917  # ice over water density, the solver's units of the standalone cases


def problem(lmax):
    """A marine ice cap over a polar basin: the sea level (ocean depth) of a
    smooth basin field, the cap grounded where rho_i I > rho_w SL."""
    theta, w, nphi = O.grid(lmax, 1.0)
    tt, pp = np.meshgrid(theta, 2 * np.pi * np.arange(nphi) / nphi, indexing="ij")
    sea = (0.3 * (0.5 * np.cos(2 * tt) + 0.3 + 0.3 * np.sin(2 * pp) * np.sin(tt))).ravel()
    ice = (0.75 * np.exp(-((tt / 0.5) ** 4))).ravel()
    degrees = np.arange(lmax + 1, dtype=np.float64)
    h = np.where(degrees > 0, -1.2 / (degrees + 1.0), 0.0)
    k = np.where(degrees > 0, -0.5 / (degrees + 1.0), 0.0)
    l = np.where(degrees > 0, 0.3 / (degrees + 1.0), 0.0)
    synth = lambda c: O.synthesise_real(lmax, theta, nphi, c)
    expand = lambda f: O.expand_real(lmax, theta, w, nphi, f)
    integ = lambda f: float(np.sum(w * f.reshape(theta.size, nphi).sum(axis=1)) * 2 * np.pi / nphi)
    ocean = S.flotation(ice, sea, 1.0, RHO_I)
    return dict(theta=theta, w=w, nphi=nphi, tt=tt.ravel(), sea=sea, ice=ice, ocean=ocean, h=h, k=k, l=l,
                synth=synth, expand=expand, integ=integ)


def solve(p, frac, forced_land=None, **kw):
    state = dict(ice=p["ice"], sea_level=p["sea"], ocean=p["ocean"], forced_land=forced_land)
    return S.solve_nonlinear(p["synth"], p["expand"], p["integ"], p["h"], p["k"], p["l"], 1.0, 1.0, RHO_I, 1.0,
                             state, ice_change=-frac * p["ice"], **kw)


def test_oracle_thinning_cap_floats_and_keeps_the_water():
    p = problem(16)
    r = solve(p, 0.6, rtol=1e-12, max_iterations=200)
    assert r["converged"]
    floated = (p["ocean"] == 0.0) & (r["ocean"] == 1.0)
    assert np.count_nonzero(floated) > 0 and np.all(p["ice"][floated] > 0.0)
    # the carried load: ice lost and water gained, no net mass
    dice = -0.6 * p["ice"]
    grounded = RHO_I * ((1.0 - r["ocean"]) * dice - (r["ocean"] - p["ocean"]) * p["ice"])
    assert abs(p["integ"](grounded)) > 0.0
    carried = p["synth"](r["load_coefficients"])
    assert abs(r["load_coefficients"][0]) < 1e-10 * np.max(np.abs(r["load_coefficients"]))
    assert abs(p["integ"](carried)) < 1e-10 * abs(p["integ"](grounded))
    # the final state: flotation of its own ice and sea level
    again = S.flotation(r["ice"], r["sea_level"], 1.0, RHO_I)
    assert np.array_equal(again, r["ocean"])


def test_oracle_still_shorelines_are_the_linear_solve():
    """A thinning that floats no cell: the linear solve under the grounded
    ice change rho_i (1 - C) dI (SolveGeneralised) to the solves' bar."""
    p = problem(14)
    r = solve(p, 0.05, rtol=1e-13, max_iterations=400)
    assert r["converged"] and np.array_equal(r["ocean"], p["ocean"])
    direct = RHO_I * (1.0 - p["ocean"]) * (-0.05 * p["ice"])
    lin = S.solve_generalised(p["synth"], p["expand"], p["integ"], p["h"], p["k"], p["l"], 1.0, 1.0, 1.0,
                              p["ocean"], direct, rtol=1e-13, max_iterations=400)
    for key in ("sea_level_change", "displacement", "potential", "tangential_potential"):
        assert rel(r[key], lin[key]) < 1e-10, key


def test_oracle_land_held_stays_land():
    p = problem(12)
    free = solve(p, 0.6, rtol=1e-12, max_iterations=200)
    floated = (p["ocean"] == 0.0) & (free["ocean"] == 1.0)
    held = np.zeros(p["ice"].size, dtype=np.uint8)
    held[np.flatnonzero(floated)[::2]] = 1
    r = solve(p, 0.6, forced_land=held, rtol=1e-12, max_iterations=200)
    assert r["converged"] and np.all(r["ocean"][held == 1] == 0.0)
    assert np.count_nonzero(r["ocean"] != free["ocean"]) >= np.count_nonzero(held)


def test_oracle_refuses_a_state_without_ocean():
    p = problem(8)
    dry = dict(p, ocean=np.zeros_like(p["ocean"]))
    with pytest.raises(ValueError):
        solve(dry, 0.1)


# -- the coupled step (oracle) ----------------------------------------------------------------------------

def basin(o, lmax, depth_m=1500.0, cap_m=2500.0):
    """A marine ice cap over a polar basin for the 3D operator (model length)."""
    theta, w, nphi = O.grid(lmax, 1.0)
    tt, pp = np.meshgrid(theta, 2 * np.pi * np.arange(nphi) / nphi, indexing="ij")
    length = o.body()["length"]
    f = 0.5 * np.cos(2 * tt) + 0.3 + 0.3 * np.sin(2 * pp) * np.sin(tt)
    f = np.where(np.abs(f) < 0.05, np.where(f < 0.0, -0.05, 0.05), f)  # no coast within 5% of the depth scale
    sea = (depth_m * f).ravel() / length
    ice = (cap_m * np.exp(-((tt / 0.45) ** 4))).ravel() / length
    return sea, ice


def _oracle_op(lmax, elements=20, rtol=1e-11):
    return O.OracleStep(O.standard_earth(elements, 0.0, 10.0), O.default_options(lmax, 5, rtol=rtol,
                                                                                   max_iterations=80))


def test_oracle_coupled_step_under_still_ice_is_the_frozen_step():
    """Under ice that does not change and a direct load that moves no
    shoreline, every pass's nonlinear solve is the linear one on the
    background's ocean: the migrating step is the frozen step (as the
    reference checks, tests/TestEvolution3D.cpp:486-507)."""
    lmax = 8
    moving, frozen = _oracle_op(lmax), _oracle_op(lmax)
    sea, ice = basin(moving, lmax)
    moving.set_migrating(ice, sea, rotation=1, rtol=1e-12, max_nonlinear_iterations=400)
    frozen.set_ocean(moving.closure.ocean, rotation=1, rtol=1e-12, max_iterations=400)
    theta, _, nphi = O.grid(lmax, 1.0)
    load = 0.02 * cap_load_field(moving, lmax)
    dt = 500 * configs.SECONDS_PER_YEAR / moving.time_scale
    for n in range(2):
        im = moving.step_migrating(dt, 2, ice, ice, n * load, (n + 1) * load)
        i_f = frozen.step_ocean(dt, 2, n * load, (n + 1) * load)
        assert im.converged and i_f.converged
        assert np.array_equal(moving.closure.current_ocean, moving.closure.ocean)
        for comp in (0, 2):
            assert rel(moving.surface(comp), frozen.surface(comp)) < 1e-8, comp


def cap_load_field(o, lmax, thickness=1000.0):
    theta, _, nphi = O.grid(lmax, 1.0)
    return configs.cap_field(theta, nphi, 15.0, thickness) / o.sigma_scale


# -- the GPU ----------------------------------------------------------------------------------------------

def _gpu_solver(gpu, p, lmax, rotation=0):
    from sl3dpp_gb300.grid import SurfaceGrid
    from sl3dpp_gb300.sealevel import SeaLevelSolver

    grid = SurfaceGrid(lmax, 0, 1.0)
    assert grid.ntheta == p["theta"].size and grid.nphi == p["nphi"]
    degrees = np.arange(lmax + 1, dtype=np.float64)
    extra = dict(ht=-0.4 / (degrees + 1.0), kt=0.2 / (degrees + 1.0), lt=0.1 / (degrees + 1.0))
    rot = dict(ROTATION, rotation=rotation) if rotation else {}
    return SeaLevelSolver(grid, p["h"], p["k"], p["l"], extra["ht"], extra["kt"], extra["lt"], 1.0, 1.0, 1.0, **rot)


@pytest.mark.gpu
@pytest.mark.parametrize("lmax,rotation,channels,held", [(16, 0, False, False), (24, 2, True, False),
                                                         (20, 1, True, True)])
def test_gpu_nonlinear_solve_matches_the_oracle(gpu, lmax, rotation, channels, held):
    import torch

    p = problem(lmax)
    ch, extra = channel_forcing(dict(p, theta=p["theta"], nphi=p["nphi"]), lmax)
    kw = {}
    if channels:
        kw = dict(displacement_response=ch["displacement_response"], potential_response=ch["potential_response"],
                  tangential_response=ch["tangential_response"], toroidal_response=ch["toroidal_response"],
                  tide=ch["tide"], direct_load_outside=ch["direct_load_outside"],
                  solid_surface_change=0.5 * ch["solid_surface_change"],
                  direct_load=0.01 * np.cos(p["tt"]) ** 2, dynamic_sea_level_change=0.005 * np.sin(p["tt"]) ** 2)
    land = None
    if held:
        free = solve(p, 0.6, rtol=1e-12, max_iterations=200)
        land = np.zeros(p["ice"].size, dtype=np.uint8)
        land[np.flatnonzero((p["ocean"] == 0.0) & (free["ocean"] == 1.0))[::2]] = 1
    r = ROTATION
    rot = dict(rotation=rotation, omega=r["omega"], polar=r["polar_moment"], equatorial=r["equatorial_moment"],
               G=r["gravitational_constant"], hc=r["hc"], kc=r["kc"], m_u=r["m_u"], m_phi=r["m_phi"],
               m_c=r["m_c"]) if rotation else {}
    want = solve(p, 0.6, forced_land=land, rtol=1e-11, max_iterations=300, ht=extra["ht"], kt=extra["kt"],
                 lt_tide=extra["lt_tide"], inertia_moment_change=0.002 if rotation else 0.0, **rot, **kw)
    assert want["converged"]
    solver = _gpu_solver(gpu, p, lmax, rotation)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device=gpu)
    state = solver.make_state(dev(p["ice"]), dev(p["sea"]), RHO_I,
                              None if land is None else dev(land))
    assert np.array_equal(state.ocean_function.cpu().numpy(), S.flotation(p["ice"], p["sea"], 1.0, RHO_I, land))
    got = solver.solve_nonlinear(state, RHO_I, rtol=1e-11, max_iterations=300, ice_thickness_change=dev(-0.6 * p["ice"]),
                                 inertia_moment_change=0.002 if rotation else 0.0,
                                 **{k: dev(v) for k, v in kw.items()})
    got = {k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in got.items()}
    assert got["converged"] and abs(got["iterations"] - want["iterations"]) <= 1, (got["iterations"],
                                                                                   want["iterations"])
    assert np.array_equal(got["ocean_function"], want["ocean"])
    assert np.count_nonzero(got["ocean_function"] != p["ocean"]) > 0
    for key in ("sea_level_change", "displacement", "potential", "tangential_potential"):
        assert rel(got[key], want[key]) < 1e-10, key
    assert rel(got["sea_level"], want["sea_level"]) < 1e-12
    assert rel(got["load_coefficients"], want["load_coefficients"]) < 1e-10
    if channels:
        assert rel(got["toroidal_potential"], want["toroidal_potential"]) < 1e-13
    if rotation:
        w = np.asarray(want["angular_velocity"])
        assert np.max(np.abs(np.asarray(got["angular_velocity"]) - w)) < 1e-10 * np.max(np.abs(w))


@pytest.mark.gpu
def test_gpu_nonlinear_solve_refuses_a_dry_state(gpu):
    import torch

    from sl3dpp_gb300._lib import Sl3dgpuError

    lmax = 8
    p = problem(lmax)
    solver = _gpu_solver(gpu, p, lmax)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device=gpu)
    state = solver.make_state(dev(p["ice"]), dev(p["sea"]), RHO_I)
    state.ocean_function = torch.zeros_like(state.ocean_function)
    with pytest.raises(Sl3dgpuError):
        solver.solve_nonlinear(state, RHO_I, ice_thickness_change=dev(-0.1 * p["ice"]))


def _gpu_pair(lmax, elements=24, ldelta=4, rms=0.5, seed=3, rotation=1, **opt):
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    o = O.OracleStep(O.standard_earth(elements, 0.0, 10.0), O.default_options(lmax, 5, **opt))
    g = Viscoelastic3D(standard_earth(elements, 0.0, 10.0), Options.defaults(lmax, 5, **opt))
    d = delta_for(o, lmax, ldelta, rms, seed)
    o.set_delta(d)
    g.set_delta(d)
    sea, ice = basin(o, lmax)
    o.set_migrating(ice, sea, rotation=rotation, rtol=1e-11, max_nonlinear_iterations=300)
    g.set_migrating_ocean(ice, sea, rotation=rotation, rtol=1e-11, max_nonlinear_iterations=300)
    return o, g, sea, ice


@pytest.mark.gpu
@pytest.mark.parametrize("rotation", [1, 0])
def test_gpu_migrating_run_matches_the_oracle(gpu, rotation):
    """A melting marine cap over four Sdirk2 steps (the undisturbed start at
    the background, then the cap thinning to 40%): U, phi and the sea level
    per node at 1e-10 of the oracle's, the ocean functions exactly, and the
    shorelines moving."""
    from sl3dpp_gb300.viscoelastic3d import Evolution3D

    lmax = 12
    o, g, sea, ice = _gpu_pair(lmax, rotation=rotation, rtol=1e-11, max_iterations=80)
    nodes = 5
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    times = np.arange(nodes) * dt
    history = np.stack([ice * (1.0 - 0.15 * n) for n in range(nodes)])
    run = Evolution3D(g, "sdirk2").RunMigrating(times, history)
    np.testing.assert_array_equal(run["ocean"][0], o.closure.ocean)
    for n in range(1, nodes):
        info = o.step_migrating(dt, 2, history[n - 1], history[n])
        assert info.converged and run["infos"][n].converged
        assert abs(run["infos"][n].iterations - info.iterations) <= 1
        for comp, key in ((0, "U"), (2, "phi")):
            assert rel(run[key][n], o.surface(comp)) < 1e-10, (n, key)
        slc_o, omega_o = o.sea_level()
        assert rel(run["sea_level"][n], slc_o) < 1e-10, n
        np.testing.assert_array_equal(run["ocean"][n], o.closure.current_ocean)
        if rotation:
            assert abs(run["omega"][n][2] - omega_o[2]) < 1e-10 * abs(omega_o[2])
    assert np.count_nonzero(run["ocean"][-1] != run["ocean"][0]) > 0


@pytest.mark.gpu
def test_gpu_migrating_run_under_still_ice_is_the_frozen_run(gpu):
    """No ice change and a direct load that moves no shoreline: the GPU's
    migrating run is its frozen run on the background's ocean
    (tests/TestEvolution3D.cpp:486-507, there at 1e-7)."""
    from sl3dpp_gb300.viscoelastic3d import Evolution3D, Options, Viscoelastic3D, standard_earth

    lmax = 12
    opts = Options.defaults(lmax, 5, rtol=1e-12, max_iterations=80)
    a = Viscoelastic3D(standard_earth(24, 0.0, 10.0), opts)
    b = Viscoelastic3D(standard_earth(24, 0.0, 10.0), opts)
    o = _oracle_op(lmax)
    sea, ice = basin(o, lmax)
    a.set_migrating_ocean(ice, sea, rotation=1, rtol=1e-12, max_nonlinear_iterations=400)
    ocean = a.OceanFunction()
    np.testing.assert_array_equal(ocean, S.flotation(ice, sea, 1000.0, 917.0))
    b.set_ocean(ocean, rotation=1, rtol=1e-12, max_iterations=400)
    nodes = 4
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    times = np.arange(nodes) * dt
    load = 0.02 * cap_load_field(o, lmax)
    loads = np.stack([n * load for n in range(nodes)])
    moving = Evolution3D(a, "sdirk2").RunMigrating(times, np.stack([ice] * nodes), loads)
    frozen = Evolution3D(b, "sdirk2").RunOcean(times, loads)
    for n in range(nodes):
        np.testing.assert_array_equal(moving["ocean"][n], ocean)
        for key in ("U", "phi", "sea_level"):
            assert rel(moving[key][n], frozen[key][n]) < 1e-7, (n, key)


@pytest.mark.gpu
def test_gpu_migrating_refusals(gpu):
    from sl3dpp_gb300._lib import Sl3dgpuError
    from sl3dpp_gb300.viscoelastic3d import Evolution3D, Options, Viscoelastic3D, standard_earth

    lmax = 8
    g = Viscoelastic3D(standard_earth(20, 0.0, 10.0), Options.defaults(lmax, 5))
    o = _oracle_op(lmax)
    sea, ice = basin(o, lmax)
    # a prescribed ocean function that is not flotation's
    wrong = S.flotation(ice, sea, 1000.0, 917.0)
    wrong[0] = 1.0 - wrong[0]
    with pytest.raises(Sl3dgpuError):
        g.set_migrating_ocean(ice, sea, ocean_function=wrong)
    g.set_migrating_ocean(ice, sea)
    # the history's first ice must be the background's
    times = np.array([0.0, 1.0])
    with pytest.raises(Sl3dgpuError):
        Evolution3D(g, "sdirk2").RunMigrating(times, np.stack([0.5 * ice, 0.5 * ice]))
    # frozen-shoreline steps are refused under a migrating ocean
    with pytest.raises(Sl3dgpuError):
        g.StepOcean(g.ZeroState(), 1.0, "sdirk2")
