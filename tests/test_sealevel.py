"""The sea-level equation's load fixed point (GRDSolver::SolveGeneralised,
src/SeaLevel.cpp:397-736, direct load, no rotational feedback): the oracle's
numpy restatement checked on the reference's structural identities
(tests/TestSeaLevel.cpp:135-206: the rigid-earth eustatic limit, the ocean
gaining the mass the load lost), then the GPU solver against the oracle and
the same identities. Synthetic Love numbers and state; non-dimensional."""

import numpy as np
import pytest

from oracle import sealevel as sle_oracle
from tests import _oracle


def problem(lmax, rigid=False, ocean_on=True):
    theta, w, nphi = _oracle.grid(lmax, 1.0)
    tt, pp = np.meshgrid(theta, 2 * np.pi * np.arange(nphi) / nphi, indexing="ij")
    ocean = (np.cos(tt) < 0.4 + 0.2 * np.sin(2 * pp)).astype(np.float64).ravel()
    if not ocean_on:
        ocean[:] = 0.0
    land = 1.0 - (np.cos(tt) < 0.4 + 0.2 * np.sin(2 * pp)).astype(np.float64)
    load = (-0.5 * np.exp(-(((tt - 0.3) / 0.2) ** 2)) * (1.0 + 0.3 * np.cos(pp)) * land).ravel()
    degrees = np.arange(lmax + 1, dtype=np.float64)
    h = np.where(degrees > 0, -1.2 / (degrees + 1.0), 0.0)
    k = np.where(degrees > 0, -0.5 / (degrees + 1.0), 0.0)
    lt = np.where(degrees > 0, 0.3 / (degrees + 1.0), 0.0)
    if rigid:
        h[:] = k[:] = lt[:] = 0.0
    synth = lambda c: _oracle.synthesise_real(lmax, theta, nphi, c)
    expand = lambda f: _oracle.expand_real(lmax, theta, w, nphi, f)
    integ = lambda f: float(np.sum(w * f.reshape(theta.size, nphi).sum(axis=1)) * 2 * np.pi / nphi)
    return dict(theta=theta, w=w, nphi=nphi, ocean=ocean, load=load, h=h, k=k, lt=lt, synth=synth,
                expand=expand, integ=integ)


def oracle_solve(p, **kw):
    return sle_oracle.solve_generalised(p["synth"], p["expand"], p["integ"], p["h"], p["k"], p["lt"], 1.0, 1.0, 1.0,
                                        p["ocean"], p["load"], **kw)


def test_oracle_rigid_earth_is_the_eustatic_value():
    p = problem(12, rigid=True)
    r = oracle_solve(p, rtol=1e-12, max_iterations=50)
    eustatic = -p["integ"](p["load"]) / p["integ"](p["ocean"])  # rho_w = a = 1
    assert r["converged"]
    assert np.max(np.abs(r["sea_level_change"] - eustatic)) < 1e-12 * abs(eustatic)
    assert np.max(np.abs(r["displacement"])) == 0.0


def test_oracle_ocean_gains_the_mass_the_load_lost():
    p = problem(16)
    r = oracle_solve(p, rtol=1e-12, max_iterations=200)
    assert r["converged"] and r["iterations"] < 60
    gained = p["integ"](p["ocean"] * r["sea_level_change"])
    assert abs(gained + p["integ"](p["load"])) < 1e-10 * abs(p["integ"](p["load"]))
    # the fingerprint's shape: far-field rise, near-field fall
    s = r["sea_level_change"]
    assert s.min() < 0.0 < s.max()


def _gpu_solve(gpu, p, lmax, **kw):
    import torch

    from sl3dpp_gb300.grid import SurfaceGrid
    from sl3dpp_gb300.sealevel import SeaLevelSolver

    grid = SurfaceGrid(lmax, 0, 1.0)
    assert grid.ntheta == p["theta"].size and grid.nphi == p["nphi"]
    solver = SeaLevelSolver(grid, p["h"], p["k"], p["lt"], p.get("ht"), p.get("kt"), p.get("lt_tide"), 1.0, 1.0, 1.0,
                            **p.get("rotation", {}))
    channels = {name: torch.tensor(v, device=gpu) for name, v in kw.pop("channels", {}).items()}
    r = solver.solve_generalised(torch.tensor(p["ocean"], device=gpu), direct_load=torch.tensor(p["load"], device=gpu),
                                 **channels, **kw)
    return {k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in r.items()}


@pytest.mark.gpu
@pytest.mark.parametrize("lmax,memory", [(16, 5), (24, 5), (24, 0)])
def test_gpu_sea_level_matches_oracle(gpu, lmax, memory):
    p = problem(lmax)
    want = oracle_solve(p, rtol=1e-11, max_iterations=300, anderson_memory=memory)
    got = _gpu_solve(gpu, p, lmax, rtol=1e-11, max_iterations=300, anderson_memory=memory)
    assert want["converged"] and got["converged"]
    assert got["iterations"] == want["iterations"]
    for key in ("sea_level_change", "displacement", "potential", "tangential_potential"):
        scale = np.max(np.abs(want[key]))
        assert np.max(np.abs(got[key] - want[key])) < 1e-10 * scale, key
    assert abs(got["uniform_shift"] - want["uniform_shift"]) < 1e-10 * abs(want["uniform_shift"])


@pytest.mark.gpu
def test_gpu_sea_level_identities(gpu):
    lmax = 20
    rigid = problem(lmax, rigid=True)
    r = _gpu_solve(gpu, rigid, lmax, rtol=1e-12, max_iterations=50)
    eustatic = -rigid["integ"](rigid["load"]) / rigid["integ"](rigid["ocean"])
    assert r["converged"]
    assert np.max(np.abs(r["sea_level_change"] - eustatic)) < 1e-11 * abs(eustatic)
    assert np.max(np.abs(r["displacement"])) < 1e-15
    p = problem(lmax)
    r = _gpu_solve(gpu, p, lmax, rtol=1e-12, max_iterations=200)
    gained = p["integ"](p["ocean"] * r["sea_level_change"])
    assert abs(gained + p["integ"](p["load"])) < 1e-10 * abs(p["integ"](p["load"]))
    # no load: nothing to solve, zero fields (the reference's !anyForcing)
    p0 = dict(p, load=np.zeros_like(p["load"]))
    r = _gpu_solve(gpu, p0, lmax)
    assert r["converged"] and r["iterations"] == 0
    assert np.max(np.abs(r["sea_level_change"])) == 0.0
    # no ocean: no water to conserve, the load alone (no shift)
    dry = problem(lmax, ocean_on=False)
    r = _gpu_solve(gpu, dry, lmax, rtol=1e-12, max_iterations=20)
    want = oracle_solve(dry, rtol=1e-12, max_iterations=20)
    assert r["uniform_shift"] == 0.0 and r["converged"] and r["iterations"] == want["iterations"]
    assert np.max(np.abs(r["sea_level_change"] - want["sea_level_change"])) < 1e-12 * np.max(
        np.abs(want["sea_level_change"]))


def channel_forcing(p, lmax, seed=5):
    """The coupled closure's other channels: ready responses, a tide (degrees
    2 and up), a load outside the water budget, a layer on the solid surface."""
    rng = np.random.default_rng(seed)
    ncoef = (lmax + 1) * (lmax + 2) // 2
    degree = np.concatenate([np.full(l + 1, l) for l in range(lmax + 1)])
    m = np.concatenate([np.arange(l + 1) for l in range(lmax + 1)])

    def coeffs(scale):
        c = (rng.standard_normal(ncoef) + 1j * rng.standard_normal(ncoef)) * scale / (1.0 + degree) ** 2
        c[m == 0] = c[m == 0].real  # a real field's m = 0 coefficients are real
        return c

    tide = coeffs(0.05)
    tide[degree < 2] = 0.0
    tt, pp = np.meshgrid(p["theta"], 2 * np.pi * np.arange(p["nphi"]) / p["nphi"], indexing="ij")
    outside = (0.05 * np.sin(3 * pp) * np.sin(tt) ** 3).ravel()
    layer = (0.02 * np.cos(tt) ** 2).ravel()
    degrees = np.arange(lmax + 1, dtype=np.float64)
    extra = dict(ht=-0.4 / (degrees + 1.0), kt=0.2 / (degrees + 1.0), lt_tide=0.1 / (degrees + 1.0))
    return dict(displacement_response=coeffs(0.01), potential_response=coeffs(0.02),
                tangential_response=coeffs(0.01), toroidal_response=coeffs(0.01), tide=tide,
                direct_load_outside=outside, solid_surface_change=layer), extra


def test_oracle_channels_keep_the_water_budget():
    """The responses, tide and layer move the sea level but only the direct
    load in the budget changes the water's mass (:577-587)."""
    lmax = 14
    p = problem(lmax)
    ch, extra = channel_forcing(p, lmax)
    r = sle_oracle.solve_generalised(p["synth"], p["expand"], p["integ"], p["h"], p["k"], p["lt"], 1.0, 1.0, 1.0,
                                     p["ocean"], p["load"], rtol=1e-12, max_iterations=300, **ch,
                                     ht=extra["ht"], kt=extra["kt"], lt_tide=extra["lt_tide"])
    assert r["converged"]
    gained = p["integ"](p["ocean"] * r["sea_level_change"])
    assert abs(gained + p["integ"](p["load"])) < 1e-10 * abs(p["integ"](p["load"]))
    assert np.max(np.abs(r["toroidal_potential"] - p["synth"](ch["toroidal_response"]))) == 0.0


@pytest.mark.gpu
def test_gpu_sea_level_channels_match_oracle(gpu):
    lmax = 18
    p = problem(lmax)
    ch, extra = channel_forcing(p, lmax)
    want = sle_oracle.solve_generalised(p["synth"], p["expand"], p["integ"], p["h"], p["k"], p["lt"], 1.0, 1.0,
                                        1.0, p["ocean"], p["load"], rtol=1e-11, max_iterations=300, **ch,
                                        ht=extra["ht"], kt=extra["kt"], lt_tide=extra["lt_tide"])
    got = _gpu_solve(gpu, dict(p, **extra), lmax, rtol=1e-11, max_iterations=300, channels=ch)
    assert want["converged"] and got["converged"] and got["iterations"] == want["iterations"]
    for key in ("sea_level_change", "displacement", "potential", "tangential_potential", "toroidal_potential"):
        scale = np.max(np.abs(want[key]))
        assert np.max(np.abs(got[key] - want[key])) < 1e-10 * scale, key


ROTATION = dict(omega=0.5, polar_moment=0.33, equatorial_moment=0.32, gravitational_constant=1.0, hc=0.1, kc=0.05,
                m_u=0.01, m_phi=0.02, m_c=0.03)


def rotation_oracle(p, ch, extra, rotation, **kw):
    r = ROTATION
    return sle_oracle.solve_generalised(p["synth"], p["expand"], p["integ"], p["h"], p["k"], p["lt"], 1.0, 1.0, 1.0,
                                        p["ocean"], p["load"], **ch, ht=extra["ht"], kt=extra["kt"],
                                        lt_tide=extra["lt_tide"], rotation=rotation, omega=r["omega"],
                                        polar=r["polar_moment"], equatorial=r["equatorial_moment"],
                                        G=r["gravitational_constant"], hc=r["hc"], kc=r["kc"], m_u=r["m_u"],
                                        m_phi=r["m_phi"], m_c=r["m_c"], **kw)


def test_oracle_rotation_moves_the_pole_and_keeps_the_budget():
    """Full feedback (tests/TestSeaLevel.cpp:167-206's checks): an off-axis
    load moves the pole; the ocean still gains the mass the load lost."""
    lmax = 12
    p = problem(lmax)
    ch, extra = channel_forcing(p, lmax)
    r = rotation_oracle(p, {}, extra, 2, rtol=1e-12, max_iterations=300)
    assert r["converged"]
    assert np.hypot(r["angular_velocity"][0], r["angular_velocity"][1]) > 0.0
    gained = p["integ"](p["ocean"] * r["sea_level_change"])
    assert abs(gained + p["integ"](p["load"])) < 1e-10 * abs(p["integ"](p["load"]))
    axial = rotation_oracle(p, {}, extra, 1, rtol=1e-12, max_iterations=300)
    assert axial["angular_velocity"][0] == 0.0 and axial["angular_velocity"][1] == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("rotation,with_channels", [(2, False), (2, True), (1, True)])
def test_gpu_sea_level_rotation_matches_oracle(gpu, rotation, with_channels):
    lmax = 16
    p = problem(lmax)
    ch, extra = channel_forcing(p, lmax)
    ch = ch if with_channels else {}
    kw = dict(inertia_moment_change=0.002, angular_momentum_change=(0.001, -0.002, 0.0005))
    want = rotation_oracle(p, ch, extra, rotation, rtol=1e-11, max_iterations=300, **kw)
    q = dict(p, **extra, rotation=dict(ROTATION, rotation=rotation))
    got = _gpu_solve(gpu, q, lmax, rtol=1e-11, max_iterations=300, channels=ch, **kw)
    # the last change sits near rtol in one case: the stopping pass may differ by one
    assert want["converged"] and got["converged"] and abs(got["iterations"] - want["iterations"]) <= 1
    for key in ("sea_level_change", "displacement", "potential", "tangential_potential"):
        scale = np.max(np.abs(want[key]))
        assert np.max(np.abs(got[key] - want[key])) < 1e-10 * scale, key
    w = np.asarray(want["angular_velocity"])
    assert np.max(np.abs(np.asarray(got["angular_velocity"]) - w)) < 1e-10 * np.max(np.abs(w))
