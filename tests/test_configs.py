"""The GPU step against the oracle at the measured configurations' sizes.

- Config 1 (lmax 32, 40 elements of order 4, Maxwell, delta to degree 8 at
  RMS 0.5 between 100 and 670 km, a 15 degree cap growing to 2 km over 10
  Sdirk2 steps of 500 yr, Anderson depth 5, rtol 1e-10): all ten steps, the
  surface U and phi and the pass counts, FP64 form, 1e-10.
- lmax 128 (80 elements of order 5, Burgers with transient viscosity / 10
  and modulus ratio 0.5, delta to degree 32 at RMS 1.0): the first three
  passes of a backward Euler stage, pass for pass.
- lmax 256 (120 elements of order 5, Maxwell, delta to degree 64 at RMS 1.0,
  the benchmark's workload): the first two passes of a backward Euler stage
  of the benchmark's first-stage length, pass for pass, FP64 form; and the
  benchmark's first Sdirk2 step in the mixed form against the FP64 form at
  the mixed form's bar, 1e-8.

A stage cut at a pass budget returns unconverged with its last iterate on
both sides, so the comparison covers the stage start, the passes and the
finish. The oracle runs these on every host core (about a minute at lmax
256)."""

import numpy as np
import pytest

from sl3dpp_gb300 import configs
from tests import _oracle as O
from tests.test_step import cap_load, delta_for, rel

TOL = 1e-10
GAMMA = 0.29289321881345247560


def _pair(lmax, elements, ngll, kelvin, ldelta, rms, seed, **opt):
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    o = O.OracleStep(O.standard_earth(elements, kelvin, 10.0), O.default_options(lmax, ngll, **opt))
    g = Viscoelastic3D(standard_earth(elements, kelvin, 10.0), Options.defaults(lmax, ngll, **opt))
    assert (g.node_count, g.ntheta, g.nphi) == (o.P, o.ntheta, o.nphi)
    d = delta_for(o, lmax, ldelta, rms, seed)
    o.set_delta(d)
    g.set_delta(d)
    return o, g


@pytest.mark.gpu
def test_gpu_config1_all_ten_steps_match_the_oracle(gpu):
    lmax = 32
    o, g = _pair(lmax, 40, 5, 0.0, 8, 0.5, 1, rtol=1e-10, max_iterations=60)
    full = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    state = g.ZeroState()
    for n in range(10):
        l0, l1 = full * n / 10, full * (n + 1) / 10
        io = o.step(dt, 2, l0, l1)
        ig = g.Step(state, dt, 2, l0, l1)
        assert ig.converged == io.converged == 1, n
        assert abs(ig.iterations - io.iterations) <= 1, (n, ig.iterations, io.iterations)
        for comp in (0, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < TOL, (n, comp)


def _stage_passes(lmax, elements, ngll, kelvin, ldelta, seed, passes, years):
    o, g = _pair(lmax, elements, ngll, kelvin, ldelta, 1.0, seed, rtol=1e-10, max_iterations=passes)
    full = cap_load(lmax, o.sigma_scale, 2000.0)
    h = GAMMA * years * configs.SECONDS_PER_YEAR / o.time_scale
    l0, l1 = 0.5 * full, 0.6 * full
    io = o.step(h, 1, l0, l1)
    ig = g.Step(g.ZeroState(), h, 1, l0, l1)
    assert ig.iterations == io.iterations == passes and not ig.converged and not io.converged
    ro, rg = o.residual_history(), g.residual_history()
    assert len(ro) == len(rg) == passes
    assert np.max(np.abs(rg - ro) / ro) < 1e-8, (rg, ro)
    for comp in (0, 2):
        assert rel(g.Surface(comp), o.surface(comp)) < TOL, comp


@pytest.mark.gpu
def test_gpu_lmax128_burgers_stage_passes_match_the_oracle(gpu):
    _stage_passes(128, 80, 6, 0.5, 32, 2, 3, 250.0)


@pytest.mark.gpu
def test_gpu_lmax256_stage_passes_match_the_oracle(gpu):
    _stage_passes(256, 120, 6, 0.0, 64, 1, 2, 500.0)


@pytest.mark.gpu
def test_gpu_lmax256_mixed_stage_meets_its_bar_against_fp64(gpu):
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    lmax = 256
    o = O.OracleStep(O.standard_earth(120), O.default_options(lmax, 6))  # the grid and delta samples only
    d = delta_for(o, lmax, 64, 1.0, 1)
    full = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    out = []
    for mixed in (0, 1):
        g = Viscoelastic3D(standard_earth(120), Options.defaults(
            lmax, 6, rtol=1e-10, max_iterations=150, precision=mixed, correction_rtol=3e-6, correction_memory=10,
            fp64_emulation=mixed))
        g.set_delta(d)
        # the benchmark's first step: from rest the plain FP64 fixed point takes
        # about 60 passes a stage (residual ratio ~0.7 a pass) to reach 1e-10
        info = g.Step(g.ZeroState(), dt, 2, 0.0 * full, 0.1 * full)
        assert info.converged, (mixed, info.iterations, info.residual, g.residual_history())
        out.append((g.Surface(0), g.Surface(2)))
        del g
    (U64, P64), (U32, P32) = out
    assert rel(U32, U64) < 1e-8 and rel(P32, P64) < 1e-8
