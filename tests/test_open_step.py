"""The open step and the grid coupling through the C ABI
(Viscoelastic3D::OpenStep, include/sl3dpp/Viscoelastic3D.hpp:440-640;
GridCoupling, include/sl3dpp/GridCoupling.hpp:82-428).

A driver's own within-step iteration -- StartStep, then Respond,
AddChannels, StrainOf and RelativeChange until the change is under the
tolerance, then Finish -- is the operator's own plain fixed point step for
step: the same passes in the same order, so the same surface values and the
same state, and the oracle's step at its bar; Close under known channels and
Finish are the operator's Step. The grid coupling's maps keep their
identities: Analyse(Synthesise(s)) = s for band-limited coefficients, the
degree forces are linear, the strain of zero solutions is zero."""

import numpy as np
import pytest

from sl3dpp_gb300 import configs
from tests import _oracle as O
from tests.test_step import cap_load, delta_for, rel

GAMMA = 0.29289321881345247560


def _ops(lmax, **opt):
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    o = O.OracleStep(O.standard_earth(24, 0.5), O.default_options(lmax, 5, **opt))
    a = Viscoelastic3D(standard_earth(24, 0.5), Options.defaults(lmax, 5, **opt))
    b = Viscoelastic3D(standard_earth(24, 0.5), Options.defaults(lmax, 5, **opt))
    d = delta_for(o, lmax, 4, 0.8, 5)
    for x in (o, a, b):
        x.set_delta(d)
    return o, a, b


@pytest.mark.gpu
def test_gpu_driver_iteration_is_the_plain_fixed_point(gpu):
    lmax = 10
    opt = dict(rtol=1e-11, max_iterations=80, anderson_memory=0)
    o, ref, drv = _ops(lmax, **opt)
    full = cap_load(lmax, o.sigma_scale, 2000.0)
    h = GAMMA * 500 * configs.SECONDS_PER_YEAR / o.time_scale
    s_ref, s_drv = ref.ZeroState(), drv.ZeroState()
    for n in range(3):
        l0, l1 = full * n / 3, full * (n + 1) / 3
        io = o.step(h, 1, l0, l1)
        info = ref.Step(s_ref, h, "backward_euler", l0, l1)
        step = drv.StartStep(s_drv, h, 1, l0)
        s = step.StartStrain()
        passes, first = 0, True
        while True:
            step.Respond(None if first else s)
            first = False
            step.AddChannels(l1)
            nxt = step.StrainOf()
            change = step.RelativeChange(nxt, s)
            passes += 1
            s = nxt
            if change <= opt["rtol"] or passes >= opt["max_iterations"]:
                break
        step.Finish(s)
        assert info.converged and passes == info.iterations == io.iterations, (passes, info.iterations)
        for comp in (0, 2, 3):
            assert rel(drv.Surface(comp), ref.Surface(comp)) == 0.0, comp
        for comp in (0, 2):
            assert rel(drv.Surface(comp), o.surface(comp)) < 1e-10, comp
    assert rel(s_drv.strain_coefficients(), s_ref.strain_coefficients()) == 0.0


@pytest.mark.gpu
def test_gpu_open_step_close_is_the_step(gpu):
    """Close under known channels (the operator's own Anderson fixed point)
    and Finish give the step's state and surface."""
    lmax = 10
    _, ref, drv = _ops(lmax, rtol=1e-11, max_iterations=80)
    o = O.OracleStep(O.standard_earth(24, 0.5), O.default_options(lmax, 5))
    full = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    s_ref, s_drv = ref.ZeroState(), drv.ZeroState()
    info = ref.Step(s_ref, dt, "exponential_trapezoid", 0 * full, full)
    step = drv.StartStep(s_drv, dt, 0, 0 * full)
    strain, ic = step.Close(full)
    step.Finish()
    assert ic.iterations == info.iterations and ic.converged
    for comp in (0, 2):
        assert rel(drv.Surface(comp), ref.Surface(comp)) == 0.0
    assert rel(s_drv.strain_coefficients(), s_ref.strain_coefficients()) == 0.0


@pytest.mark.gpu
def test_gpu_grid_coupling_identities(gpu):
    import torch

    lmax = 8
    _, op, _ = _ops(lmax)
    full = cap_load(lmax, op.surface_density_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / op.time_scale
    state = op.ZeroState()
    op.Step(state, dt, "backward_euler", 0 * full, full)
    step = op.StartStep(state, dt, 1, None)
    s = step.StartStrain()
    # Analyse(Synthesise(s)) = s: s is band-limited and the grid oversampled
    c0, c1, r = op.SynthesiseTensor(s)
    back = op.AnalyseTensor(c0, c1, r)
    err = (torch.max(torch.abs(back - s)) / torch.max(torch.abs(s))).item()
    assert err < 1e-12, err
    # a driver's pass on the open step
    step.Respond(s)
    step.AddChannels(full)
    mine = step.StrainOf()
    lay = op.layout()
    # the degree forces are linear
    f1s, f1t = op.DegreeForces(s)
    f2s, f2t = op.DegreeForces(2.5 * s)
    assert (torch.max(torch.abs(f2s - 2.5 * f1s)) / torch.max(torch.abs(f2s))).item() < 1e-14
    # the strain of zero solutions
    sph = torch.zeros(lay["spheroidal"], dtype=torch.complex128, device="cuda")
    tor = torch.zeros(max(lay["toroidal"], 1), dtype=torch.complex128, device="cuda")
    zero = op.StrainOfSolutions(sph, tor)
    assert torch.max(torch.abs(zero)).item() == 0.0
    step.Finish(mine)
    layout = op.solution_layout(3)
    assert layout["sph_dofs"] > 0 and layout["tor_dofs"] > 0


@pytest.mark.gpu
def test_gpu_conjugate_gradient_close_through_the_open_step(gpu):
    """Under the conjugate-gradient step solver: Forces, Solve and Apply of
    the open step (OpenStep::Forces / Solve / Apply) close the stage as the
    operator's own Step does -- the solution satisfies Apply(x) = Forces to
    the solve's tolerance, its strain finishes the stage to the step's
    surface and state."""
    import torch

    lmax = 10
    opt = dict(rtol=1e-11, max_iterations=80, solver=1, solve_rtol=1e-12, solve_max_iterations=300)
    o, ref, drv = _ops(lmax, **opt)
    full = cap_load(lmax, o.sigma_scale, 2000.0)
    h = GAMMA * 500 * configs.SECONDS_PER_YEAR / o.time_scale
    s_ref, s_drv = ref.ZeroState(), drv.ZeroState()
    info = ref.Step(s_ref, h, "backward_euler", 0 * full, full)
    step = drv.StartStep(s_drv, h, 1, 0 * full)
    f = step.Forces(full)
    x, si = step.Solve(f)
    assert si.converged and si.solve_iterations == info.solve_iterations
    resid = (torch.max(torch.abs(step.Apply(x) - f)) / torch.max(torch.abs(f))).item()
    assert resid < 1e-9, resid
    strain = step.StrainOf()
    step.Finish(strain)
    for comp in (0, 2):
        assert rel(drv.Surface(comp), ref.Surface(comp)) < 1e-13
    assert rel(s_drv.strain_coefficients(), s_ref.strain_coefficients()) < 1e-13
