"""Evolution3D's march without an ocean or rotational feedback
(src/Evolution3D.cpp:184-449 under GRDSolver::NoOceanState), and the
warm-start hook of the step (OpenStep::Converge's start,
include/sl3dpp/Viscoelastic3D.hpp:562-569).

The march is node 0's instantaneous elastic response, then one step per
node; against the oracle stepping the same nodes (1e-10). A warm start that
is the converged answer is kept and closes the stage in fewer passes (FP64
passes in the FP64 form, FP32 correction passes in the mixed form) at the same
result; a wild one is discarded and changes nothing but one pass.""" 

import numpy as np
import pytest

from tests import _oracle as O
from tests.test_step import _pair, cap_load, rel
from sl3dpp_gb300 import configs

TOL = 1e-10


@pytest.mark.gpu
def test_gpu_evolution_run_matches_the_oracle_march(gpu):
    from sl3dpp_gb300.viscoelastic3d import Evolution3D

    lmax = 8
    o, g = _pair(lmax, 20, 5, rms=0.8)
    full = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    nodes = 4
    times = dt * np.arange(nodes)
    loads = np.stack([full * min(k, 3) / 3 for k in range(nodes)])
    out = Evolution3D(g).Run(times, loads)
    for k in range(nodes):
        step_dt = 0.0 if k == 0 else times[k] - times[k - 1]
        io = o.step(step_dt, 2, loads[max(k - 1, 0)], loads[k])
        assert out["infos"][k].converged == io.converged == 1
        assert rel(out["U"][k], o.surface(0)) < TOL, k
        assert rel(out["phi"][k], o.surface(2)) < TOL, k
    inst = Evolution3D(g).Instantaneous(loads[1])
    o2, _ = _pair(lmax, 20, 5, rms=0.8)
    o2.step(0.0, 2, loads[1], loads[1])
    assert rel(inst["U"], o2.surface(0)) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_warm_start_is_kept_when_better_and_discarded_otherwise(gpu, precision):
    lmax = 8
    _, a = _pair(lmax, 20, 5, rms=0.8, precision=precision, rtol=1e-10, max_iterations=60)
    _, b = _pair(lmax, 20, 5, rms=0.8, precision=precision, rtol=1e-10, max_iterations=60)
    _, c = _pair(lmax, 20, 5, rms=0.8, precision=precision, rtol=1e-10, max_iterations=60)
    o = O.OracleStep(O.standard_earth(20), O.default_options(lmax, 5))
    full = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    sa, sb, sc = a.ZeroState(), b.ZeroState(), c.ZeroState()
    for n in range(3):
        l0, l1 = full * n / 10, full * (n + 1) / 10
        ia = a.Step(sa, dt, 2, l0, l1)
        answer = sa.device_layout_coefficients()
        b.set_start(answer)
        ib = b.Step(sb, dt, 2, l0, l1)
        assert b.start_taken
        assert ib.converged == 1
        if precision == 0:
            # the FP64 form tries the guess as a first pass
            assert ib.iterations < ia.iterations
        else:
            # the mixed form starts its first FP32 correction from it
            assert ib.correction_passes < ia.correction_passes
        wild = np.random.default_rng(n).standard_normal(answer.size) * 1e3 * np.max(np.abs(answer))
        c.set_start(wild)
        ic = c.Step(sc, dt, 2, l0, l1)
        assert not c.start_taken
        assert ic.iterations == ia.iterations
        if precision == 1:
            # the dropped guess's one pass in each Sdirk2 stage that took it
            # (the first stage only from a state with strain coefficients)
            assert ia.correction_passes < ic.correction_passes <= ia.correction_passes + 2
        for comp in (0, 2):
            assert rel(b.Surface(comp), a.Surface(comp)) < 1e-8
            assert rel(c.Surface(comp), a.Surface(comp)) < 1e-12
