"""The mixed form of the 3D step (precision 1): FP64 passes and stopping rule,
FP32 corrections between them. Its steps against the FP64 oracle on the same
inputs, at the mixed form's bar of 1e-8 relative on the surface displacement,
the potential and the strain coefficients."""

import numpy as np
import pytest

from tests import _oracle as O
from tests.test_step import _pair, cap_load, rel
from sl3dpp_gb300 import configs

TOL_MIXED = 1e-8


def test_mixed_options_are_checked_before_device_work():
    import __graft_entry__

    __graft_entry__.build()
    from sl3dpp_gb300 import _lib
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    layers = standard_earth(20)
    for bad, text in ((dict(precision=2), "precision"), (dict(precision=1, correction_rtol=0.0), "correction_rtol"),
                      (dict(precision=1, correction_rtol=1.5), "correction_rtol")):
        with pytest.raises(_lib.Sl3dgpuError) as err:
            Viscoelastic3D(layers, Options.defaults(8, **bad))
        assert err.value.status == _lib.ERR_ARGUMENT and text in str(err.value)


def _run(o, g, scheme, steps, dt, load):
    state = g.ZeroState()
    infos = []
    for n in range(steps):
        l0, l1 = load * n / 10, load * (n + 1) / 10
        io = o.step(dt, scheme, l0, l1)
        ig = g.Step(state, dt, scheme, l0, l1)
        assert io.converged == 1 and ig.converged == 1, (n, ig.iterations, ig.residual)
        for comp in (0, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < TOL_MIXED, (n, comp)
        infos.append((io, ig))
    want = np.zeros(g.spectral_size, dtype=np.complex128)
    o.L.oracle_v3d_state_strain(o.state, want.ctypes.data)
    assert rel(state.strain_coefficients(), want) < TOL_MIXED
    return infos


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [2, 0, 1])
def test_mixed_step_matches_fp64_oracle(gpu, scheme):
    lmax = 8
    o, g = _pair(lmax, 20, 5, rms=0.8, precision=1, rtol=1e-10, max_iterations=60)
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    infos = _run(o, g, scheme, 3, dt, load)
    for io, ig in infos:
        # the FP64 passes the mixed form spends are a few per stage
        assert ig.iterations <= io.iterations
        assert ig.correction_passes > 0
    hist = g.correction_history()
    assert hist.size > 0 and np.all(np.isfinite(hist))
    # every FP64 pass but the last of a stage is followed by a correction that
    # ends at the correction tolerance or at the pass limit
    assert g.residual_history().size == infos[-1][1].iterations


@pytest.mark.gpu
def test_mixed_step_matches_fp64_oracle_burgers_ngll6_lmax16(gpu):
    lmax = 16
    o, g = _pair(lmax, 24, 6, kelvin=0.5, rms=1.0, ldelta=6, seed=3, precision=1, rtol=1e-10, max_iterations=60)
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 250 * configs.SECONDS_PER_YEAR / o.time_scale
    infos = _run(o, g, 2, 2, dt, load)
    io, ig = infos[-1]
    assert ig.iterations < io.iterations


@pytest.mark.gpu
def test_mixed_and_fp64_gpu_forms_agree_and_fp64_passes_drop(gpu):
    # the same operator in both forms: the mixed form reaches the FP64 form's
    # tolerance with a handful of FP64 passes
    lmax = 12
    results = {}
    for precision in (0, 1):
        o, g = _pair(lmax, 20, 5, rms=1.0, ldelta=5, seed=5, precision=precision, rtol=1e-10, max_iterations=60)
        state = g.ZeroState()
        load = cap_load(lmax, o.sigma_scale, 2000.0)
        dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
        passes = 0
        for n in range(3):
            info = g.Step(state, dt, 2, load * n / 10, load * (n + 1) / 10)
            assert info.converged == 1
            passes += info.iterations
        results[precision] = (g.Surface(0), g.Surface(2), passes)
    for comp in (0, 1):
        assert rel(results[1][comp], results[0][comp]) < TOL_MIXED
    assert results[1][2] * 3 <= results[0][2]


@pytest.mark.gpu
def test_mixed_warm_start_extrapolation_saves_correction_passes(gpu):
    # warm_start 1: the extrapolation 2 s_n - s_{n-1} starts the FP32
    # correction; same results (1e-8 against the oracle), fewer passes
    lmax = 12
    o, g0 = _pair(lmax, 20, 5, rms=1.0, ldelta=5, seed=5, precision=1, rtol=1e-10, max_iterations=60)
    _, g1 = _pair(lmax, 20, 5, rms=1.0, ldelta=5, seed=5, precision=1, rtol=1e-10, max_iterations=60,
                  warm_start=1)
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    s0, s1 = g0.ZeroState(), g1.ZeroState()
    saved = 0
    for n in range(5):
        l0, l1 = load * n / 10, load * (n + 1) / 10
        io = o.step(dt, 2, l0, l1)
        i0 = g0.Step(s0, dt, 2, l0, l1)
        i1 = g1.Step(s1, dt, 2, l0, l1)
        assert io.converged == i0.converged == i1.converged == 1
        for comp in (0, 2):
            assert rel(g1.Surface(comp), o.surface(comp)) < TOL_MIXED, (n, comp)
        if n >= 2:
            assert g1.start_taken
            saved += i0.correction_passes - i1.correction_passes
    assert saved > 0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_fp64_contractions_emulated_on_the_tensor_cores_keep_the_bar(gpu, precision):
    # fp64_emulation 1: the FP64 passes' Legendre contractions from exact
    # BF16 slice products; the steps still meet the oracle at the form's bar
    # (1e-10 FP64, 1e-8 mixed) with the oracle's pass counts or fewer
    lmax = 12
    tol = 1e-10 if precision == 0 else TOL_MIXED
    o, g = _pair(lmax, 20, 5, rms=1.0, ldelta=5, seed=5, precision=precision, rtol=1e-10, max_iterations=60,
                 fp64_emulation=1, warm_start=1)
    load = cap_load(lmax, o.sigma_scale, 2000.0)
    dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
    state = g.ZeroState()
    for n in range(4):
        l0, l1 = load * n / 10, load * (n + 1) / 10
        io = o.step(dt, 2, l0, l1)
        ig = g.Step(state, dt, 2, l0, l1)
        assert io.converged == ig.converged == 1
        for comp in (0, 2):
            assert rel(g.Surface(comp), o.surface(comp)) < tol, (n, comp)


@pytest.mark.gpu
@pytest.mark.parametrize("memory,rate", [(10, 0.5), (5, 0.0)])
def test_correction_loop_on_the_device_is_the_host_loop(gpu, monkeypatch, memory, rate):
    """The FP32 correction's loop run as a CUDA graph (a while node whose
    body is one pass and the device's decision) takes the host loop's
    decisions on the same numbers: the same passes, the same changes, the
    same results, bit for bit -- adaptive mixing (rate 0.5) and mixing from
    the start (rate 0)."""
    from sl3dpp_gb300 import _lib

    lmax = 12
    runs = {}
    for graphs in (True, False):
        if graphs:
            monkeypatch.delenv("SL3DGPU_NO_GRAPHS", raising=False)
        else:
            monkeypatch.setenv("SL3DGPU_NO_GRAPHS", "1")
        o, g = _pair(lmax, 20, 5, rms=1.0, ldelta=5, seed=5, precision=1, rtol=1e-10, max_iterations=60,
                     correction_memory=memory, anderson_rate=rate)
        load = cap_load(lmax, o.sigma_scale, 2000.0)
        dt = 500 * configs.SECONDS_PER_YEAR / o.time_scale
        state = g.ZeroState()
        before = _lib.lib().sl3dgpu_launch_count()
        out = []
        for n in range(3):
            info = g.Step(state, dt, 2, load * n / 10, load * (n + 1) / 10)
            assert info.converged == 1
            out.append((info.iterations, info.correction_passes, g.correction_history(), g.Surface(0), g.Surface(2)))
        runs[graphs] = (out, _lib.lib().sl3dgpu_launch_count() - before)
    for (a, b) in zip(runs[True][0], runs[False][0]):
        assert a[0] == b[0] and a[1] == b[1]
        assert np.array_equal(a[2], b[2])
        assert np.array_equal(a[3], b[3]) and np.array_equal(a[4], b[4])
    # the graph's kernels are counted as launched
    assert runs[True][1] > 0.8 * runs[False][1]
