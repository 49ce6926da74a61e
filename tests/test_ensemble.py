"""The ensemble workload: independent 3D evolutions run at once through
sl3dgpu_v3d_run_many (a native thread pool, one stream per member). The
concurrent run gives the members the snapshots the one-by-one run gives."""

import numpy as np
import pytest

from sl3dpp_gb300.ensemble import LMAX_CHOICES, elements_for, ensemble_members


def test_members_are_seeded_and_in_range():
    a, b = ensemble_members(48, seed=4), ensemble_members(48, seed=4)
    assert a == b and ensemble_members(48, seed=5) != a
    assert {m["lmax"] for m in a} <= set(LMAX_CHOICES) and len({m["lmax"] for m in a}) == 4
    for m in a:
        assert 0.3 <= m["rms"] <= 1.5 and 5.0 <= m["cap_degrees"] <= 20.0
        assert m["ldelta"] == m["lmax"] // 4 and m["steps"] == 20
        assert m["elements"] == elements_for(m["lmax"])
    assert elements_for(32) == 40 and elements_for(128) == 80


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_concurrent_members_match_their_one_by_one_runs(gpu, precision):
    from sl3dpp_gb300.ensemble import Ensemble

    members = ensemble_members(5, seed=7, steps=3, lmax_choices=(8, 12))
    for m in members:
        m["elements"] = 20
    ens = Ensemble(members, precision=precision)
    together = ens.run(threads=3)
    alone = ens.run_sequential()
    for k in range(len(members)):
        for key in ("U", "phi"):
            a, b = together[key][k], alone[key][k]
            assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b)), (k, key)
        # the same passes and verdicts, step for step
        assert [(i.iterations, i.converged) for i in together["infos"][k]] == \
               [(i.iterations, i.converged) for i in alone["infos"][k]], k
    assert ens.member_steps() == 15


@pytest.mark.gpu
def test_run_many_refuses_shared_operators(gpu):
    import ctypes

    from sl3dpp_gb300 import _lib
    from sl3dpp_gb300.ensemble import Ensemble

    ens = Ensemble(ensemble_members(1, seed=3, steps=1, lmax_choices=(8,)), precision=0)
    op = ens.ops[0]
    s1, s2 = op.ZeroState(), op.ZeroState()
    P = ctypes.c_void_p
    t = ens.times[0]
    st = (ctypes.c_int * 2)()
    code = _lib.lib().sl3dgpu_v3d_run_many(2, (P * 2)(op._h.value, op._h.value), (P * 2)(s1._h.value, s2._h.value),
                                           (P * 2)(t.ctypes.data, t.ctypes.data), (ctypes.c_int * 2)(t.size, t.size),
                                           2, (P * 2)(ens.loads[0].ctypes.data, ens.loads[0].ctypes.data),
                                           None, None, None, 0, st)
    assert code == _lib.ERR_ARGUMENT and b"distinct" in _lib.lib().sl3dgpu_last_error()


@pytest.mark.gpu
def test_autotuned_schedule_runs_longest_first_and_keeps_the_results(gpu):
    """The autotuner's queue order puts the costlier members first and its
    chosen concurrency is one it measured; a run in that order gives every
    member the one-by-one run's snapshots (outputs stay in member order)."""
    from sl3dpp_gb300.ensemble import Ensemble, autotune

    members = ensemble_members(6, seed=9, steps=2, lmax_choices=(8, 16))
    for m in members:
        m["elements"] = 20
    ens = Ensemble(members, precision=1)
    tune = autotune(ens, probe_steps=1, thread_choices=[1, 3, 6])
    cost = tune["member_seconds"]
    assert sorted(tune["order"]) == list(range(6))
    assert all(cost[a] >= cost[b] for a, b in zip(tune["order"], tune["order"][1:]))
    assert tune["threads"] in (1, 3, 6) and set(tune["probe_seconds"]) == {1, 3, 6}
    together = ens.run(threads=tune["threads"], order=tune["order"])
    alone = ens.run_sequential()
    for k in range(len(members)):
        for key in ("U", "phi"):
            a, b = together[key][k], alone[key][k]
            assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b)), (k, key)
