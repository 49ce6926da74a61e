"""An ensemble of independent 3D evolutions run at once (the reference's
fourth workload: the members of a calibration or a line search, each an
Evolution3D run with its own lateral viscosity and ice history).

Each member is a `Viscoelastic3D` operator with its own state and CUDA
stream; `Ensemble.run` hands all members to `sl3dgpu_v3d_run_many`, whose
native thread pool drives them concurrently so that the small members'
kernels overlap on the GPU; `autotune` chooses the pool's queue order
(longest member first) and its size (the members in flight) by measuring
them. `Ensemble.run_sequential` runs them one after
another through the same per-member entry point (the comparison, and the
parity check: both give the same snapshots).

Members (`ensemble_members`, seeded): lmax drawn uniformly from
{32, 64, 96, 128}; delta RMS uniform in [0.3, 1.5] with L_delta = lmax / 4
between 100 and 670 km depth; an ice cap of half-angle uniform in [5, 20]
degrees ramping to 2 km over 10 steps of 500 years; 20 Sdirk2 steps. The
radial mesh follows lmax: 40 elements at lmax 32 growing linearly to 80 at
lmax 128 (the first two workloads' meshes), GLL order 4.
"""

from __future__ import annotations

import ctypes
import time

import numpy as np

from . import configs
from ._lib import check, lib
from .viscoelastic3d import SCHEMES, Options, StepInfo, Viscoelastic3D, standard_earth

LMAX_CHOICES = (32, 64, 96, 128)
RAMP_STEPS = 10
DT_YEARS = 500.0
THICKNESS = 2000.0


def elements_for(lmax: int) -> int:
    return int(round(40 + (lmax - 32) * 40 / 96))


def ensemble_members(count: int = 48, seed: int = 4, steps: int = 20, lmax_choices=LMAX_CHOICES) -> list[dict]:
    """The members' parameters, drawn from numpy's default_rng(seed)."""
    rng = np.random.default_rng(seed)
    members = []
    for i in range(count):
        lmax = int(rng.choice(lmax_choices))
        members.append({"lmax": lmax, "elements": elements_for(lmax), "ngll": 5,
                        "rms": float(rng.uniform(0.3, 1.5)), "ldelta": max(1, lmax // 4),
                        "cap_degrees": float(rng.uniform(5.0, 20.0)), "delta_seed": 1000 * seed + i,
                        "steps": steps})
    return members


class Ensemble:
    """The members' operators, delta fields and load histories, built once."""

    def __init__(self, members: list[dict], precision: int = 1, scheme: str = "sdirk2", **options):
        import torch

        from .grid import SurfaceGrid

        device = torch.device("cuda", torch.cuda.current_device())
        self.members = members
        self.scheme = SCHEMES[scheme]
        self.ops, self.times, self.loads = [], [], []
        for m in members:
            lmax = m["lmax"]
            opts = dict(rtol=1e-10, max_iterations=60, precision=precision, warm_start=1 if precision == 1 else 0,
                        fp64_emulation=1 if precision == 1 else 0)
            opts.update(options)
            op = Viscoelastic3D(standard_earth(m["elements"]), Options.defaults(lmax, m["ngll"], **opts))
            grid = SurfaceGrid(lmax, 0, op.options.oversampling)
            c = configs.delta_coefficients(lmax, m["ldelta"], m["rms"], m["delta_seed"])
            pattern = grid.SynthesiseBatch(torch.tensor(c, device=device), 1)
            ind = torch.tensor(configs.delta_indicator(op.radius), device=device)
            op.set_delta((ind[:, None] * pattern[None, :]).contiguous().view(-1))
            exact = SurfaceGrid(lmax, 0, 1.0)
            cap = configs.cap_field(exact.theta, exact.nphi, m["cap_degrees"], THICKNESS)
            full = (exact.ExpandBatch(torch.tensor(cap, device=device), 1) / op.surface_density_scale).cpu().numpy()
            dt = DT_YEARS * configs.SECONDS_PER_YEAR / op.time_scale
            nodes = m["steps"] + 1
            self.times.append(np.arange(nodes, dtype=np.float64) * dt)
            ramp = np.minimum(np.arange(nodes), RAMP_STEPS) / RAMP_STEPS
            self.loads.append(np.ascontiguousarray(ramp[:, None] * full[None, :], dtype=np.complex128))
            self.ops.append(op)

    def _outputs(self):
        U = [np.zeros_like(ld) for ld in self.loads]
        phi = [np.zeros_like(ld) for ld in self.loads]
        infos = [(StepInfo * t.size)() for t in self.times]
        return U, phi, infos

    def run(self, threads: int = 0, steps: int | None = None, order=None) -> dict:
        """Every member from a zero state, concurrently (the first `steps`
        steps of each, all by default), the pool taking the members in
        `order` (a permutation, index order by default); wall-clock seconds.
        Outputs stay in member order."""
        n = len(self.ops)
        order = list(range(n)) if order is None else list(order)
        if sorted(order) != list(range(n)):
            raise ValueError("order is a permutation of the members")
        states = [op.ZeroState() for op in self.ops]
        U, phi, infos = self._outputs()
        P = ctypes.c_void_p
        ops = (P * n)(*[self.ops[k]._h.value for k in order])
        sts = (P * n)(*[states[k]._h.value for k in order])
        times = (P * n)(*[self.times[k].ctypes.data for k in order])
        nodes = (ctypes.c_int * n)(*[self.times[k].size if steps is None else min(self.times[k].size, steps + 1)
                                     for k in order])
        loads = (P * n)(*[self.loads[k].ctypes.data for k in order])
        us = (P * n)(*[U[k].ctypes.data for k in order])
        ps = (P * n)(*[phi[k].ctypes.data for k in order])
        inf = (P * n)(*[ctypes.cast(infos[k], P).value for k in order])
        statuses = (ctypes.c_int * n)()
        t0 = time.perf_counter()
        check(lib().sl3dgpu_v3d_run_many(n, ops, sts, times, nodes, self.scheme, loads, us, ps, inf, threads,
                                         statuses))
        wall = time.perf_counter() - t0
        return {"U": U, "phi": phi, "infos": [[i[k] for k in range(len(i))] for i in infos], "seconds": wall,
                "states": states}

    def run_sequential(self) -> dict:
        """The same runs one after another (sl3dgpu_v3d_run per member)."""
        states = [op.ZeroState() for op in self.ops]
        U, phi, infos = self._outputs()
        t0 = time.perf_counter()
        for k, op in enumerate(self.ops):
            check(lib().sl3dgpu_v3d_run(op._h, states[k]._h, self.times[k].ctypes.data_as(ctypes.POINTER(
                ctypes.c_double)), self.times[k].size, self.scheme, self.loads[k].ctypes.data, U[k].ctypes.data,
                phi[k].ctypes.data, infos[k]))
        wall = time.perf_counter() - t0
        return {"U": U, "phi": phi, "infos": [[i[k] for k in range(len(i))] for i in infos], "seconds": wall,
                "states": states}

    def member_steps(self, steps: int | None = None) -> int:
        return sum(t.size - 1 if steps is None else min(t.size - 1, steps) for t in self.times)

    def member_seconds(self, steps: int = 1) -> list[float]:
        """Each member's first `steps` steps run alone (node 0 and the steps),
        wall-clock seconds: the schedule's cost model."""
        out = []
        for k, op in enumerate(self.ops):
            state = op.ZeroState()
            U = np.zeros((steps + 1, self.loads[k].shape[1]), dtype=np.complex128)
            phi = np.zeros_like(U)
            infos = (StepInfo * (steps + 1))()
            t0 = time.perf_counter()
            check(lib().sl3dgpu_v3d_run(op._h, state._h, self.times[k].ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                        steps + 1, self.scheme, self.loads[k].ctypes.data, U.ctypes.data,
                                        phi.ctypes.data, infos))
            out.append(time.perf_counter() - t0)
        return out


def autotune(ens: Ensemble, probe_steps: int = 2, thread_choices=None) -> dict:
    """The ensemble's queue schedule and concurrency, chosen by measurement.

    The members' costs are measured (each member's first step alone), the
    queue ordered longest first (the pool then ends with the short members,
    which fill the GPU's gaps -- LPT scheduling), and each candidate number of
    concurrent members (host threads, one member each) timed over the first
    `probe_steps` steps of the whole ensemble in that order; the fastest is
    kept. Returns the order, the threads, and every measurement."""
    n = len(ens.ops)
    cost = ens.member_seconds(1)
    order = sorted(range(n), key=lambda k: -cost[k])
    if thread_choices is None:
        thread_choices = sorted({max(1, n // 8), max(1, n // 4), max(1, n // 2), n})
    timings = {}
    for threads in thread_choices:
        r = ens.run(threads=threads, steps=probe_steps, order=order)
        timings[threads] = r["seconds"]
    best = min(timings, key=timings.get)
    return {"order": order, "threads": best, "probe_seconds": timings, "member_seconds": cost,
            "probe_steps": probe_steps}
