"""Benchmark: 3D viscoelastic steps per second on GB300.

One step is one Sdirk2 step (two backward Euler stages, each closed by the
within-step fixed point, Picard then Anderson, to the tolerance) of the 3D
quasi-static operator at lmax 256: 120 radial elements of order 5, the
configurations' layered Earth (Maxwell mantle, 100 km elastic lid), delta a
seeded random spherical-harmonic field to degree 64 with RMS 1.0 between 100
and 670 km depth, and a 15-degree polar ice cap growing to 2 km over 10 steps
of 500 yr. All inputs are synthetic (numpy default_rng, seeds below).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). `value` is steps/s of the mixed form (FP64
passes and stopping rule, FP32 corrections between them; each step starts
from the previous step's strain and its corrections from the extrapolation of
the last two steps) with the load coefficients
resident in device memory, timed with CUDA events on the operator's stream;
`e2e` is the same through the C ABI with the loads copied from pinned host
memory and the surface U and phi read back every step. The plain FP64 form
then runs the same step sequence: its steps/s (`fp64_gpu`), and the mixed
form's relative error against it on U and phi at every end-to-end step
(`rel_err_vs_fp64`; the FP64 form matches the FP64 oracle to 1e-10 in the
tests). `--precision fp64` makes the FP64 form the headline. `--impl
reference` times the CPU restatement of the reference's path (oracle/,
OpenMP on every host core) on a bounded sample of the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import pathlib
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

LMAX = 256
ELEMENTS = 120
NGLL = 6
LDELTA = 64
DELTA_RMS = 1.0
DELTA_SEED = 1
CAP_DEGREES = 15.0
CAP_THICKNESS = 2000.0
RAMP_STEPS = 10
DT_YEARS = 500.0
RTOL = 1e-10
MAX_ITERATIONS = 60
CORRECTION_RTOL = 3e-6
CORRECTION_MEMORY = 10
METRIC = "3D steps/sec at lmax=256: mixed+warm-start vs plain FP64 GPU at rel err <=1e-8"
# The FP64 fixed point's passes per step at this workload (both stages), as
# this script's plain FP64 GPU arm measured it on a GB300 (86.0 a step over
# the 20 timed steps; the CPU oracle runs the same iterate sequence, pinned
# pass for pass against the GPU). The reference arm, which runs without a
# GPU, extrapolates its CPU sample to a step with it; the GPU arm's own line
# uses the count it measures.
PASSES_PER_STEP = 86


def _rescale(lmax):
    """A smaller workload of the same shape (development runs only)."""
    global LMAX, ELEMENTS, LDELTA
    LMAX = lmax
    ELEMENTS = max(20, int(round(120 * lmax / 256)))
    LDELTA = max(2, lmax // 4)


def workload_config(precision="mixed"):
    return {"workload": f"3d_step_lmax{LMAX}_{precision}_sdirk2", "lmax": LMAX, "elements": ELEMENTS,
            "order": NGLL - 1, "delta_degree": LDELTA, "delta_rms": DELTA_RMS, "delta_seed": DELTA_SEED,
            "rheology": "maxwell", "cap_degrees": CAP_DEGREES, "cap_thickness_m": CAP_THICKNESS,
            "dt_years": DT_YEARS, "scheme": "sdirk2", "rtol": RTOL, "max_iterations": MAX_ITERATIONS,
            "anderson_memory": 5, "oversampling": 1.5, "precision": precision,
            "correction_rtol": CORRECTION_RTOL if precision == "mixed" else None,
            "correction_memory": CORRECTION_MEMORY if precision == "mixed" else None,
            "warm_start": ("the previous step's strain, and the extrapolation 2 s_n - s_{n-1} of the last two "
                           "steps as the FP32 correction's start" if precision == "mixed" else
                           "the previous step's strain coefficients (the reference's plain warm start)"),
            "fp64_contractions": ("the FP64 passes' Legendre contractions emulated on the tensor cores: 7 BF16 "
                                  "slices a value under power-of-two row/column scales, exact FP32 slice products, "
                                  "levels joined in FP64 (about 49 bits)" if precision == "mixed" else
                                  "FP64 units"),
            "fp64_ring_transforms": ("the FP64 passes' ring FFTs in double-float on the FP32 pipe (hi + lo FP32 "
                                     "pairs, about 48 bits)" if precision == "mixed" else "FP64 units"),
            "l2": "working set far above L2 (memory tensors ~3.3 GB per array)",
            "parallelism": "replicas (one independent operator per GPU)"}


def load_ramp(full, step):
    return full * min(step, RAMP_STEPS) / RAMP_STEPS


# -- clocks ----------------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for name, flag in zip(names, f[5:9]):
                if flag.lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# -- the GPU arm --------------------------------------------------------------------------------

KIND_NAMES = ["legendre_synthesis", "legendre_analysis", "ring_fft", "force_assembly", "strain_recovery",
              "band_solve", "streaming", "anderson", "other", "legendre_f32", "ring_fft_f32", "band_solve_f32",
              "legendre_f64_tc"]


def profile_read():
    import ctypes

    from sl3dpp_gb300._lib import lib

    out = {}
    for k, name in enumerate(KIND_NAMES):
        ms, n, fl, by = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
        lib().sl3dgpu_profile_read(k, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(fl), ctypes.byref(by))
        out[name] = {"ms": ms.value, "launches": n.value, "flops": fl.value, "bytes": by.value}
    return out


def measured_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        return json.loads(path.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# The committed ncu summary holding a kernel kind's DRAM bytes per launch.
TRAFFIC_PROFILES = {"ring_fft": "ring_fft_df_3d_step_lmax256.md", "legendre_f32": "tcgemm_3d_step_lmax256_traffic.md"}


def ncu_traffic(kernel: str):
    """DRAM bytes per launch from the committed ncu summary of a kernel, if any."""
    path = ROOT / "profiles" / TRAFFIC_PROFILES.get(kernel, f"{kernel}.md")
    if not path.exists():
        return None
    for line in path.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def build_operator(device, precision, emulation=None):
    import torch

    from sl3dpp_gb300 import configs
    from sl3dpp_gb300.grid import SurfaceGrid
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    op = Viscoelastic3D(standard_earth(ELEMENTS),
                        Options.defaults(LMAX, NGLL, rtol=RTOL, max_iterations=MAX_ITERATIONS,
                                         precision=1 if precision == "mixed" else 0,
                                         correction_rtol=CORRECTION_RTOL, correction_memory=CORRECTION_MEMORY,
                                         warm_start=1 if precision == "mixed" else 0,
                                         fp64_emulation=(1 if precision == "mixed" else 0) if emulation is None
                                         else emulation))
    grid = SurfaceGrid(LMAX, 0, 1.5)
    c = configs.delta_coefficients(LMAX, LDELTA, DELTA_RMS, DELTA_SEED)
    pattern = grid.SynthesiseBatch(torch.tensor(c, device=device), 1)
    ind = torch.tensor(configs.delta_indicator(op.radius), device=device)
    op.set_delta((ind[:, None] * pattern[None, :]).contiguous().view(-1))
    exact = SurfaceGrid(LMAX, 0, 1.0)
    cap = configs.cap_field(exact.theta, exact.nphi, CAP_DEGREES, CAP_THICKNESS)
    full = exact.ExpandBatch(torch.tensor(cap, device=device), 1) / op.surface_density_scale
    dt = DT_YEARS * configs.SECONDS_PER_YEAR / op.time_scale
    return op, full, dt


def max_over_ranks(values, device=None):
    """The largest of each value over the ranks (the slowest rank's times):
    an all-reduce MAX over the process group (on the device under NCCL, on
    the host under gloo); the values themselves with one rank."""
    import torch

    dist = torch.distributed
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    on = device if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=on)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu().tolist()]


def aggregate_rate(steps_per_rank: int, world: int, seconds: float) -> float:
    """Whole-job steps/s: every rank's steps (replicas of the workload, the
    weak-scaling form) over the slowest rank's time."""
    return steps_per_rank * world / seconds


def gpu_arm(args, rank, world, device, precision, emulation=None, e2e=True, profile_apart=True):
    """Steps W .. W + K - 1 of the workload, from the same warmed start each
    time: timed with the loads resident in device memory (CUDA events on the
    operator's stream; each step's surface U and phi copied into device
    buffers, stream-ordered, for the error comparison); with profile_apart,
    once more with the per-kernel timing events on, for the breakdown (else
    the timed run carries them); then end to end through the C ABI with the
    loads copied from pinned host memory and U and phi read back every step
    (host wall clock). The state is rebuilt by the same W warm-up steps
    before each run."""
    import torch

    from sl3dpp_gb300._lib import lib

    t_setup = time.time()
    op, full, dt = build_operator(device, precision, emulation)
    torch.cuda.synchronize()
    setup_s = time.time() - t_setup
    loads = [load_ramp(full, n).contiguous() for n in range(args.warmup + args.steps + 1)]
    lm = full.numel()
    surfaces_dev = torch.zeros((args.steps, 2, lm), dtype=torch.complex128, device=device)

    def warm_state():
        state = op.ZeroState()
        for n in range(args.warmup):
            op.StepDevice(state, dt, "sdirk2", loads[n], loads[n + 1])
        return state

    state = warm_state()
    stream = torch.cuda.ExternalStream(op.stream, device=device)
    lib().sl3dgpu_profile_reset()
    lib().sl3dgpu_profile_enable(0 if profile_apart else 1)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = lib().sl3dgpu_launch_count()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    passes = corrections = 0
    infos = []
    with ClockSampler(torch.cuda.current_device()) as clocks:
        start.record(stream)
        for k in range(args.steps):
            n = args.warmup + k
            info = op.StepDevice(state, dt, "sdirk2", loads[n], loads[n + 1])
            op.SurfaceDevice("U", surfaces_dev[k, 0])
            op.SurfaceDevice("phi", surfaces_dev[k, 1])
            passes += info.iterations
            corrections += info.correction_passes
            infos.append(info)
        stop.record(stream)
        stop.synchronize()
    torch.cuda.synchronize()
    launches = lib().sl3dgpu_launch_count() - launches0
    history = {"fp64_pass_residuals": [float(f"{v:.3e}") for v in op.residual_history()],
               "correction_passes": int(op.correction_history().size)}
    lib().sl3dgpu_profile_enable(0)
    ms = start.elapsed_time(stop)
    surfaces = surfaces_dev.cpu().numpy()
    del state
    if profile_apart:
        # the per-kind breakdown from the same steps run again with the
        # kernel timing events on (they cost a few per cent of a step)
        state = warm_state()
        lib().sl3dgpu_profile_reset()
        lib().sl3dgpu_profile_enable(1)
        for k in range(args.steps):
            n = args.warmup + k
            op.StepDevice(state, dt, "sdirk2", loads[n], loads[n + 1])
        torch.cuda.synchronize()
        lib().sl3dgpu_profile_enable(0)
        del state
    prof = profile_read()
    e2e_s = float("nan")
    if e2e:
        host_loads = [l.cpu().pin_memory().numpy() for l in loads]
        state = warm_state()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for k in range(args.steps):
            n = args.warmup + k
            op.Step(state, dt, "sdirk2", host_loads[n], host_loads[n + 1])
            U = op.Surface("U")
            phi = op.Surface("phi")
            if not (np.all(np.isfinite(U)) and np.all(np.isfinite(phi))):
                raise RuntimeError(f"non-finite surface at end-to-end step {n}")
        e2e_s = time.perf_counter() - t0
        del state
    seconds, e2e_seconds = max_over_ranks([ms / 1e3, e2e_s], device)
    return {"op": op, "seconds": seconds, "e2e_seconds": e2e_seconds, "passes": passes,
            "corrections": corrections, "surfaces": surfaces, "history": history,
            "infos": infos, "profile": prof, "launches": launches, "clocks": clocks.summary(),
            "setup_s": setup_s, "load_bytes": int(full.numel() * 16)}


def roofline(prof, fp64_gflops, fp32_gflops, double_float_rings=False):
    """The dominant kernel kind against the bound of its work: the FP64
    Legendre GEMM, the FP64 ring FFTs and band solves against the FP64 FMA throughput
    measured live, the emulated FP64 contraction against the measured BF16
    tensor rate (algorithmic FP64 flops), the rest -- the 3xTF32 contraction
    streaming its table panels included -- against the measured HBM copy
    bandwidth with their algorithmic bytes. Under FP64 emulation the FP64
    rings' transforms run in double-float on the FP32 pipe: their nominal
    FFT flops are then FP64-equivalent work, still set against the FP64
    FMA rate they replace (a fraction above 1 is possible), and said so."""
    kind = max(prof, key=lambda k: prof[k]["ms"])
    p = prof[kind]
    peaks, source = measured_peaks()
    per_launch_s = p["ms"] / 1e3 / max(p["launches"], 1)
    share = p["ms"] / sum(v["ms"] for v in prof.values())
    flops_bound = {"legendre_synthesis": ("fp64", fp64_gflops / 1e3), "legendre_analysis": ("fp64", fp64_gflops / 1e3),
                   "ring_fft": ("fp64", fp64_gflops / 1e3), "band_solve": ("fp64", fp64_gflops / 1e3),
                   "legendre_f64_tc": ("tensor", peaks["bf16_tflops"])}
    if p["flops"] > 0 and kind in flops_bound:
        bound, peak = flops_bound[kind]
        achieved = p["flops"] / max(p["launches"], 1) / per_launch_s / 1e12
        peak_source = (source + " (dense BF16; the 28 slice products a step are not counted)" if bound == "tensor"
                       else "FP64 FMA throughput measured live by sl3dgpu_fp64_fma_peak (CUDA-core arithmetic: "
                            "MEASURED_PEAKS.json holds HBM and bf16 tensor figures only)")
        if kind == "ring_fft" and double_float_rings:
            bound = "fp64-equivalent"
            peak_source += ("; the transforms run in double-float on the FP32 pipe, their nominal 5 n log2 n FP64 "
                            "flops set against the FP64 rate they replace")
        return {"kernel": kind, "bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": ncu_traffic(kind), "peak_source": peak_source,
                "share_of_timed": share}
    achieved = p["bytes"] / max(p["launches"], 1) / per_launch_s / 1e9
    return {"kernel": kind, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / peaks["hbm_gbs"], "traffic": ncu_traffic(kind), "peak_source": source,
            "share_of_timed": share}


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


# -- the CPU restatement (oracle), a bounded sample --------------------------------------------

class CpuSampler:
    """The oracle (FP64 C++ + OpenMP, every host core) at the same workload:
    a backward Euler stage's start timed once and passes timed one by one
    (the Sdirk2 first stage's length and loads), each pass extrapolated to a
    step of two stage starts and passes_per_step passes -- an extrapolation,
    not a timed step, and labelled so."""

    def __init__(self):
        from sl3dpp_gb300 import configs
        from tests import _oracle as O  # the checker, as the CPU baseline

        t0 = time.time()
        self.O = O
        self.st = O.OracleStep(O.standard_earth(ELEMENTS),
                               O.default_options(LMAX, NGLL, rtol=RTOL, max_iterations=MAX_ITERATIONS))
        c = configs.delta_coefficients(LMAX, LDELTA, DELTA_RMS, DELTA_SEED)
        pattern = O.synthesise_real(LMAX, self.st.theta, self.st.nphi, c)
        self.st.set_delta(configs.delta_samples(pattern, self.st.radius))
        theta, w, nphi = O.grid(LMAX, 1.0)
        full = O.expand_real(LMAX, theta, w, nphi, configs.cap_field(theta, nphi, CAP_DEGREES, CAP_THICKNESS))
        self.full = full / self.st.sigma_scale
        self.dt = DT_YEARS * configs.SECONDS_PER_YEAR / self.st.time_scale
        self.setup = time.time() - t0
        self.threads = O.load().oracle_threads()

    def sample(self, passes_per_step, sample_passes=1, source="measured by the GPU arm of this run"):
        t_start, each = self.st.sample(0.29289321881345247560 * self.dt, sample_passes, 0.5 * self.full,
                                       0.6 * self.full)
        step_s = [2 * t_start + passes_per_step * t for t in each]
        value = 1.0 / float(np.median(step_s))
        return {"value": value, "unit": "steps/s", "cores": self.threads, "kind": "port", "extrapolated": True,
                "sample": (f"one backward Euler stage start ({t_start:.1f} s) and {sample_passes} pass(es) "
                           f"(median {float(np.median(each)):.2f} s) of the same lmax-{LMAX} workload, extrapolated "
                           f"to a step of two stages and {passes_per_step:.1f} passes ({source}); construction "
                           f"{self.setup:.0f} s untimed"),
                "step_seconds": step_s, "start_seconds": t_start, "pass_seconds": [float(t) for t in each]}


def config1_cpu_run():
    """The first configuration as a whole, timed, on the CPU oracle: lmax 32,
    40 elements of order 4, delta to degree 8 at RMS 0.5, the 15 degree cap
    ramping to 2 km over 10 Sdirk2 steps of 500 yr, rtol 1e-10 -- every pass
    of every step (no extrapolation)."""
    from sl3dpp_gb300 import configs
    from tests import _oracle as O

    lmax = 32
    st = O.OracleStep(O.standard_earth(40), O.default_options(lmax, 5, rtol=1e-10, max_iterations=MAX_ITERATIONS))
    c = configs.delta_coefficients(lmax, 8, 0.5, DELTA_SEED)
    st.set_delta(configs.delta_samples(O.synthesise_real(lmax, st.theta, st.nphi, c), st.radius))
    theta, w, nphi = O.grid(lmax, 1.0)
    full = O.expand_real(lmax, theta, w, nphi, configs.cap_field(theta, nphi, CAP_DEGREES, CAP_THICKNESS))
    full = full / st.sigma_scale
    dt = DT_YEARS * configs.SECONDS_PER_YEAR / st.time_scale
    passes = 0
    t0 = time.perf_counter()
    for n in range(10):
        info = st.step(dt, 2, full * n / 10, full * (n + 1) / 10)
        passes += info.iterations
    seconds = time.perf_counter() - t0
    return {"workload": "config 1: lmax 32, 40 elements of order 4, Maxwell, delta degree 8 RMS 0.5, 10 Sdirk2 "
                        "steps of 500 yr, rtol 1e-10 (every step run in full)",
            "value": 10.0 / seconds, "unit": "steps/s", "seconds": seconds, "passes_per_step": passes / 10,
            "cores": O.load().oracle_threads(), "kind": "port", "extrapolated": False}


# -- the Legendre contraction alone -------------------------------------------------------------

def legendre_case(args, device):
    """The mixed form's correction contraction alone at the workload's size:
    the 3xTF32 tensor-core Legendre analysis and synthesis of spin -2 over
    the 55 lateral nodes of the lmax-256 grid (FP32 device buffers, random
    values), timed with CUDA events -- the case a single-kernel profile of
    TcGemmKernel runs (a few hundred MB on the device)."""
    import ctypes

    import torch

    from sl3dpp_gb300._lib import lib
    from sl3dpp_gb300.grid import SurfaceGrid

    count, N = 55, -2
    g = SurfaceGrid(LMAX, 2, 1.5)
    rows = (LMAX + 1) ** 2 - N * N
    gen = torch.Generator(device=device).manual_seed(5)
    coeffs = torch.randn(rows * count * 2, dtype=torch.float32, device=device, generator=gen)
    spectra = torch.randn((2 * LMAX + 1) * g.ntheta * count * 2, dtype=torch.float32, device=device, generator=gen)
    out_c = torch.empty_like(coeffs)
    out_s = torch.empty_like(spectra)
    stream = torch.cuda.current_stream().cuda_stream

    def once():
        lib().sl3dgpu_legendre_device(g._handle, N, 0, 1, 1, ctypes.c_void_p(spectra.data_ptr()), count,
                                      ctypes.c_void_p(out_c.data_ptr()), ctypes.c_void_p(stream))
        lib().sl3dgpu_legendre_device(g._handle, N, 0, 0, 1, ctypes.c_void_p(coeffs.data_ptr()), count,
                                      ctypes.c_void_p(out_s.data_ptr()), ctypes.c_void_p(stream))

    for _ in range(args.warmup):
        once()
    torch.cuda.synchronize()
    lib().sl3dgpu_profile_reset()
    lib().sl3dgpu_profile_enable(1)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(args.steps):
        once()
    stop.record()
    stop.synchronize()
    lib().sl3dgpu_profile_enable(0)
    prof = profile_read()["legendre_f32"]
    ms = start.elapsed_time(stop)
    flops = prof["flops"] / max(prof["launches"], 1)
    per_launch = prof["ms"] / max(prof["launches"], 1)
    return {"case": f"legendre_f32 spin -2, lmax {LMAX}, {count} nodes, analysis + synthesis",
            "ms_per_pair": ms / args.steps, "launches": prof["launches"], "ms_per_launch": per_launch,
            "algorithmic_tflops": flops / (per_launch / 1e3) / 1e12 if per_launch > 0 else None}


# -- the learned warm start ----------------------------------------------------------------------

def warmstart_case(args):
    """Config 5, bounded: held-out delta fields (degree 32, RMS 1.0; seeds
    outside the training runs') at lmax 128 (80 elements of order 5), 16
    Sdirk2 steps each, with and without the committed network -- the plain
    FP64 form against its own start (the previous step's strain), the mixed
    form against its extrapolated start; passes a step, steps/s (host wall
    clock, synchronised each step) and the largest relative difference of
    the surface U between the two runs."""
    from sl3dpp_gb300 import warmstart as W

    net = W.WarmStartNet.load(W.default_weights())
    out = {"case": "learned warm start, lmax 128, 80 elements of order 5, delta degree 32 RMS 1.0, 16 Sdirk2 "
                   "steps of 500 yr, held-out seeds 90001-90002",
           "parameters": net.parameter_count, "forms": {}}
    for name, precision in (("fp64", 0), ("mixed", 1)):
        rows = []
        for seed in (90_001, 90_002):
            kw = dict(seed=seed, steps=16, lmax=128, elements=80, ngll=6, rms=1.0, ldelta=32, precision=precision)
            plain, learned = W.evaluate(None, **kw), W.evaluate(net, **kw)
            err = max(float(np.max(np.abs(a - b)) / np.max(np.abs(b))) for a, b in zip(learned["U"], plain["U"]))
            work = (lambda r: [p + c for p, c in zip(r["passes"], r["corrections"])])
            rows.append({"seed": seed, "passes_plain": plain["passes"], "passes_learned": learned["passes"],
                         "correction_passes_plain": plain["corrections"],
                         "correction_passes_learned": learned["corrections"], "taken": sum(learned["taken"]),
                         "steps_per_s_plain": 16 / plain["seconds"], "steps_per_s_learned": 16 / learned["seconds"],
                         "total_passes_plain": sum(work(plain)), "total_passes_learned": sum(work(learned)),
                         "max_rel_diff_U": err})
        out["forms"][name] = rows
    return out


# -- config 2: the coupled step under an ocean -----------------------------------------------------

def ocean_case(args, device):
    """Config 2 on the GPU, lmax 128, 80 elements of order 5, Burgers
    (transient viscosity / 10, modulus ratio 0.5), delta to degree 32 at RMS
    1.0, an ocean with frozen shorelines over a land mask at 30% of the area
    (a seeded smooth field thresholded), axial rotational feedback, 50 Sdirk2
    steps of 250 yr under config 1's 15 degree cap growing to 2 km over the
    first 10 steps and held; every pass closed by the sea-level equation
    (rtol 1e-10). Node 0 is the instantaneous response. Two forms: the plain
    FP64 fixed point, and the mixed form (FP64 passes closed by the sea-level
    equation, FP32 corrections without the ocean's feedback, refined away by
    the FP64 passes; the Legendre contractions emulated on the tensor cores,
    the extrapolated warm start). Steps/s by CUDA events over the 50 steps
    (one synchronised step at a time, as the run's host decides each step's
    loads); passes, closure iterations, the final sea level's range, and
    the mixed form's largest relative difference from the FP64 form in the
    surface U and the sea level over the steps. Parity with the oracle at
    this shape is tests/test_ocean.py's."""
    import torch

    from sl3dpp_gb300 import configs
    from sl3dpp_gb300.grid import SurfaceGrid
    from sl3dpp_gb300.viscoelastic3d import Options, Viscoelastic3D, standard_earth

    lmax, elements, ngll, steps, years = 128, 80, 6, 50, 250.0

    def run(mixed):
        kw = dict(rtol=1e-10, max_iterations=120)
        if mixed:
            kw.update(precision=1, correction_rtol=CORRECTION_RTOL, correction_memory=CORRECTION_MEMORY,
                      warm_start=1, fp64_emulation=1)
        op = Viscoelastic3D(standard_earth(elements, 0.5, 10.0), Options.defaults(lmax, ngll, **kw))
        grid = SurfaceGrid(lmax, 0, 1.5)
        c = configs.delta_coefficients(lmax, 32, 1.0, 2)
        pattern = grid.SynthesiseBatch(torch.tensor(c, device=device), 1)
        ind = torch.tensor(configs.delta_indicator(op.radius), device=device)
        op.set_delta((ind[:, None] * pattern[None, :]).contiguous().view(-1))
        theta, w, nphi = op.ocean_grid()
        sle_grid = SurfaceGrid(lmax, 0, 1.0)
        land = sle_grid.SynthesiseBatch(torch.tensor(configs.land_field_coefficients(lmax, 11), device=device), 1)
        ocean = configs.ocean_from_field(land.cpu().numpy(), w, nphi, 0.3)
        op.set_ocean(ocean, rotation=1, rtol=1e-10, max_iterations=200, anderson_memory=5)
        cap = configs.cap_field(theta, nphi, CAP_DEGREES, CAP_THICKNESS) / op.surface_density_scale
        ice = lambda n: cap * min(n, 10) / 10.0
        dt = years * configs.SECONDS_PER_YEAR / op.time_scale
        state = op.ZeroState()
        op.StepOcean(state, 0.0, 2, ice(0), ice(0))
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        passes, corrections, closure_iterations, surfaces, ms = [], [], [], [], 0.0
        for n in range(1, steps + 1):
            torch.cuda.synchronize()
            start.record()
            info = op.StepOcean(state, dt, 2, ice(n - 1), ice(n))
            stop.record()
            stop.synchronize()
            ms += start.elapsed_time(stop)
            if not info.converged:
                raise RuntimeError(f"config 2: step {n} did not converge ({info.iterations} passes)")
            passes.append(info.iterations)
            corrections.append(info.correction_passes)
            slc_n, _, res = op.SeaLevel()
            closure_iterations.append(res.iterations)
            surfaces.append((op.Surface(0), slc_n))
        slc, omega, _ = op.SeaLevel()
        field = sle_grid.SynthesiseBatch(torch.tensor(slc, device=device), 1).cpu().numpy() * op.length_scale
        out = {"steps_per_s": steps / (ms / 1e3), "ms_per_step": ms / steps, "passes_per_step": float(np.mean(passes)),
               "passes": passes, "last_closure_iterations": closure_iterations[-1],
               "sea_level_range_m": [float(field.min()), float(field.max())],
               "axial_angular_velocity": float(omega[2] / op.time_scale)}
        if mixed:
            out["correction_passes_per_step"] = float(np.mean(corrections))
        return out, surfaces

    fp64, s64 = run(False)
    mixed, smx = run(True)
    mixed["max_rel_diff_vs_fp64"] = {
        "U": max(rel_err(a[0], b[0]) for a, b in zip(smx, s64)),
        "sea_level": max(rel_err(a[1], b[1]) for a, b in zip(smx, s64))}
    mixed["speedup_vs_fp64"] = mixed["steps_per_s"] / fp64["steps_per_s"]
    return {"case": "config 2: lmax 128, 80 elements of order 5, Burgers, delta degree 32 RMS 1.0, ocean with "
                    "frozen shorelines over 70% of the area, axial rotation, 50 Sdirk2 steps of 250 yr",
            **fp64, "mixed": mixed}


# -- the discrete adjoint ---------------------------------------------------------------------------

def adjoint_case(args, device):
    """The discrete 3D adjoint of the run without an ocean on the GPU, two
    workloads: config 1's (lmax 32, 40 elements of order 4, Maxwell, delta to
    degree 8 at RMS 0.5, FP64) and config 2's Earth without its ocean (lmax
    128, 80 elements of order 5, Burgers, delta to degree 32 at RMS 1.0, the
    mixed form); both under config 1's cap ramping to 2 km over 10 Sdirk2
    steps of 500 yr (11 nodes), rtol 1e-10, the objective a seeded pattern of
    U and one of phi read at every node with a weight growing in time. Per
    workload: the forward run's seconds (Evolution3D::Run), the adjoint
    call's (its own recorded forward run and the transposed sweep), the same
    with the record stride 3 and its largest relative gap from the first, the
    pairing identity's relative gap (the load kernels against the
    objective), and the log-viscosity gradient against Richardson-
    extrapolated central differences of the forward run along a seeded
    smooth direction over every node."""
    import torch

    from sl3dpp_gb300 import configs
    from sl3dpp_gb300.grid import SurfaceGrid
    from sl3dpp_gb300.viscoelastic3d import Evolution3D, Options, Viscoelastic3D, standard_earth

    def pairing(lmax, a, b):
        w = np.concatenate([[1.0] + [2.0] * l for l in range(lmax + 1)])
        return float(np.sum(w * (a * np.conj(b)).real))

    def real_coefficients(lmax, rng, count):
        lm = (lmax + 1) * (lmax + 2) // 2
        c = rng.standard_normal((count, lm)) + 1j * rng.standard_normal((count, lm))
        for l in range(lmax + 1):
            c[:, l * (l + 1) // 2] = c[:, l * (l + 1) // 2].real
        return c

    def workload(name, lmax, elements, ngll, kelvin, ldelta, rms, mixed):
        kw = dict(rtol=1e-10, max_iterations=120)
        if mixed:
            kw.update(precision=1, correction_rtol=CORRECTION_RTOL, correction_memory=CORRECTION_MEMORY,
                      fp64_emulation=1)
        op = Viscoelastic3D(standard_earth(elements, kelvin, 10.0), Options.defaults(lmax, ngll, **kw))
        grid = SurfaceGrid(lmax, 0, 1.5)
        pattern = grid.SynthesiseBatch(torch.tensor(configs.delta_coefficients(lmax, ldelta, rms, DELTA_SEED),
                                                    device=device), 1)
        ind = torch.tensor(configs.delta_indicator(op.radius), device=device)
        delta = (ind[:, None] * pattern[None, :]).contiguous().view(-1).cpu().numpy()
        op.set_delta(delta)
        sle = SurfaceGrid(lmax, 0, 1.0)
        theta, w, nphi = op.ocean_grid()
        cap = configs.cap_field(theta, nphi, CAP_DEGREES, CAP_THICKNESS) / op.surface_density_scale
        full = sle.ExpandBatch(torch.tensor(cap, device=device).contiguous().view(-1), 1).cpu().numpy().ravel()
        nodes = 11
        dt = DT_YEARS * configs.SECONDS_PER_YEAR / op.time_scale
        times = dt * np.arange(nodes)
        loads = np.stack([full * min(k, RAMP_STEPS) / RAMP_STEPS for k in range(nodes)])
        loads[0] = loads[1] * 0.5
        # one seeded pattern of U and one of phi, read at every node with a
        # weight growing in time (a time series of one field's observations)
        rng = np.random.default_rng(7)
        decay = 1.0 / (1.0 + np.repeat(np.arange(lmax + 1), np.arange(lmax + 1) + 1))
        weight = (0.5 + np.arange(nodes) / nodes)[:, None]
        gU = weight * (real_coefficients(lmax, rng, 1) * decay)
        gPhi = weight * (real_coefficients(lmax, rng, 1) * decay)
        ev = Evolution3D(op, "sdirk2")

        def objective(out):
            return sum(pairing(lmax, gU[k], out["U"][k]) + pairing(lmax, gPhi[k], out["phi"][k])
                       for k in range(nodes))

        ev.Run(times, loads)  # warm: flavours built, buffers allocated
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        forward = ev.Run(times, loads)
        torch.cuda.synchronize()
        forward_s = time.perf_counter() - t0
        ev.Adjoint(times[:2], loads[:2], gU[:2], gPhi[:2])  # warm: the sweep's buffers
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        adj = ev.Adjoint(times, loads, gU, gPhi)
        torch.cuda.synchronize()
        adjoint_s = time.perf_counter() - t0
        J = objective(forward)
        paired = sum(pairing(lmax, adj["load_kernels"][k], loads[k]) for k in range(nodes))
        # the record stride 3: 4 of the 11 states kept, the gaps rebuilt
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sparse = ev.Adjoint(times, loads, gU, gPhi, stride=3)
        torch.cuda.synchronize()
        stride_s = time.perf_counter() - t0
        stride_gap = max(rel_err(sparse["load_kernels"], adj["load_kernels"]),
                         rel_err(sparse["delta_gradient"], adj["delta_gradient"]))
        # the gradient along a smooth direction over every node
        prng = np.random.default_rng(17)
        coeffs = real_coefficients(lmax, prng, 1)[0]
        coeffs *= 1.0 / (1.0 + np.repeat(np.arange(lmax + 1), np.arange(lmax + 1) + 1)) ** 2
        field = grid.SynthesiseBatch(torch.tensor(coeffs, device=device), 1).cpu().numpy().ravel()
        radial = 1.0 + 0.5 * np.sin(7.0 * np.asarray(op.radius))
        p = (radial[:, None] * field[None, :]).ravel()
        p /= np.max(np.abs(p))
        predicted = float(adj["delta_gradient"] @ p)

        def J_at(h):
            op.set_delta(delta + h * p)
            return objective(ev.Run(times, loads))

        h = 1e-2
        d1 = (J_at(h) - J_at(-h)) / (2 * h)
        d2 = (J_at(h / 2) - J_at(-h / 2)) / h
        richardson = (4 * d2 - d1) / 3
        op.set_delta(delta)
        return {"workload": name, "nodes": nodes, "forward_s": forward_s, "adjoint_s": adjoint_s,
                "sweep_over_forward": (adjoint_s - forward_s) / forward_s,
                "stride3_adjoint_s": stride_s, "stride3_rel_gap": stride_gap,
                "forward_passes_per_step": float(np.mean([i.iterations for i in forward["infos"][1:]])),
                "pairing_identity_rel_gap": abs(paired - J) / abs(J),
                "gradient_vs_differences_rel_gap": abs(predicted - richardson) / abs(richardson),
                "directional_derivative": predicted}

    out = [workload("config 1: lmax 32, 40 elements of order 4, Maxwell, delta degree 8 RMS 0.5, FP64",
                    32, 40, 5, 0.0, 8, 0.5, False),
           workload("config 2's Earth without its ocean: lmax 128, 80 elements of order 5, Burgers, delta degree "
                    "32 RMS 1.0, mixed form", 128, 80, 6, 0.5, 32, 1.0, True)]
    return {"case": "discrete 3D adjoint (load kernels and log-viscosity gradient), 10 Sdirk2 steps of 500 yr",
            "workloads": out}


# -- config 4: the ensemble ----------------------------------------------------------------------

def ensemble_case(args):
    """Config 4: the seeded members (48 by default; lmax from {32, 64, 96,
    128}, delta RMS 0.3-1.5 to degree lmax / 4, a cap of 5-20 degrees to 2 km
    over 10 steps of 500 yr, 20 Sdirk2 steps, 40-80 elements of order 4) in
    the mixed form with the extrapolated warm start. The autotuner picks the
    queue order and the members in flight; then the whole ensemble runs
    concurrently (sl3dgpu_v3d_run_many) and one member after another, each
    timed by the host clock around the call (inputs and outputs on the host,
    a run's copies inside it). Aggregate member-steps/s for both; the
    concurrent snapshots against the one-by-one ones; per-instance error of
    U and phi against the plain FP64 GPU form (itself pinned to the FP64
    oracle) for one member of each lmax."""
    from sl3dpp_gb300.ensemble import Ensemble, autotune, ensemble_members

    members = ensemble_members(args.ensemble_members, seed=4, steps=args.ensemble_steps)
    ens = Ensemble(members, precision=1)
    tune = autotune(ens, probe_steps=1)
    together = ens.run(threads=tune["threads"], order=tune["order"])
    alone = ens.run_sequential()
    steps = ens.member_steps()
    same = max(float(np.max(np.abs(together["U"][k] - alone["U"][k])) / np.max(np.abs(alone["U"][k])))
               for k in range(len(members)))
    picks = []
    for lmax in sorted({m["lmax"] for m in members}):
        picks.append(next(k for k, m in enumerate(members) if m["lmax"] == lmax))
    # the plain FP64 form to its tolerance (a pass budget the hard members' stages need)
    ref = Ensemble([members[k] for k in picks], precision=0, max_iterations=400).run_sequential()
    errors = []
    for j, k in enumerate(picks):
        err = lambda a, b: float(max(np.max(np.abs(a[n] - b[n])) / np.max(np.abs(b[n])) for n in range(1, len(b))))
        errors.append({"member": k, "lmax": members[k]["lmax"], "U": err(together["U"][k], ref["U"][j]),
                       "phi": err(together["phi"][k], ref["phi"][j])})
    passes = [sum(i.iterations for i in infos[1:]) for infos in together["infos"]]
    unconverged = sum(1 for infos in together["infos"] for i in infos if not i.converged)
    unconverged_ref = sum(1 for infos in ref["infos"] for i in infos if not i.converged)
    return {"case": f"config 4: {len(members)} members, lmax 32-128, mixed form, {args.ensemble_steps} Sdirk2 steps",
            "member_steps": steps, "concurrent_steps_per_s": steps / together["seconds"],
            "sequential_steps_per_s": steps / alone["seconds"],
            "speedup_concurrent": alone["seconds"] / together["seconds"],
            "threads": tune["threads"], "probe_seconds": tune["probe_seconds"],
            "order_first": tune["order"][:8], "concurrent_vs_sequential_max_rel_U": same,
            "fp64_passes_per_member": passes, "unconverged_steps": unconverged,
            "unconverged_steps_fp64_reference": unconverged_ref, "per_instance_error_vs_fp64": errors,
            "lmax_counts": {str(l): sum(1 for m in members if m["lmax"] == l) for l in (32, 64, 96, 128)}}


# -- main ------------------------------------------------------------------------------------------

def main():
    global CORRECTION_RTOL, CORRECTION_MEMORY
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-fp64-compare", action="store_true", help="skip the plain FP64 form's run")
    ap.add_argument("--lmax", type=int, default=LMAX, help="a smaller workload for development runs")
    ap.add_argument("--correction-rtol", type=float, default=CORRECTION_RTOL)
    ap.add_argument("--correction-memory", type=int, default=CORRECTION_MEMORY)
    ap.add_argument("--warmstart-case", action="store_true",
                    help="instead: the learned warm start against the plain starts on held-out fields at lmax 128")
    ap.add_argument("--legendre-case", action="store_true",
                    help="instead: the FP32 tensor-core Legendre contraction alone at the workload's lmax")
    ap.add_argument("--ocean-case", action="store_true",
                    help="instead: config 2, the coupled step under an ocean at lmax 128, 50 steps")
    ap.add_argument("--adjoint-case", action="store_true",
                    help="instead: the discrete 3D adjoint at config 1's and config 2's Earth (no ocean)")
    ap.add_argument("--ensemble-case", action="store_true",
                    help="instead: config 4, the seeded ensemble (autotuned schedule, concurrent and one by one)")
    ap.add_argument("--ensemble-members", type=int, default=48)
    ap.add_argument("--ensemble-steps", type=int, default=20)
    args = ap.parse_args()
    if args.lmax != LMAX:
        _rescale(args.lmax)
    CORRECTION_RTOL, CORRECTION_MEMORY = args.correction_rtol, args.correction_memory
    if args.warmup < 3:
        raise SystemExit("at least three warm-up steps")
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))

    if args.impl == "reference":
        if rank != 0:
            return
        import __graft_entry__

        from oracle import build as oracle_build

        oracle_build.build()
        sampler = CpuSampler()
        # one untimed warm-up pass (the CPU needs no more), then a pass per
        # timed step after a single stage start
        r = sampler.sample(PASSES_PER_STEP, 1 + args.steps,
                           source="the plain FP64 GPU arm's measured passes a step at this workload")
        step_s = r["step_seconds"][1:]
        value = 1.0 / float(np.median(step_s))
        whole = config1_cpu_run()
        line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": 0,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / value,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": workload_config("fp64"), "impl": "reference",
                "extrapolated": True,
                "timed_seconds": r["start_seconds"] + sum(r["pass_seconds"]),
                "cpu_baseline": {"value": value, "unit": "steps/s", "cores": r["cores"], "kind": "port",
                                 "sample": r["sample"], "extrapolated": True},
                "config1_full_run": whole,
                "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch

    if world > 1:
        torch.distributed.init_process_group("nccl")
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
    device = torch.device("cuda", torch.cuda.current_device())
    import __graft_entry__

    __graft_entry__.build()
    from sl3dpp_gb300._lib import lib
    import ctypes

    if args.warmstart_case:
        if rank == 0:
            print(json.dumps(warmstart_case(args)), flush=True)
        return
    if args.legendre_case:
        if rank == 0:
            print(json.dumps(legendre_case(args, device)), flush=True)
        return
    if args.ocean_case:
        if rank == 0:
            print(json.dumps(ocean_case(args, device)), flush=True)
        return
    if args.adjoint_case:
        if rank == 0:
            print(json.dumps(adjoint_case(args, device)), flush=True)
        return
    if args.ensemble_case:
        if rank == 0:
            print(json.dumps(ensemble_case(args)), flush=True)
        return
    fp64, fp32 = ctypes.c_double(), ctypes.c_double()
    lib().sl3dgpu_fp64_fma_peak(ctypes.byref(fp64))
    lib().sl3dgpu_fp32_fma_peak(ctypes.byref(fp32))
    r = gpu_arm(args, rank, world, device, args.precision)
    steps_total = args.steps * world
    value = aggregate_rate(args.steps, world, r["seconds"])
    e2e = aggregate_rate(args.steps, world, r["e2e_seconds"])
    passes_per_step = r["passes"] / args.steps
    line = {"metric": METRIC if args.precision == "mixed" else "3D steps/sec at lmax=256 (plain FP64 GPU)",
            "value": value, "unit": "steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["seconds"] * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+f32" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded delta field and ice-cap load; random-free radial Earth)",
            "config": workload_config(args.precision),
            "passes_per_step": passes_per_step,
            "correction_passes_per_step": r["corrections"] / args.steps,
            "last_step": r["history"],
            "converged_steps": sum(int(i.converged) for i in r["infos"]),
            "timing": ("value: steps W .. W + K - 1 with device-resident loads, CUDA events on the operator's "
                       "stream, kernel timing events off; kernel_ms: the same steps again with them on; e2e: the "
                       "same steps from the same warmed state, host loads and surface read-back"),
            "final_residual": r["infos"][-1].residual,
            "roofline": roofline(r["profile"], fp64.value, fp32.value, double_float_rings=args.precision == "mixed"),
            "kernel_ms": {k: round(v["ms"], 3) for k, v in r["profile"].items() if v["launches"]},
            "gpu_launches": int(r["launches"]),
            "clocks": r["clocks"],
            "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": 2 * r["load_bytes"],
                    "d2h_bytes_per_step": 2 * r["load_bytes"]},
            "setup_seconds": r["setup_s"],
            "fma_peaks_gflops": {"fp64": fp64.value, "fp32": fp32.value}}
    fp64_passes = None
    if args.precision == "mixed" and not args.no_fp64_compare:
        mixed_surfaces = r["surfaces"]
        del r
        arms = {}
        # the plain FP64 form as the reference computes it (the FP64 units),
        # and with its Legendre contractions emulated on the tensor cores and
        # its ring transforms in double-float on the FP32 pipe
        for name, emulation in (("fp64_gpu", 0), ("fp64_gpu_tc_emulated", 1)):
            # timed with the kernel events on: a few ms of a 2-5 s step
            rr = gpu_arm(args, rank, world, device, "fp64", emulation=emulation, e2e=False, profile_apart=False)
            errs = [(rel_err(m[0], f[0]), rel_err(m[1], f[1])) for m, f in zip(mixed_surfaces, rr["surfaces"])]
            arms[name] = rr
            line[name] = {"value": steps_total / rr["seconds"], "unit": "steps/s",
                          "ms_per_step": rr["seconds"] * 1e3 / args.steps,
                          "passes_per_step": rr["passes"] / args.steps,
                          "kernel_ms": {k: round(v["ms"], 3) for k, v in rr["profile"].items() if v["launches"]},
                          "roofline": roofline(rr["profile"], fp64.value, fp32.value,
                                               double_float_rings=emulation == 1),
                          "clocks": rr["clocks"],
                          "mixed_rel_err": {"U": max(e[0] for e in errs), "phi": max(e[1] for e in errs),
                                            "steps_compared": len(errs),
                                            "per_step": [[round(a, 14), round(b, 14)] for a, b in errs]}}
            del rr
        fastest = max(("fp64_gpu", "fp64_gpu_tc_emulated"), key=lambda k: line[k]["value"])
        fp64_passes = line["fp64_gpu"]["passes_per_step"]
        line["speedup_vs_fp64_gpu"] = value / line[fastest]["value"]
        line["speedup_vs_fp64_gpu_against"] = fastest
        line["speedup_vs_fp64_gpu_units"] = value / line["fp64_gpu"]["value"]
        line["rel_err_vs_fp64"] = dict(line["fp64_gpu"]["mixed_rel_err"], against="fp64_gpu (the FP64 units)")
    elif args.precision == "fp64":
        fp64_passes = passes_per_step
    if rank == 0 and not args.no_cpu_baseline:
        try:
            sampler = CpuSampler()
            src = "measured by the plain FP64 GPU arm of this run" if fp64_passes else \
                  "the plain FP64 GPU arm's measured passes a step at this workload"
            line["cpu_baseline"] = {k: v for k, v in sampler.sample(fp64_passes or PASSES_PER_STEP, 2,
                                                                    source=src).items()
                                    if k not in ("step_seconds", "start_seconds", "pass_seconds")}
        except Exception as exc:  # the baseline is reported, not required
            line["cpu_baseline"] = {"value": None, "error": str(exc)[:200]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
