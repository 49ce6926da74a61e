"""The learned warm start of the 3D step (sl3dgpu_wsnet_*, csrc/warmstart.cu).

A network guesses the strain coefficients at the end of the next step from
the last three strain changes; Viscoelastic3D takes the guess through its
start hook (Converge's `start`, reference include/sl3dpp/Viscoelastic3D.hpp:
562-569) and keeps it only when its first residual beats the plain start's,
so the iteration still runs to the tolerance. This module holds the
network handle, the generation of training pairs from runs of the plain
method, the training loop (forward, backward and Adam on the GPU, one call
per batch) and the driver that feeds an operator its guesses.

Training pairs: config-1-style runs (lmax 32, 40 elements of order 4,
Maxwell mantle, a polar cap growing over 10 steps of 500 yr then held),
each on its own seeded delta field (degree 8, RMS and cap radius drawn per
run), every step converged to the tolerance; a pair is four consecutive
changes of the strain coefficients at the lateral nodes, Delta_n-2 ..
Delta_n+1, as FP32 complex columns.
"""

from __future__ import annotations

import ctypes
import pathlib

import numpy as np

from ._lib import P_double, check, lib

HIDDEN, DEPTH = 768, 6
_SIGNED = False


def _signatures():
    global _SIGNED
    if _SIGNED:
        return
    L = lib()
    v, i, d, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_float
    P_float = ctypes.POINTER(ctypes.c_float)
    sig = {
        "sl3dgpu_wsnet_create": (i, [i, i, ctypes.c_ulonglong, ctypes.POINTER(v)]),
        "sl3dgpu_wsnet_destroy": (None, [v]),
        "sl3dgpu_wsnet_parameter_count": (ctypes.c_longlong, [v]),
        "sl3dgpu_wsnet_parameters": (i, [v, P_float]),
        "sl3dgpu_wsnet_set_parameters": (i, [v, P_float]),
        "sl3dgpu_wsnet_bind": (i, [v, i, i, P_double, P_double]),
        "sl3dgpu_wsnet_gradient": (i, [v, i, v, v, v, v, P_float, P_float, P_float, P_float]),
        "sl3dgpu_wsnet_train_step": (i, [v, i, v, v, v, v, P_float, P_float, f, P_float]),
        "sl3dgpu_wsnet_predict": (i, [v, i, i, v, v, v, v, d, v, v]),
        "sl3dgpu_wsnet_gemm": (i, [v, v, v, i, i, i, v]),
        "sl3dgpu_v3d_lateral_range": (i, [v, ctypes.POINTER(i), ctypes.POINTER(i)]),
        "sl3dgpu_v3d_node_relaxation": (i, [v, P_double]),
        "sl3dgpu_v3d_state_coefficients_copy": (i, [v, v, v]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _SIGNED = True


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _ptrs(tensors):
    return (ctypes.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])


class Pair:
    """Four consecutive lateral-column changes of one run (device complex64
    tensors [rows, lateral]), the load ratio of the predicted step and the
    extrapolation's squared error (the pair's normaliser)."""

    def __init__(self, d2, d1, d0, target, ratio: float):
        self.d2, self.d1, self.d0, self.target = d2, d1, d0, target
        self.ratio = float(ratio)
        self.norm = float((target - d0).abs().pow(2).sum().item())


class WarmStartNet:
    def __init__(self, hidden: int = HIDDEN, depth: int = DEPTH, seed: int = 0):
        _signatures()
        h = ctypes.c_void_p()
        check(lib().sl3dgpu_wsnet_create(hidden, depth, seed, ctypes.byref(h)))
        self._h = h
        self.hidden, self.depth = hidden, depth
        self.layout = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().sl3dgpu_wsnet_destroy(h)
            self._h = None

    @property
    def parameter_count(self) -> int:
        return int(lib().sl3dgpu_wsnet_parameter_count(self._h))

    def parameters(self) -> np.ndarray:
        out = np.empty(self.parameter_count, dtype=np.float32)
        check(lib().sl3dgpu_wsnet_parameters(self._h, _fptr(out)))
        return out

    def set_parameters(self, values: np.ndarray) -> None:
        a = np.ascontiguousarray(values, dtype=np.float32)
        assert a.size == self.parameter_count
        check(lib().sl3dgpu_wsnet_set_parameters(self._h, _fptr(a)))

    def save(self, path) -> None:
        """The BF16-rounded parameters (what the products use) and the shape."""
        p = self.parameters()
        bits = (p.view(np.uint32) + 0x7FFF + ((p.view(np.uint32) >> 16) & 1)) >> 16
        np.savez_compressed(path, bf16=bits.astype(np.uint16), hidden=self.hidden, depth=self.depth)

    @classmethod
    def load(cls, path) -> "WarmStartNet":
        d = np.load(path)
        net = cls(int(d["hidden"]), int(d["depth"]))
        net.set_parameters((d["bf16"].astype(np.uint32) << 16).view(np.float32))
        return net

    def bind(self, lmax: int, depth_fraction: np.ndarray, relax: np.ndarray) -> None:
        depth_fraction = np.ascontiguousarray(depth_fraction, dtype=np.float64)
        relax = np.ascontiguousarray(relax, dtype=np.float64)
        check(lib().sl3dgpu_wsnet_bind(self._h, lmax, depth_fraction.size, depth_fraction.ctypes.data_as(P_double),
                                       relax.ctypes.data_as(P_double)))
        self.layout = (lmax, depth_fraction.size)

    def _batch(self, pairs):
        ratio = np.array([p.ratio for p in pairs], dtype=np.float32)
        norm = np.array([p.norm for p in pairs], dtype=np.float32)
        return (len(pairs), _ptrs([p.d2 for p in pairs]), _ptrs([p.d1 for p in pairs]),
                _ptrs([p.d0 for p in pairs]), _ptrs([p.target for p in pairs]), ratio, norm)

    def gradient(self, pairs):
        n, a, b, c, t, ratio, norm = self._batch(pairs)
        grad = np.empty(self.parameter_count, dtype=np.float32)
        loss = ctypes.c_float()
        check(lib().sl3dgpu_wsnet_gradient(self._h, n, a, b, c, t, _fptr(ratio), _fptr(norm), _fptr(grad),
                                           ctypes.byref(loss)))
        return loss.value, grad

    def train_step(self, pairs, lr: float) -> float:
        n, a, b, c, t, ratio, norm = self._batch(pairs)
        loss = ctypes.c_float()
        check(lib().sl3dgpu_wsnet_train_step(self._h, n, a, b, c, t, _fptr(ratio), _fptr(norm), float(lr),
                                             ctypes.byref(loss)))
        return loss.value

    def gemm(self, A, B):
        """C = A B^T on the tensor cores (BF16 operands, FP32 sums); CUDA float32 tensors."""
        import torch

        M, K = A.shape
        N = B.shape[0]
        C = torch.empty((M, N), dtype=torch.float32, device=A.device)
        torch.cuda.synchronize()
        check(lib().sl3dgpu_wsnet_gemm(self._h, A.data_ptr(), B.data_ptr(), M, N, K, C.data_ptr()))
        return C


# -- the operator side ----------------------------------------------------------------------------

def lateral_layout(op, dt: float):
    """The operator's lateral node range and, per lateral node, its depth
    fraction in the range and log10(dt itau) / 4."""
    _signatures()
    first, end = ctypes.c_int(), ctypes.c_int()
    check(lib().sl3dgpu_v3d_lateral_range(op._h, ctypes.byref(first), ctypes.byref(end)))
    itau = np.empty(op.node_count)
    check(lib().sl3dgpu_v3d_node_relaxation(op._h, itau.ctypes.data_as(P_double)))
    p0, p1 = first.value, end.value
    r = op.radius[p0:p1]
    depth = (r - r.min()) / max(r.max() - r.min(), 1e-300)
    relax = np.log10(np.maximum(dt * itau[p0:p1], 1e-12)) / 4.0
    return p0, p1, depth, relax


def _coefficients(op, state):
    """A copy of a state's strain coefficients (device layout) as a complex128
    device tensor [rows, nodes]."""
    import torch

    _, count = state.device_coefficients()
    out = torch.empty(count // 2, dtype=torch.complex128, device=torch.device("cuda", torch.cuda.current_device()))
    check(lib().sl3dgpu_v3d_state_coefficients_copy(op._h, state._h, out.data_ptr()))
    return out.view(-1, op.node_count)


class LearnedStart:
    """Feeds an operator the network's guess before each step: keeps the last
    four strain snapshots (device) and the load history."""

    def __init__(self, net: WarmStartNet, op, dt: float):
        self.net, self.op, self.dt = net, op, dt
        self.p0, self.p1, depth, relax = lateral_layout(op, dt)
        net.bind(op.lmax, depth, relax)
        self.snapshots = []
        self.loads = []

    def record(self, state, load) -> None:
        self.snapshots = (self.snapshots + [_coefficients(self.op, state)])[-4:]
        self.loads = (self.loads + [np.asarray(load)])[-3:]

    def arm(self, next_load) -> bool:
        """The guess for the next step (True), once four snapshots are held."""
        import torch

        if len(self.snapshots) < 4:
            return False
        ratio = load_ratio(self.loads[-2], self.loads[-1], next_load)
        s3, s2, s1, s0 = self.snapshots
        L = self.op.lmax
        rows = 2 * (L + 1) ** 2 - 5 + (L + 1) * (L + 2) // 2  # spin -2, -1 and real spin 0 rows
        assert all(s.numel() == rows * self.op.node_count for s in self.snapshots)
        guess = torch.empty_like(s0)
        check(lib().sl3dgpu_wsnet_predict(self.net._h, self.op.node_count, self.p0, s0.data_ptr(), s1.data_ptr(),
                                          s2.data_ptr(), s3.data_ptr(), ratio, guess.data_ptr(), self.op.stream))
        self.op.set_start(guess.view(-1).view(torch.float64))
        return True


def load_ratio(previous, current, following) -> float:
    """The coming load increment's size over the last one's (0 when the
    last was none)."""
    last = np.linalg.norm(np.asarray(current) - np.asarray(previous))
    coming = np.linalg.norm(np.asarray(following) - np.asarray(current))
    return float(min(coming / last, 4.0)) if last > 0 else 0.0


# -- training pairs from the plain method ---------------------------------------------------------

def run_member(seed: int, steps: int, lmax: int = 32, elements: int = 40, ngll: int = 5, rms: float = 0.5,
               ldelta: int = 8, cap_degrees: float = 15.0, ramp_steps: int = 10, dt_years: float = 500.0,
               precision: int = 1, device=None):
    """One config-1-style run, every step converged; returns the lateral
    columns' changes (complex64 device tensors, one per step), the loads'
    ratios per step, the layout (depth fractions, relaxation) and the pass
    counts."""
    import torch

    from . import configs
    from .grid import SurfaceGrid
    from .viscoelastic3d import Options, Viscoelastic3D, standard_earth

    device = device or torch.device("cuda", torch.cuda.current_device())
    op = Viscoelastic3D(standard_earth(elements), Options.defaults(
        lmax, ngll, rtol=1e-10, max_iterations=150, precision=precision, correction_rtol=3e-6,
        correction_memory=10, warm_start=1 if precision == 1 else 0, fp64_emulation=precision))
    grid = SurfaceGrid(lmax, 0, 1.5)
    c = configs.delta_coefficients(lmax, ldelta, rms, seed)
    pattern = grid.SynthesiseBatch(torch.tensor(c, device=device), 1)
    ind = torch.tensor(configs.delta_indicator(op.radius), device=device)
    op.set_delta((ind[:, None] * pattern[None, :]).contiguous().view(-1))
    exact = SurfaceGrid(lmax, 0, 1.0)
    cap = configs.cap_field(exact.theta, exact.nphi, cap_degrees, 2000.0)
    full = (exact.ExpandBatch(torch.tensor(cap, device=device), 1) / op.surface_density_scale).cpu().numpy()
    dt = dt_years * configs.SECONDS_PER_YEAR / op.time_scale
    p0, p1, depth, relax = lateral_layout(op, dt)
    state = op.ZeroState()
    loads = [full * min(n, ramp_steps) / ramp_steps for n in range(steps + 1)]
    prev = None
    changes, ratios, passes = [], [], []
    for n in range(steps):
        info = op.Step(state, dt, "sdirk2", loads[n], loads[n + 1])
        assert info.converged, (seed, n)
        passes.append(info.iterations)
        s = _coefficients(op, state)
        if prev is not None:
            changes.append((s - prev)[:, p0:p1].to(torch.complex64).contiguous())
            ratios.append(load_ratio(loads[n - 1], loads[n], loads[n + 1]))
        prev = s
    return {"changes": changes, "ratios": ratios, "depth": depth, "relax": relax, "passes": passes}


def pairs_of(run):
    """Every window of four consecutive changes; the ratio is the predicted
    step's."""
    ch, ra = run["changes"], run["ratios"]
    return [Pair(ch[k - 3], ch[k - 2], ch[k - 1], ch[k], ra[k]) for k in range(3, len(ch))]


def train(net: WarmStartNet, pairs, epochs: int, batch: int = 16, lr: float = 3e-4, seed: int = 0,
          log=None, decay: bool = False) -> list[float]:
    """Adam over shuffled batches (the rate cosine-decayed to a tenth over
    the epochs with decay); returns each epoch's mean loss."""
    rng = np.random.default_rng(seed)
    history = []
    for epoch in range(epochs):
        order = rng.permutation(len(pairs))
        losses = []
        rate = lr * (0.55 + 0.45 * np.cos(np.pi * epoch / max(epochs - 1, 1))) if decay else lr
        for k in range(0, len(order) - batch + 1, batch):
            losses.append(net.train_step([pairs[i] for i in order[k:k + batch]], rate))
        history.append(float(np.mean(losses)))
        if log:
            log(f"epoch {epoch}: loss {history[-1]:.4f}")
    return history


def default_weights() -> pathlib.Path:
    return pathlib.Path(__file__).resolve().parent / "warmstart_weights.npz"


def evaluate(net: WarmStartNet | None, seed: int, steps: int, lmax: int, elements: int, ngll: int, rms: float,
             ldelta: int, precision: int, cap_degrees: float = 15.0, ramp_steps: int = 10, dt_years: float = 500.0,
             device=None):
    """One held-out run with (net) or without (None) the learned start: the
    passes of every step and the surface U and phi after each."""
    import torch

    from . import configs
    from .grid import SurfaceGrid
    from .viscoelastic3d import Options, Viscoelastic3D, standard_earth

    device = device or torch.device("cuda", torch.cuda.current_device())
    op = Viscoelastic3D(standard_earth(elements), Options.defaults(
        lmax, ngll, rtol=1e-10, max_iterations=150, precision=precision, correction_rtol=3e-6,
        correction_memory=10, warm_start=1 if precision == 1 else 0, fp64_emulation=precision))
    grid = SurfaceGrid(lmax, 0, 1.5)
    c = configs.delta_coefficients(lmax, ldelta, rms, seed)
    pattern = grid.SynthesiseBatch(torch.tensor(c, device=device), 1)
    ind = torch.tensor(configs.delta_indicator(op.radius), device=device)
    op.set_delta((ind[:, None] * pattern[None, :]).contiguous().view(-1))
    exact = SurfaceGrid(lmax, 0, 1.0)
    cap = configs.cap_field(exact.theta, exact.nphi, cap_degrees, 2000.0)
    full = (exact.ExpandBatch(torch.tensor(cap, device=device), 1) / op.surface_density_scale).cpu().numpy()
    dt = dt_years * configs.SECONDS_PER_YEAR / op.time_scale
    helper = LearnedStart(net, op, dt) if net is not None else None
    state = op.ZeroState()
    loads = [full * min(n, ramp_steps) / ramp_steps for n in range(steps + 1)]
    out = {"passes": [], "corrections": [], "taken": [], "U": [], "phi": [], "seconds": 0.0}
    import time

    for n in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        armed = helper.arm(loads[n + 1]) if helper is not None else False
        info = op.Step(state, dt, "sdirk2", loads[n], loads[n + 1])
        if helper is not None:
            helper.record(state, loads[n + 1])
        torch.cuda.synchronize()
        out["seconds"] += time.perf_counter() - t0
        assert info.converged, (seed, n)
        out["passes"].append(info.iterations)
        out["corrections"].append(info.correction_passes)
        out["taken"].append(bool(armed and op.start_taken))
        out["U"].append(op.Surface("U"))
        out["phi"].append(op.Surface("phi"))
    return out


def main(argv=None):
    """Train the network on pairs of config-1-style runs and save it:
    python -m sl3dpp_gb300.warmstart OUT.npz [--runs 64] [--steps 66] [--epochs 40]"""
    import argparse
    import json
    import time

    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("out")
    ap.add_argument("--runs", type=int, default=64)
    ap.add_argument("--steps", type=int, default=66)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--decay", action="store_true", help="cosine-decay the rate to a tenth over the epochs")
    args = ap.parse_args(argv)
    rng = np.random.default_rng(args.seed)
    t0 = time.time()
    pairs, layout, passes = [], None, []
    for k in range(args.runs):
        run = run_member(seed=10_000 + k, steps=args.steps, rms=float(rng.uniform(0.3, 1.0)),
                         cap_degrees=float(rng.uniform(5.0, 20.0)))
        layout = layout or (run["depth"], run["relax"])
        pairs += pairs_of(run)
        passes.append(float(np.mean(run["passes"])))
    gen_s = time.time() - t0
    net = WarmStartNet(seed=args.seed)
    net.bind(32, *layout)
    torch.cuda.synchronize()
    t1 = time.time()
    history = train(net, pairs, args.epochs, args.batch, args.lr, args.seed, log=print, decay=args.decay)
    net.save(args.out)
    print(json.dumps({"pairs": len(pairs), "runs": args.runs, "generation_s": gen_s,
                      "training_s": time.time() - t1, "loss_first_epoch": history[0], "loss_last_epoch": history[-1],
                      "parameters": net.parameter_count, "mean_passes_per_step": float(np.mean(passes))}))


if __name__ == "__main__":
    main()
