"""The learned warm start: its CPU oracle (oracle/warmstart_ref.py) against
finite differences, the GPU's tensor-core product and gradient against the
oracle, training on the GPU, and what the trained network gains over the
plain start on held-out delta fields with the error bar unchanged."""

import pathlib

import numpy as np
import pytest

from oracle import warmstart_ref as R

WEIGHTS = pathlib.Path(__file__).resolve().parent.parent / "sl3dpp_gb300" / "warmstart_weights.npz"


def _random_pairs(rng, lmax, lateral, count, scale=1.0):
    _, rows = R.row_lists(lmax)
    pairs, ratios = [], []
    for _ in range(count):
        base = rng.standard_normal((rows, lateral)) + 1j * rng.standard_normal((rows, lateral))
        d = [base * (0.8 ** k) * scale + 0.1 * (rng.standard_normal((rows, lateral)) + 1j * rng.standard_normal(
            (rows, lateral))) for k in range(4)]
        d2, d1, d0, t = d[3], d[2], d[1], d[0]
        pairs.append((d2, d1, d0, t, float(np.sum(np.abs(t - d0) ** 2))))
        ratios.append(float(rng.uniform(0, 1)))
    return pairs, ratios


def _params(rng, hidden, depth, last_zero=False):
    out = []
    for i, (fin, fout) in enumerate(R.layer_shapes(hidden, depth)):
        W = rng.standard_normal((fout, fin)) * np.sqrt(2.0 / fin)
        if last_zero and i == depth:
            W[:] = 0
        out += [W.ravel(), 0.1 * rng.standard_normal(fout)]
    return np.concatenate(out)


def test_row_lists_cover_every_row_once():
    for lmax in (4, 9):
        lists, rows = R.row_lists(lmax)
        seen = np.concatenate([x for blk in lists for x in blk])
        assert np.array_equal(np.sort(seen), np.arange(rows))
        assert rows == ((lmax + 1) ** 2 - 4) + ((lmax + 1) ** 2 - 1) + (lmax + 1) * (lmax + 2) // 2


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    lmax, lateral, hidden, depth = 4, 3, 16, 2
    pairs, ratios = _random_pairs(rng, lmax, lateral, 2)
    p = _params(rng, hidden, depth)
    dfrac, relax = np.linspace(0, 1, lateral), np.full(lateral, 0.3)
    loss, g = R.gradient(p, hidden, depth, lmax, dfrac, relax, pairs, ratios)
    for k in rng.choice(p.size, 12, replace=False):
        h = 1e-6 * max(1.0, abs(p[k]))
        up, dn = p.copy(), p.copy()
        up[k] += h
        dn[k] -= h
        fd = (R.gradient(up, hidden, depth, lmax, dfrac, relax, pairs, ratios)[0] -
              R.gradient(dn, hidden, depth, lmax, dfrac, relax, pairs, ratios)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def test_untrained_network_is_the_extrapolation():
    """The last layer starts at zero: the prediction is Delta_n, whose loss
    is one by the normaliser's definition."""
    rng = np.random.default_rng(1)
    pairs, ratios = _random_pairs(rng, 4, 3, 3)
    p = _params(rng, 16, 2, last_zero=True)
    n_last = R.layer_shapes(16, 2)[-1][1]
    p[-n_last:] = 0.0  # and its bias
    loss, _ = R.gradient(p, 16, 2, 4, np.linspace(0, 1, 3), np.zeros(3), pairs, ratios)
    assert abs(loss - 1.0) < 1e-12


@pytest.mark.gpu
def test_gpu_tensor_core_product_matches_numpy(gpu):
    import torch

    from sl3dpp_gb300.warmstart import WarmStartNet

    net = WarmStartNet(hidden=768, depth=2)
    gen = torch.Generator(device=gpu).manual_seed(3)
    for M, N, K in [(300, 200, 768), (129, 65, 16), (1000, 768, 200)]:
        A = torch.randn((M, K), device=gpu, generator=gen)
        B = torch.randn((N, K), device=gpu, generator=gen)
        C = net.gemm(A, B).double().cpu().numpy()
        a = A.to(torch.bfloat16).double().cpu().numpy()
        b = B.to(torch.bfloat16).double().cpu().numpy()
        want = a @ b.T
        assert np.max(np.abs(C - want)) <= 1e-5 * np.max(np.abs(want)), (M, N, K)


@pytest.mark.gpu
def test_gpu_gradient_matches_the_cpu_oracle(gpu):
    """The full network (768 wide, six hidden layers) on a small batch: the
    GPU's BF16-product gradient against the oracle's FP64 one."""
    import torch

    from sl3dpp_gb300.warmstart import Pair, WarmStartNet

    rng = np.random.default_rng(2)
    lmax, lateral = 6, 4
    pairs, ratios = _random_pairs(rng, lmax, lateral, 3)
    net = WarmStartNet(seed=5)
    p = net.parameters().astype(np.float64)
    # a non-zero last layer, so that every layer's gradient is exercised
    n_last_w = R.layer_shapes(768, 6)[-1][0] * R.layer_shapes(768, 6)[-1][1]
    p[-(n_last_w + 16):-16] = 0.01 * rng.standard_normal(n_last_w)
    net.set_parameters(p.astype(np.float32))
    p = net.parameters().astype(np.float64)
    dfrac, relax = np.linspace(0, 1, lateral), np.full(lateral, -0.2)
    net.bind(lmax, dfrac, relax)
    dev = [Pair(*[torch.tensor(x, dtype=torch.complex64, device=gpu) for x in pr[:4]], r)
           for pr, r in zip(pairs, ratios)]
    # the oracle on the same FP32-rounded inputs
    pairs32 = [tuple(x.astype(np.complex64).astype(np.complex128) for x in pr[:4]) + (d.norm,)
               for pr, d in zip(pairs, dev)]
    torch.cuda.synchronize()
    loss_gpu, g_gpu = net.gradient(dev)
    loss_cpu, g_cpu = R.gradient(p, 768, 6, lmax, dfrac, relax, pairs32, ratios)
    assert abs(loss_gpu - loss_cpu) <= 1e-2 * abs(loss_cpu)
    cos = float(g_gpu @ g_cpu / (np.linalg.norm(g_gpu) * np.linalg.norm(g_cpu)))
    # BF16 operands in every product (about 3 significant digits each), seven
    # layers deep: agreement to a few per cent, in direction to 0.5%
    err = np.linalg.norm(g_gpu - g_cpu) / np.linalg.norm(g_cpu)
    assert cos > 0.995 and err <= 0.1, (cos, err)


@pytest.mark.gpu
def test_gpu_training_lowers_the_loss_below_the_extrapolation(gpu):
    """A short training on pairs of two small runs (lmax 16): the loss falls
    below the extrapolation's (one)."""
    from sl3dpp_gb300 import warmstart as W

    runs = [W.run_member(seed=s, steps=24, lmax=16, elements=24, rms=0.7) for s in (11, 12)]
    pairs = W.pairs_of(runs[0]) + W.pairs_of(runs[1])
    net = W.WarmStartNet(hidden=256, depth=3, seed=1)
    net.bind(16, runs[0]["depth"], runs[0]["relax"])
    untrained, _ = net.gradient(pairs)
    assert abs(untrained - 1.0) < 1e-3  # the untrained network is the extrapolation
    history = W.train(net, pairs, epochs=30, batch=8, lr=1e-3)
    trained, _ = net.gradient(pairs)
    assert trained < 0.7 and history[-1] < 0.7, (trained, history)


@pytest.mark.gpu
def test_gpu_trained_network_saves_passes_at_lmax_128(gpu):
    """The committed network on held-out delta fields at lmax 128 (80
    elements of order 5): fewer passes of the plain FP64 fixed point than
    its own start (the previous step's strain), the same results to the
    tolerance."""
    from sl3dpp_gb300 import warmstart as W

    net = W.WarmStartNet.load(WEIGHTS)
    plain = W.evaluate(None, seed=90_001, steps=16, lmax=128, elements=80, ngll=6, rms=1.0, ldelta=32, precision=0)
    learned = W.evaluate(net, seed=90_001, steps=16, lmax=128, elements=80, ngll=6, rms=1.0, ldelta=32, precision=0)
    assert sum(learned["passes"]) < sum(plain["passes"]), (learned["passes"], plain["passes"])
    for a, b in zip(learned["U"] + learned["phi"], plain["U"] + plain["phi"]):
        assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(b))
