"""ORACLE -- test infrastructure only: the learned warm start's network on
the CPU in numpy (FP64 unless asked), the checker of the GPU's forward and
backward kernels (sl3dpp_gb300/csrc/warmstart.cu).

The same computation written plainly: the per-(degree, lateral node) unit
features from the last three strain changes of each spin block, the
multilayer perceptron (GELU, tanh form), the predicted change a Delta_n +
b Delta_n-1 + c Delta_n-2 per block and order, the loss (the squared error
over the extrapolation's, averaged over the pairs) and its gradient with
respect to every parameter by reverse accumulation. The parameter vector's
layout is the library's: per layer the weights (out x in, row-major), then
the biases.
"""

from __future__ import annotations

import numpy as np

FEATURES = 16
OUTPUTS = 16
BLOCKS = 3


def row_lists(lmax: int):
    """The rows of each (spin block, degree) in the m-major device layout:
    blocks spin -2 and -1 over every order, then the real spin 0 over m >= 0;
    within a block, order by order, rows l = max(|m|, |N|) .. lmax."""
    lists = [[[] for _ in range(lmax + 1)] for _ in range(BLOCKS)]
    row = 0
    for b, N in enumerate((-2, -1, 0)):
        for m in range(0 if b == 2 else -lmax, lmax + 1):
            for l in range(max(abs(m), abs(N)), lmax + 1):
                lists[b][l].append(row)
                row += 1
    return [[np.array(x, dtype=np.int64) for x in blk] for blk in lists], row


def layer_shapes(hidden: int, depth: int):
    ins = [FEATURES] + [hidden] * depth
    outs = [hidden] * depth + [OUTPUTS]
    return list(zip(ins, outs))


def unpack(params: np.ndarray, hidden: int, depth: int):
    layers, at = [], 0
    for fin, fout in layer_shapes(hidden, depth):
        W = params[at:at + fin * fout].reshape(fout, fin)
        at += fin * fout
        b = params[at:at + fout]
        at += fout
        layers.append((W, b))
    assert at == params.size
    return layers


def features(lists, lmax, depth_fraction, relax, d2, d1, d0, ratio):
    """(units, 16) for one pair; units in (l, p) order."""
    lateral = d0.shape[1]
    f = np.zeros(((lmax + 1) * lateral, FEATURES))
    for l in range(lmax + 1):
        for b in range(BLOCKS):
            rows = lists[b][l]
            a, c, e = d0[rows], d1[rows], d2[rows]
            n0 = np.sum(np.abs(a) ** 2, axis=0)
            n1 = np.sum(np.abs(c) ** 2, axis=0)
            n2 = np.sum(np.abs(e) ** 2, axis=0)
            c01 = np.sum((a * np.conj(c)).real, axis=0)
            c12 = np.sum((c * np.conj(e)).real, axis=0)
            tiny = 1e-300
            with np.errstate(divide="ignore", invalid="ignore"):
                r1 = np.where(n1 > tiny, c01 / np.where(n1 > tiny, n1, 1.0), 0.0)
                r2 = np.where(n2 > tiny, c12 / np.where(n2 > tiny, n2, 1.0), 0.0)
                lr = np.where((n0 > tiny) & (n1 > tiny),
                              0.5 * np.log(np.where(n0 > tiny, n0, 1.0) / np.where(n1 > tiny, n1, 1.0)), 0.0)
            sl = slice(l * lateral, (l + 1) * lateral)
            f[sl, 4 * b] = np.clip(r1, -4, 4)
            f[sl, 4 * b + 1] = np.clip(r2, -4, 4)
            f[sl, 4 * b + 2] = np.clip(lr, -8, 8) * 0.25
            f[sl, 4 * b + 3] = (n0 > tiny).astype(float)
        sl = slice(l * lateral, (l + 1) * lateral)
        f[sl, 12] = l / (l + 10.0)
        f[sl, 13] = depth_fraction
        f[sl, 14] = relax
        f[sl, 15] = ratio
    return f


def gelu(x):
    c = np.sqrt(2.0 / np.pi)
    return 0.5 * x * (1.0 + np.tanh(c * (x + 0.044715 * x ** 3)))


def gelu_slope(x):
    c = np.sqrt(2.0 / np.pi)
    t = np.tanh(c * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * c * (1.0 + 3 * 0.044715 * x * x)


def forward(layers, X):
    Zs, Hs = [], [X]
    for i, (W, b) in enumerate(layers):
        Z = Hs[-1] @ W.T + b
        Zs.append(Z)
        Hs.append(Z if i == len(layers) - 1 else gelu(Z))
    return Zs, Hs


def loss_and_output_grad(lists, lmax, out, pairs):
    """out: (pairs, units, 16); pairs: list of (d2, d1, d0, target, norm)."""
    loss = 0.0
    g = np.zeros_like(out)
    P = len(pairs)
    for q, (d2, d1, d0, t, norm) in enumerate(pairs):
        lateral = d0.shape[1]
        for l in range(lmax + 1):
            sl = slice(l * lateral, (l + 1) * lateral)
            for b in range(BLOCKS):
                rows = lists[b][l]
                a = 1.0 + out[q, sl, 3 * b]
                bb = out[q, sl, 3 * b + 1]
                c = out[q, sl, 3 * b + 2]
                x0, x1, x2, tt = d0[rows], d1[rows], d2[rows], t[rows]
                r = a * x0 + bb * x1 + c * x2 - tt
                scale = 1.0 / (norm * P)
                loss += np.sum(np.abs(r) ** 2) * scale
                g[q, sl, 3 * b] = np.sum(2 * (r * np.conj(x0)).real, axis=0) * scale
                g[q, sl, 3 * b + 1] = np.sum(2 * (r * np.conj(x1)).real, axis=0) * scale
                g[q, sl, 3 * b + 2] = np.sum(2 * (r * np.conj(x2)).real, axis=0) * scale
    return loss, g


def gradient(params, hidden, depth, lmax, depth_fraction, relax, pairs, ratios):
    """The loss and the FP64 gradient of the parameter vector."""
    lists, _ = row_lists(lmax)
    layers = unpack(np.asarray(params, dtype=np.float64), hidden, depth)
    X = np.concatenate([features(lists, lmax, depth_fraction, relax, d2, d1, d0, r)
                        for (d2, d1, d0, _, _), r in zip(pairs, ratios)])
    Zs, Hs = forward(layers, X)
    units = X.shape[0] // len(pairs)
    out = Hs[-1].reshape(len(pairs), units, OUTPUTS)
    loss, g = loss_and_output_grad(lists, lmax, out, pairs)
    dZ = g.reshape(-1, OUTPUTS)
    grads = []
    for i in range(len(layers) - 1, -1, -1):
        W, _ = layers[i]
        grads.append((dZ.T @ Hs[i], dZ.sum(axis=0)))
        if i == 0:
            break
        dZ = (dZ @ W) * gelu_slope(Zs[i - 1])
    flat = []
    for dW, db in reversed(grads):
        flat += [dW.ravel(), db.ravel()]
    return loss, np.concatenate(flat)
