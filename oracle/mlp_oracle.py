"""CPU oracle of the learned proposal's network (TEST INFRASTRUCTURE ONLY).

Only tests/, the smoke check and bench.py's CPU legs may import this module;
the product path never does.

The reference has no collision surrogate, so there is no reference code to
follow: this module restates the network defined in include/pw_mlp.h in
numpy.  It rounds to BF16 at exactly the points the device kernels do (input
features, hidden weights, hidden activations, back-propagated dL/dZ) and does
every other operation in FP64, so the device result differs from it only by
FP32 accumulation order.  Its gradient formulas are pinned against central
finite differences of its own loss (tests/test_mlp_oracle.py), which needs no
device.
"""
from __future__ import annotations

import numpy as np

H = 256
KIN = 16
NLAYER = 4


def bf16(a) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float32."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(f.shape)


def layout():
    """Offsets of the parameter block (pw_mlp.h): list of (W offset, in, b offset), w5, b5, total."""
    o = 0
    layers = []
    for l in range(NLAYER):
        fin = KIN if l == 0 else H
        layers.append((o, fin, o + H * fin))
        o += H * fin + H
    return layers, o, o + H, o + H + 1


def unpack(p):
    layers, ow5, ob5, n = layout()
    assert p.shape == (n,)
    Ws = [p[o:o + H * fin].reshape(H, fin) for o, fin, _ in layers]
    bs = [p[ob:ob + H] for _, _, ob in layers]
    return Ws, bs, p[ow5:ow5 + H], p[ob5]


def pack(Ws, bs, w5, b5):
    out = []
    for W, b in zip(Ws, bs):
        out += [np.asarray(W, np.float64).ravel(), np.asarray(b, np.float64).ravel()]
    out += [np.asarray(w5, np.float64).ravel(), np.atleast_1d(np.float64(b5))]
    return np.concatenate(out)


def features(states) -> np.ndarray:
    """[n, 16] float32 features before BF16 rounding: translation, R(q)[:, 0], R(q)[:, 1]."""
    q = np.asarray(states, np.float64)
    f32 = np.float32
    t = q[:, :3].astype(f32)
    w, x, y, z = (q[:, 3 + i].astype(f32) for i in range(4))
    one, two = f32(1), f32(2)
    f = np.zeros((q.shape[0], KIN), f32)
    f[:, :3] = t
    f[:, 3] = one - two * (y * y + z * z)
    f[:, 4] = two * (x * y + w * z)
    f[:, 5] = two * (x * z - w * y)
    f[:, 6] = two * (x * y - w * z)
    f[:, 7] = one - two * (x * x + z * z)
    f[:, 8] = two * (y * z + w * x)
    return f


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, states, rounding=True):
    """Logits and the per-layer (input, pre-activation) pairs."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    Ws, bs, w5, b5 = unpack(np.asarray(p, np.float64))
    x = r(features(states)).astype(np.float64)
    cache = []
    for W, b in zip(Ws, bs):
        z = x @ r(W).astype(np.float64).T + b
        cache.append((x, z))
        x = r(_silu(z)).astype(np.float64)
    s = x @ w5 + b5
    return s, x, cache


def predict(p, states, rounding=True):
    s, _, _ = forward(p, states, rounding)
    return 1.0 / (1.0 + np.exp(-s))


def loss(p, states, labels, rounding=True):
    s, _, _ = forward(p, states, rounding)
    y = np.asarray(labels, np.float64)
    return float(np.mean(np.log1p(np.exp(-np.abs(s))) + np.maximum(s, 0) - y * s))


def gradients(p, states, labels, rounding=True):
    """(loss, gradient block) of the mean binary cross-entropy, label 1 = free."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    Ws, bs, w5, b5 = unpack(np.asarray(p, np.float64))
    s, h4, cache = forward(p, states, rounding)
    y = np.asarray(labels, np.float64)
    n = s.shape[0]
    L = float(np.mean(np.log1p(np.exp(-np.abs(s))) + np.maximum(s, 0) - y * s))
    g = (1.0 / (1.0 + np.exp(-s)) - y) / n
    dw5 = h4.T @ g
    db5 = g.sum()
    dWs, dbs = [None] * NLAYER, [None] * NLAYER
    G = r(np.outer(g, w5) * _dsilu(cache[-1][1])).astype(np.float64)
    for l in range(NLAYER - 1, -1, -1):
        x, _ = cache[l]
        dWs[l] = G.T @ x
        dbs[l] = G.sum(axis=0)
        if l == 0:
            break
        G = r((G @ r(Ws[l]).astype(np.float64)) * _dsilu(cache[l - 1][1])).astype(np.float64)
    return L, pack(dWs, dbs, dw5, db5)


def adam(p, grad, m1, m2, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015, bias-corrected), returns new (p, m1, m2)."""
    m1 = b1 * m1 + (1 - b1) * grad
    m2 = b2 * m2 + (1 - b2) * grad * grad
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    return p - lr * (m1 / c1) / (np.sqrt(m2 / c2) + eps), m1, m2
