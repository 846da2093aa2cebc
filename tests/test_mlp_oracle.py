"""The network oracle (oracle/mlp_oracle.py) on the CPU: its BF16 rounding
matches torch's, and its analytic gradients match central finite differences
of its own loss.  With no reference implementation of the surrogate, this is
what pins the oracle that the device gradients are checked against."""
import numpy as np
import pytest
import torch

from conftest import ROOT  # noqa: F401  (puts the repo root on sys.path)


@pytest.fixture(scope="module")
def mo():
    from oracle import mlp_oracle
    return mlp_oracle


def _params(mo, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    layers, ow5, ob5, n = mo.layout()
    p = np.zeros(n)
    for o, fin, ob in layers:
        a = np.sqrt(6.0 / (9 if fin == mo.KIN else mo.H)) * scale
        W = rng.uniform(-a, a, (mo.H, fin))
        if fin == mo.KIN:
            W[:, 9:] = 0.0
        p[o:o + mo.H * fin] = W.ravel()
        p[ob:ob + mo.H] = rng.normal(0, 0.05, mo.H)
    p[ow5:ow5 + mo.H] = rng.uniform(-0.1, 0.1, mo.H)
    p[ob5] = 0.1
    return p


def _states(n, seed):
    from puzzletunneldiscovery_gb300 import workloads as W
    return W.uniform_states(n, -2.0, 2.0, 0.4, seed=seed)


def test_bf16_rounding_matches_torch(mo):
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(0, 1, 10000), rng.normal(0, 1e-3, 1000), [0.0, -0.0, 1.0, 3.0e38]])
    x = x.astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).float().numpy()
    assert (mo.bf16(x) == ref).all()


def test_features_are_rotation_columns(mo):
    q = _states(200, 1)
    f = mo.features(q).astype(np.float64)
    for i in range(0, 200, 37):
        w, x, y, z = q[i, 3:]
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        assert np.allclose(f[i, 3:6], R[:, 0], atol=1e-6)
        assert np.allclose(f[i, 6:9], R[:, 1], atol=1e-6)
        assert np.allclose(f[i, :3], q[i, :3], atol=1e-6)
        assert (f[i, 9:] == 0).all()


def test_oracle_gradient_matches_finite_differences(mo):
    p = _params(mo, 3)
    q = _states(48, 4)
    y = (np.arange(48) % 3 == 0).astype(np.float64)
    _, g = mo.gradients(p, q, y, rounding=False)
    layers, ow5, ob5, n = mo.layout()
    rng = np.random.default_rng(5)
    picks = [ob5] + list(rng.integers(ow5, ow5 + mo.H, 4))
    for o, fin, ob in layers:
        rows = rng.integers(0, mo.H, 4)
        cols = rng.integers(0, 9, 4)
        picks += [o + r * fin + c for r, c in zip(rows, cols)]
        picks += list(ob + rng.integers(0, mo.H, 2))
    h = 1e-6
    for i in picks:
        e = np.zeros(n)
        e[i] = h
        fd = (mo.loss(p + e, q, y, rounding=False) - mo.loss(p - e, q, y, rounding=False)) / (2 * h)
        # central differences in FP64: truncation O(h^2), cancellation ~1e-16/h
        assert abs(fd - g[i]) <= 1e-7 + 1e-4 * abs(fd), (i, fd, g[i])


def test_rounded_gradient_close_to_exact(mo):
    """BF16 rounding of weights and activations moves the gradient by a few
    percent at most: the device is compared with the rounded oracle, and this
    bounds how far that is from the exact-arithmetic gradient."""
    p = _params(mo, 6)
    q = _states(256, 7)
    y = (np.arange(256) % 2).astype(np.float64)
    _, g0 = mo.gradients(p, q, y, rounding=False)
    _, g1 = mo.gradients(p, q, y, rounding=True)
    assert np.linalg.norm(g1 - g0) <= 0.05 * np.linalg.norm(g0)


def test_adam_step(mo):
    p = np.array([1.0, -2.0, 0.5])
    g = np.array([0.1, -0.2, 0.0])
    p1, m1, m2 = mo.adam(p, g, np.zeros(3), np.zeros(3), 1, 1e-3)
    # first bias-corrected step moves each parameter by lr * sign(g)
    assert np.allclose(p1 - p, [-1e-3, 1e-3, 0.0], atol=1e-10)
