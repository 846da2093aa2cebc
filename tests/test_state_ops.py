"""pyosr's module-level state helpers (state_ops.py) on the CPU: round trips,
agreement with an independent rotation library (scipy), and the path helpers."""
import math

import numpy as np
import pytest

from puzzletunneldiscovery_gb300 import state_ops as S


def _rand_states(n, seed):
    rng = np.random.default_rng(seed)
    q = np.zeros((n, 7))
    q[:, :3] = rng.uniform(-1, 1, (n, 3))
    r = rng.normal(size=(n, 4))
    q[:, 3:] = r / np.linalg.norm(r, axis=1, keepdims=True)
    return q


def test_decompose_compose_round_trips(built_lib):
    for q in _rand_states(50, 1):
        t, angle, axis = S.decompose_3(q)
        back = S.compose_from_angleaxis(t, angle, axis)
        # the same rotation (quaternions agree up to sign)
        assert np.allclose(back[:3], q[:3])
        assert min(np.abs(back[3:] - q[3:]).max(), np.abs(back[3:] + q[3:]).max()) < 1e-12
        t2, R = S.decompose_2(q)
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-12) and abs(np.linalg.det(R) - 1) < 1e-12
        assert np.allclose(R, S.extract_rotation_matrix(q), atol=1e-12)
    assert S.decompose_3([0, 0, 0, 1, 0, 0, 0])[1] == 0.0


def test_angleaxis_matches_scipy(built_lib):
    Rotation = pytest.importorskip("scipy.spatial.transform").Rotation
    for q in _rand_states(50, 2):
        _, angle, axis = S.decompose_3(q)
        rv = Rotation.from_quat([q[4], q[5], q[6], q[3]]).as_rotvec()
        assert np.allclose(angle * axis, rv, atol=1e-12)
        assert np.allclose(S.extract_rotation_matrix(q), Rotation.from_quat([q[4], q[5], q[6], q[3]]).as_matrix(),
                           atol=1e-12)


def test_differential_then_apply_returns_the_target(built_lib):
    import puzzletunneldiscovery_gb300 as pw
    a, b = _rand_states(40, 3), _rand_states(40, 4)
    rows = S.multi_differential(a[0], b, with_se3=True)
    assert rows.shape == (40, 13)
    for i in range(40):
        tr, aav, se3 = S.differential(a[i], b[i])
        got = pw.apply(a[i], tr, aav)
        assert np.allclose(got[:3], b[i, :3], atol=1e-12)
        assert min(np.abs(got[3:] - b[i, 3:]).max(), np.abs(got[3:] + b[i, 3:]).max()) < 1e-9
        assert np.linalg.norm(aav) <= math.pi + 1e-12
        tr0, aav0, se30 = S.differential(a[0], b[i])
        assert np.allclose(rows[i], np.concatenate([tr0, aav0, se30]))


def test_path_metrics_and_interpolation(built_lib):
    import puzzletunneldiscovery_gb300 as pw
    qs = _rand_states(6, 5)
    m = S.path_metrics(qs)
    assert m[0] == 0.0 and np.all(np.diff(m) > 0)
    assert np.isclose(m[2] - m[1], pw.distance(qs[1], qs[2]))
    assert np.array_equal(S.path_interpolate(qs, m, m[3]), pw.interpolate(qs[3], qs[4], 0.0))
    mid = 0.5 * (m[1] + m[2])
    assert np.array_equal(S.path_interpolate(qs, m, mid), pw.interpolate(qs[1], qs[2], (mid - m[1]) / (m[2] - m[1])))
    # past the end (and before the start) the first state comes back, as in the reference
    assert np.array_equal(S.path_interpolate(qs, m, m[-1] + 1.0), qs[0])
