"""pyosr's module-level state helpers (lib/pyosr/module.cc:77-99, lib/osr/osr_state.cc).

Host-side numpy restatements of the functions the planner's scripts call next
to the collision queries: decompositions and compositions of states
(w-first quaternions), the SE(3) differential between two states, and the
arc-length parametrisation of a path.  Quaternion / angle-axis conversions
follow Eigen's documented conventions (angle-axis from a quaternion: angle
2 atan2(|v|, |w|), axis v / |v| with the sign of w; identity -> angle 0, axis x).
"""
from __future__ import annotations

import math

import numpy as np

from .unit_world import distance, interpolate

__all__ = ["decompose", "decompose_2", "decompose_3", "compose", "compose_from_angleaxis", "extract_rotation_matrix",
           "differential", "multi_differential", "path_metrics", "path_interpolate", "quat_mul", "quat_to_matrix",
           "quat_from_angleaxis", "angleaxis_from_quat"]


def _state(q) -> np.ndarray:
    q = np.asarray(q, dtype=np.float64).reshape(-1)
    if q.shape != (7,):
        raise ValueError("a state has 7 values [x, y, z, w, qx, qy, qz]")
    return q


def quat_mul(a, b) -> np.ndarray:
    """Hamilton product of (w, x, y, z) quaternions."""
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])


def quat_inverse(q) -> np.ndarray:
    q = np.asarray(q, dtype=np.float64)
    return np.array([q[0], -q[1], -q[2], -q[3]]) / float(np.dot(q, q))


def quat_to_matrix(q) -> np.ndarray:
    """Rotation matrix of a (w, x, y, z) quaternion by the unit-quaternion formula
    applied to its coefficients as given (no normalisation)."""
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def quat_from_angleaxis(angle: float, axis) -> np.ndarray:
    """(cos(a/2), sin(a/2) axis): the axis is taken as given (unit length assumed)."""
    axis = np.asarray(axis, dtype=np.float64).reshape(3)
    h = 0.5 * float(angle)
    return np.concatenate([[math.cos(h)], math.sin(h) * axis])


def angleaxis_from_quat(q):
    """(angle, axis) of a quaternion, any norm."""
    q = np.asarray(q, dtype=np.float64)
    v = q[1:]
    n = float(np.linalg.norm(v))
    if n == 0.0:
        return 0.0, np.array([1.0, 0.0, 0.0])
    angle = 2.0 * math.atan2(n, abs(q[0]))
    axis = (-v if q[0] < 0 else v) / n
    return angle, axis


def decompose(state):
    """(translation, unit quaternion (w, x, y, z)) of a state (osr_state.cc:85-92)."""
    q = _state(state)
    r = q[3:7] / np.linalg.norm(q[3:7])
    return q[:3].copy(), r


def decompose_2(state):
    """(translation, rotation matrix) (osr_state.cc:94-99)."""
    t, r = decompose(state)
    return t, quat_to_matrix(r)


def decompose_3(state):
    """(translation, angle, axis) (osr_state.cc:101-107)."""
    t, r = decompose(state)
    angle, axis = angleaxis_from_quat(r)
    return t, angle, axis


def compose(base, rot) -> np.ndarray:
    """State from a translation and a quaternion, normalised (osr_state.cc:109-119)."""
    r = np.asarray(rot, dtype=np.float64)
    return np.concatenate([np.asarray(base, dtype=np.float64).reshape(3), r / np.linalg.norm(r)])


def compose_from_angleaxis(tr, angle: float, axis) -> np.ndarray:
    """osr_state.cc:121-127."""
    return compose(tr, quat_from_angleaxis(angle, axis))


def extract_rotation_matrix(state) -> np.ndarray:
    """Rotation matrix of the state's quaternion as given (osr_state.cc:170-175)."""
    q = _state(state)
    return quat_to_matrix(q[3:7])


def _angular_distance(a, b) -> float:
    a = np.asarray(a) / np.linalg.norm(a)
    b = np.asarray(b) / np.linalg.norm(b)
    d = quat_mul(a, quat_inverse(b))
    return 2.0 * math.atan2(float(np.linalg.norm(d[1:])), abs(float(d[0])))


def differential(from_state, to_state):
    """(translation, angle-axis vector, composed state) taking from -> to
    (osr_state.cc:177-226), with the reference's round-trip checks: a rotation
    that does not map back within 1e-3 rad raises RuntimeError."""
    a, b = _state(from_state), _state(to_state)
    tr = b[:3] - a[:3]
    rot_from, rot_to = a[3:7], b[3:7]
    rot_delta = quat_mul(rot_to, quat_inverse(rot_from))
    angle, axis = angleaxis_from_quat(rot_delta)
    aav = axis * angle
    if _angular_distance(rot_to, quat_mul(quat_from_angleaxis(angle, axis), rot_from)) > 1e-3:
        raise RuntimeError("differential is buggy")
    n = float(np.linalg.norm(aav))
    ax = aav / n if n > 0 else aav
    if _angular_distance(rot_to, quat_mul(quat_from_angleaxis(n, ax), rot_from)) > 1e-3:
        raise RuntimeError("differential is buggy in aa->quat")
    return tr, aav, compose(tr, rot_delta)


def multi_differential(from_state, tos, with_se3: bool = False) -> np.ndarray:
    """Rows [translation (3), angle-axis (3)] (+ the composed state (7) with
    with_se3) of differential(from, tos[i]) (osr_state.cc:228-242)."""
    tos = np.asarray(tos, dtype=np.float64).reshape(-1, 7)
    out = np.zeros((tos.shape[0], 13 if with_se3 else 6))
    for i, t in enumerate(tos):
        tr, aav, se3 = differential(from_state, t)
        out[i, :3], out[i, 3:6] = tr, aav
        if with_se3:
            out[i, 6:] = se3
    return out


def path_metrics(qs) -> np.ndarray:
    """Cumulative state distance along a path (osr_state.cc:46-58)."""
    qs = np.asarray(qs, dtype=np.float64).reshape(-1, 7)
    m = np.zeros(qs.shape[0])
    d = 0.0
    for i in range(1, qs.shape[0]):
        d += distance(qs[i - 1], qs[i])
        m[i] = d
    return m


def path_interpolate(qs, metrics, tau: float) -> np.ndarray:
    """The state at arc length tau (osr_state.cc:60-83): the first segment with
    metrics[i] <= tau < metrics[i+1], interpolated; the first state if none."""
    qs = np.asarray(qs, dtype=np.float64).reshape(-1, 7)
    metrics = np.asarray(metrics, dtype=np.float64).reshape(-1)
    for i in range(qs.shape[0] - 1):
        if metrics[i] <= tau < metrics[i + 1]:
            d = metrics[i + 1] - metrics[i]
            t = 0.0 if d < 1e-6 else (tau - metrics[i]) / d
            return interpolate(qs[i], qs[i + 1], t)
    return qs[0].copy()
