"""Batched samplers around the collision queries: key configurations and touch
configurations.

* ``enum_free_configuration`` / ``sample_free_configuration`` -- the key
  configuration generator of ``UnitWorld::enumFreeConfiguration`` and
  ``sampleFreeConfiguration`` (lib/osr/unit_world.cc:1294-1367): place the robot
  so that a robot surface point touches an environment surface point with
  opposed normals (plus a margin), spin it about the environment normal, and
  keep the spins that are collision free.  The reference checks one spin at a
  time; here every spin of every surface pair is one batched
  ``pw_states_valid`` call.  Callers: src/GP/pipeline/keyconf.py:106-160.
* ``calc_touch`` / ``sample_one_touch`` -- src/GP/pipeline/touchq_util.py:8-27:
  random segments from one root, each stepped to its first contact; here all
  segments are one ``pw_segments_first_contact`` call plus one
  ``pw_segments_contact_states`` call.

The rotations are built from the published formulas (shortest-arc quaternion,
Melax 2000; angle-axis quaternion; Hamilton product) in FP64 numpy.  Verdicts
on the resulting states are the engine's exact ones; agreement of the states
themselves with Eigen's last-ulp rounding is not pinned (the reference cannot
be built here).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .unit_world import UnitWorld


# ---------------------------------------------------------------- quaternion helpers (w, x, y, z), FP64

def quat_mul(a, b):
    """Hamilton product of [..., 4] arrays."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    w1, x1, y1, z1 = np.moveaxis(a, -1, 0)
    w2, x2, y2, z2 = np.moveaxis(b, -1, 0)
    return np.stack([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2], axis=-1)


def quat_rotate(q, v):
    """Rotate [..., 3] vectors by unit quaternions [..., 4]."""
    q = np.asarray(q, np.float64)
    v = np.asarray(v, np.float64)
    w = q[..., :1]
    u = q[..., 1:]
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def quat_from_angle_axis(angle, axis):
    """Quaternion of a rotation by `angle` about unit `axis` (broadcasting)."""
    angle = np.asarray(angle, np.float64)
    axis = np.asarray(axis, np.float64)
    h = 0.5 * angle
    return np.concatenate([np.cos(h)[..., None], np.sin(h)[..., None] * axis], axis=-1)


def quat_between(a, b):
    """Shortest-arc rotation taking direction a to direction b (Melax 2000).
    For opposite directions, a half turn about an axis perpendicular to a."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    v0 = a / np.linalg.norm(a, axis=-1, keepdims=True)
    v1 = b / np.linalg.norm(b, axis=-1, keepdims=True)
    c = np.sum(v0 * v1, axis=-1)
    out = np.empty(v0.shape[:-1] + (4,))
    opp = c < -1.0 + 1e-12
    s = np.sqrt(np.maximum(2.0 * (1.0 + c), 0.0))
    with np.errstate(divide="ignore", invalid="ignore"):
        axis = np.cross(v0, v1) / np.where(opp, 1.0, s)[..., None]
    out[..., 0] = 0.5 * s
    out[..., 1:] = axis
    if np.any(opp):
        v = v0[opp]
        # any unit vector perpendicular to v: cross with the least aligned basis vector
        basis = np.eye(3)[np.argmin(np.abs(v), axis=-1)]
        perp = np.cross(v, basis)
        perp /= np.linalg.norm(perp, axis=-1, keepdims=True)
        out[opp, 0] = 0.0
        out[opp, 1:] = perp
    return out


def compose(trans, rot):
    """osr::compose (osr_state.cc:109-119): translation + normalised quaternion."""
    rot = np.asarray(rot, np.float64)
    rot = rot / np.linalg.norm(rot, axis=-1, keepdims=True)
    return np.concatenate([np.asarray(trans, np.float64), rot], axis=-1)


def apply_batch(from_state, tr, aa):
    """osr::apply (osr_state.cc:244-259) for one state and [N, 3] translations
    and angle-axis vectors: translate, then rotate by the angle-axis on the left."""
    q = np.asarray(from_state, np.float64).reshape(7)
    rot = q[3:] / np.linalg.norm(q[3:])
    tr = np.atleast_2d(np.asarray(tr, np.float64))
    aa = np.atleast_2d(np.asarray(aa, np.float64))
    ang = np.linalg.norm(aa, axis=1)
    axis = np.where(ang[:, None] == 0.0, np.array([1.0, 0.0, 0.0]), aa / np.where(ang == 0.0, 1.0, ang)[:, None])
    r = quat_mul(quat_from_angle_axis(ang, axis), rot[None, :])
    return compose(q[:3][None, :] + tr, r)


# ---------------------------------------------------------------- key configurations

def _touch_states(rob_point, rob_normal, env_point, env_normal, margin, angles):
    """[P, A, 7] states: robot point + margin·normal on env point + margin·normal,
    normals opposed, spun by `angles` [P, A] about the env normal
    (unit_world.cc:1307-1330, 1342-1366)."""
    rp = np.atleast_2d(np.asarray(rob_point, np.float64))
    rn = np.atleast_2d(np.asarray(rob_normal, np.float64))
    ep = np.atleast_2d(np.asarray(env_point, np.float64))
    en = np.atleast_2d(np.asarray(env_normal, np.float64))
    rob_o = rp + rn * margin
    env_o = ep + en * margin
    rot1 = quat_between(rn, -en)                                     # [P, 4]
    rot2 = quat_from_angle_axis(angles, en[:, None, :])              # [P, A, 4]
    acc = quat_mul(rot2, rot1[:, None, :])                           # [P, A, 4]
    trans = env_o[:, None, :] - quat_rotate(acc, np.broadcast_to(rob_o[:, None, :], acc.shape[:-1] + (3,)))
    return compose(trans, acc)


def enum_free_configurations(uw: UnitWorld, rob_points, rob_normals, env_points, env_normals, margin: float,
                             denominator: int, only_median: bool = False):
    """enumFreeConfiguration for P surface pairs at once; returns a list of P
    arrays [m_i, 7] (unit_world.cc:1336-1389).  With only_median, each run of
    consecutive free spins contributes its middle spin, and, as in the
    reference, a run still open at the last spin contributes nothing."""
    if denominator <= 0:
        raise ValueError("denominator must be positive")
    P = np.atleast_2d(np.asarray(rob_points)).shape[0]
    delta = 2 * math.pi / float(denominator)
    angles = np.broadcast_to(np.arange(denominator, dtype=np.float64) * delta, (P, denominator))
    qs = _touch_states(rob_points, rob_normals, env_points, env_normals, margin, angles)
    flat = torch.from_numpy(np.ascontiguousarray(qs.reshape(-1, 7))).to(uw._device)
    valid = uw.is_valid_states(flat).cpu().numpy().reshape(P, denominator)
    return _free_spins(qs, valid, only_median)


def _free_spins(qs, valid, only_median):
    """The free spins of every surface pair ([P, A, 7] states, [P, A] verdicts):
    all of them, or the middle spin of every run of consecutive free spins that
    ends before the last spin (unit_world.cc:1367-1386)."""
    P, A = valid.shape
    if not only_median:
        rows, cols = np.nonzero(valid)
    else:
        v = valid.astype(np.int8)
        prev = np.zeros_like(v)
        prev[:, 1:] = v[:, :-1]
        nxt = np.zeros_like(v)
        nxt[:, :-1] = v[:, 1:]
        sr, sc = np.nonzero(v & (1 - prev))            # run starts, row-major
        er, ec = np.nonzero(v & (1 - nxt))             # run ends, in the same order
        keep = ec < A - 1                              # a run still open at the last spin is dropped
        rows, cols = sr[keep], (sc + (ec - sc + 1) // 2)[keep]
    picked = qs[rows, cols]
    bounds = np.searchsorted(rows, np.arange(P + 1))
    return [picked[bounds[p]:bounds[p + 1]] if bounds[p + 1] > bounds[p] else np.zeros((0, 7)) for p in range(P)]


def enum_free_configuration(uw: UnitWorld, rob_surface_point, rob_surface_normal, env_surface_point,
                            env_surface_normal, margin: float, denominator: int, only_median: bool = False):
    """UnitWorld::enumFreeConfiguration for one surface pair (pyosr signature)."""
    return enum_free_configurations(uw, rob_surface_point, rob_surface_normal, env_surface_point,
                                    env_surface_normal, margin, denominator, only_median)[0]


def sample_free_configurations(uw: UnitWorld, rob_points, rob_normals, env_points, env_normals, margin: float,
                               max_trials: int = 16, rng=None):
    """sampleFreeConfiguration for P surface pairs: up to max_trials + 1 random
    spins each, all checked in one batch; returns ([P, 7] states, [P] found).
    Where no spin is free, the state is the last one tried, as in the
    reference (unit_world.cc:1294-1334).  The reference's max_trials < 0 (try
    forever) is served by calling again for the pairs not found."""
    if max_trials < 0:
        raise ValueError("max_trials < 0 loops forever in the reference; pass a bound and retry the misses")
    rng = np.random.default_rng() if rng is None else rng
    P = np.atleast_2d(np.asarray(rob_points)).shape[0]
    A = max_trials + 1
    angles = rng.uniform(0.0, 2 * math.pi, (P, A))
    qs = _touch_states(rob_points, rob_normals, env_points, env_normals, margin, angles)
    flat = torch.from_numpy(np.ascontiguousarray(qs.reshape(-1, 7))).to(uw._device)
    valid = uw.is_valid_states(flat).cpu().numpy().reshape(P, A)
    found = valid.any(axis=1)
    first = np.where(found, np.argmax(valid, axis=1), A - 1)
    return qs[np.arange(P), first], found


def sample_free_configuration(uw: UnitWorld, rob_surface_point, rob_surface_normal, env_surface_point,
                              env_surface_normal, margin: float, max_trials: int = 16, rng=None):
    """UnitWorld::sampleFreeConfiguration for one surface pair."""
    q, _ = sample_free_configurations(uw, rob_surface_point, rob_surface_normal, env_surface_point,
                                      env_surface_normal, margin, max_trials, rng)
    return q[0]


# ---------------------------------------------------------------- touch configurations

def random_on_sphere(n, scale=1.0, rng=None):
    """n points on the sphere of radius `scale` (Marsaglia 1972), as uw_random.random_on_sphere."""
    rng = np.random.default_rng() if rng is None else rng
    out = np.empty((0, 2))
    while out.shape[0] < n:
        x = 2.0 * (rng.random((2 * (n - out.shape[0]) + 8, 2)) - 0.5)
        l2 = np.sum(x * x, axis=1)
        out = np.concatenate([out, x[l2 < 1]])
    x1, x2 = out[:n, 0], out[:n, 1]
    l2 = x1 * x1 + x2 * x2
    return np.stack([2 * x1 * np.sqrt(1 - l2), 2 * x2 * np.sqrt(1 - l2), 1 - 2 * l2], axis=1) * scale


def random_within_sphere(n, scale=1.0, rng=None):
    """n points uniform in the ball of radius `scale` (rejection from the cube)."""
    rng = np.random.default_rng() if rng is None else rng
    out = np.empty((0, 3))
    while out.shape[0] < n:
        x = 2.0 * (rng.random((2 * (n - out.shape[0]) + 8, 3)) - 0.5)
        out = np.concatenate([out, x[np.sum(x * x, axis=1) <= 1]])
    return out[:n] * scale


def calc_touch(uw: UnitWorld, q0, batch_size: int, stepping: float, rng=None):
    """touchq_util.calc_touch: batch_size random segments from q0 (unit
    translation on the sphere, rotation uniform within 2π), each stepped to its
    first contact.  Returns the reference's five arrays: last free states
    [B, 7], contact states [B, 7], done [B], last_tau [B], tau [B]."""
    tr = random_on_sphere(batch_size, 1.0, rng)
    aa = random_within_sphere(batch_size, 2 * math.pi, rng)
    to = apply_batch(q0, tr, aa)
    q0s = np.broadcast_to(np.asarray(q0, np.float64).reshape(1, 7), (batch_size, 7))
    dev = uw._device
    a = torch.from_numpy(np.ascontiguousarray(q0s)).to(dev)
    b = torch.from_numpy(np.ascontiguousarray(to)).to(dev)
    lf, st, done, lt, tt = uw.transit_states_to_with_contact(a, b, stepping)
    return [lf.cpu().numpy(), st.cpu().numpy(), done.cpu().numpy(), lt.cpu().numpy(), tt.cpu().numpy()]


def calc_touch_batch(uw: UnitWorld, keys, per_key: int, stepping: float, rng=None):
    """calc_touch for K keys at once (the loop over keys of keyconf.py:306-316 and
    preprocess_key.py:174): per_key random segments from every key (translation
    on the unit sphere, rotation uniform within 2π, drawn for all keys in one
    go), all stepped to their first contact in one batch.  Row i * per_key + j
    of the five arrays belongs to key i.  Returns (the five arrays, the
    segments' end states)."""
    keys = np.atleast_2d(np.asarray(keys, np.float64))
    rng = np.random.default_rng() if rng is None else rng
    K = keys.shape[0]
    frm = np.repeat(keys, per_key, axis=0)
    tr = random_on_sphere(K * per_key, 1.0, rng)
    aa = random_within_sphere(K * per_key, 2 * math.pi, rng)
    to = apply_rows(frm, tr, aa)
    dev = uw._device
    a = torch.from_numpy(frm).to(dev)
    b = torch.from_numpy(to).to(dev)
    lf, st, done, lt, tt = uw.transit_states_to_with_contact(a, b, stepping)
    return [lf.cpu().numpy(), st.cpu().numpy(), done.cpu().numpy(), lt.cpu().numpy(), tt.cpu().numpy()], to


def apply_rows(states, tr, aa):
    """osr::apply (osr_state.cc:244-259) row by row: state i translated by tr[i] and
    rotated on the left by the angle-axis vector aa[i]."""
    states = np.atleast_2d(np.asarray(states, np.float64))
    rot = states[:, 3:] / np.linalg.norm(states[:, 3:], axis=1, keepdims=True)
    ang = np.linalg.norm(aa, axis=1)
    axis = np.where(ang[:, None] == 0.0, np.array([1.0, 0.0, 0.0]), aa / np.where(ang == 0.0, 1.0, ang)[:, None])
    r = quat_mul(quat_from_angle_axis(ang, axis), rot)
    return compose(states[:, :3] + tr, r)


def sample_one_touch(uw: UnitWorld, q0, stepping: float, rng=None):
    """touchq_util.sample_one_touch: one random segment from q0 to its first contact."""
    r = calc_touch(uw, q0, 1, stepping, rng)
    return r[0][0], r[1][0], bool(r[2][0]), r[3][0], r[4][0]
