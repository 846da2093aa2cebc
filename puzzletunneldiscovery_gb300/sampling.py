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

The key-configuration states are built on the device (``pw_keyconf_states``)
from Eigen's published forms (shortest-arc quaternion, angle-axis quaternion,
Hamilton product, quaternion-vector product), every FP64 operation rounded on
its own in a fixed order, so the oracle's ``or_keyconf_states`` gives the same
bits; agreement with Eigen's own last-ulp rounding is not pinned (the
reference cannot be built here).  The touch segments' random targets are drawn
on the device too (``pw_touch_targets``).  The numpy helpers below (quaternion
products, ``apply_batch``, ``apply_rows``) serve callers that build single
states on the host.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib
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


def quat_from_angle_axis(angle, axis):
    """Quaternion of a rotation by `angle` about unit `axis` (broadcasting)."""
    angle = np.asarray(angle, np.float64)
    axis = np.asarray(axis, np.float64)
    h = 0.5 * angle
    return np.concatenate([np.cos(h)[..., None], np.sin(h)[..., None] * axis], axis=-1)


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

def _pairs_dev(dev, *arrays):
    return [torch.from_numpy(np.ascontiguousarray(np.atleast_2d(np.asarray(x, np.float64)))).to(dev) for x in arrays]


def keyconf_states(uw: UnitWorld, rob_points, rob_normals, env_points, env_normals, margin: float, half_cos,
                   half_sin) -> torch.Tensor:
    """Device tensor [P, A, 7] of the candidate states of P surface pairs and A
    spins (unit_world.cc:1301-1330, 1342-1366): robot point + margin x normal on
    env point + margin x normal, normals opposed, spun about the env normal by
    the angle whose half has cosine half_cos and sine half_sin ([A] for every
    pair, or [P, A])."""
    dev = uw._device
    rp, rn, ep, en = _pairs_dev(dev, rob_points, rob_normals, env_points, env_normals)
    P = rp.shape[0]
    hc = np.ascontiguousarray(half_cos, dtype=np.float64)
    hs = np.ascontiguousarray(half_sin, dtype=np.float64)
    per_pair = hc.ndim == 2
    if per_pair and hc.shape[0] != P:
        raise ValueError("half-angle tables must be [A] or [P, A]")
    A = hc.shape[-1]
    thc, ths = torch.from_numpy(hc).to(dev), torch.from_numpy(hs).to(dev)
    out = torch.empty((P, A, 7), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(uw._L.pw_keyconf_states(rp.data_ptr(), rn.data_ptr(), ep.data_ptr(), en.data_ptr(), P,
                                       float(margin), thc.data_ptr(), ths.data_ptr(), A, int(per_pair),
                                       out.data_ptr(), stream), "pw_keyconf_states")
    return out


def enum_free_configurations(uw: UnitWorld, rob_points, rob_normals, env_points, env_normals, margin: float,
                             denominator: int, only_median: bool = False):
    """enumFreeConfiguration for P surface pairs at once; returns a list of P
    arrays [m_i, 7] (unit_world.cc:1336-1389).  With only_median, each run of
    consecutive free spins contributes its middle spin, and, as in the
    reference, a run still open at the last spin contributes nothing."""
    if denominator <= 0:
        raise ValueError("denominator must be positive")
    delta = 2 * math.pi / float(denominator)
    half = [0.5 * (i * delta) for i in range(denominator)]      # AngleAxis(i * delta, normal)
    qs = keyconf_states(uw, rob_points, rob_normals, env_points, env_normals, margin,
                        [math.cos(h) for h in half], [math.sin(h) for h in half])
    P = qs.shape[0]
    valid = uw.is_valid_states(qs.view(-1, 7)).cpu().numpy().reshape(P, denominator)
    return _free_spins(qs, valid, only_median)


def _free_spins(qs, valid, only_median):
    """The free spins of every surface pair ([P, A, 7] states on the device, [P, A]
    verdicts): all of them, or the middle spin of every run of consecutive free
    spins that ends before the last spin (unit_world.cc:1367-1386)."""
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
    idx = torch.from_numpy((rows * A + cols).astype(np.int64)).to(qs.device)
    picked = qs.reshape(-1, 7).index_select(0, idx).cpu().numpy()
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
    half = 0.5 * rng.uniform(0.0, 2 * math.pi, (P, A))
    qs = keyconf_states(uw, rob_points, rob_normals, env_points, env_normals, margin, np.cos(half), np.sin(half))
    valid = uw.is_valid_states(qs.view(-1, 7)).cpu().numpy().reshape(P, A)
    found = valid.any(axis=1)
    first = np.where(found, np.argmax(valid, axis=1), A - 1)
    idx = torch.from_numpy((np.arange(P) * A + first).astype(np.int64)).to(qs.device)
    return qs.view(-1, 7).index_select(0, idx).cpu().numpy(), found


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


def touch_segments(uw: UnitWorld, keys, per_key: int, seed: int):
    """Device tensors (from, to) [K * per_key, 7] of the random segments of
    touchq_util.calc_touch for K keys: row i * per_key + j goes from key i to
    the key translated by a random point of the unit sphere and rotated on the
    left by a rotation vector uniform in the ball of radius 2 pi (osr::apply)."""
    dev = uw._device
    k = torch.from_numpy(np.ascontiguousarray(np.atleast_2d(np.asarray(keys, np.float64)))).to(dev)
    n = k.shape[0] * per_key
    frm = torch.empty((n, 7), dtype=torch.float64, device=dev)
    to = torch.empty((n, 7), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(uw._L.pw_touch_targets(k.data_ptr(), k.shape[0], int(per_key), int(seed) & (2 ** 64 - 1),
                                      frm.data_ptr(), to.data_ptr(), stream), "pw_touch_targets")
    return frm, to


def _seed(rng):
    rng = np.random.default_rng() if rng is None else rng
    return int(rng.integers(0, 2 ** 63))


def calc_touch(uw: UnitWorld, q0, batch_size: int, stepping: float, rng=None):
    """touchq_util.calc_touch: batch_size random segments from q0 (unit
    translation on the sphere, rotation uniform within 2 pi), each stepped to its
    first contact.  Returns the reference's five arrays: last free states
    [B, 7], contact states [B, 7], done [B], last_tau [B], tau [B]."""
    res, _ = calc_touch_batch(uw, np.asarray(q0, np.float64).reshape(1, 7), batch_size, stepping, rng)
    return res


def calc_touch_batch(uw: UnitWorld, keys, per_key: int, stepping: float, rng=None):
    """calc_touch for K keys at once (the loop over keys of keyconf.py:306-316 and
    preprocess_key.py:174): per_key random segments from every key, drawn on the
    device (``touch_segments``, seeded from rng), all stepped to their first
    contact in one batch.  Row i * per_key + j of the five arrays belongs to key
    i.  Returns (the five arrays, the segments' end states as a device tensor)."""
    frm, to = touch_segments(uw, keys, per_key, _seed(rng))
    lf, st, done, lt, tt = uw.transit_states_to_with_contact(frm, to, stepping)
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
