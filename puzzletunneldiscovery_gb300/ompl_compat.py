"""Batch screening of OMPL-frame states and motions on the GPU.

pyse3ompl's ``OmplDriver.validate_states`` and ``validate_motion_pairs``
(lib/pyse3ompl/ompldriver.cc:566-621, callers src/GP/pipeline/solve2.py:54,219)
check the planner's key configurations and candidate edges, one state or one
motion at a time through OMPL's space information.  Here both are one batched
call on a world set up for the same puzzle:

* ``validate_states``: OMPL states (x, y, z, qx, qy, qz, qw in the puzzle's
  frame, about the robot's OMPL centre) are converted with
  translateOMPLStateToUnitState (unit_world.cc:689-711) and checked with
  ``pw_states_valid``.  Collision is invariant under the unit frame's
  scaling, so the verdicts are the engine's exact ones.
* ``validate_motion_pairs``: both ends are converted the same way and the
  motion is checked with ``pw_segments_first_contact`` in is_valid_transition
  mode at ``verify_delta`` (unit frame).  This is UnitWorld's stepping rule
  (unit_world.cc:477-486), not OMPL's discrete motion validator, whose
  resolution is a fraction of the state space's extent: the two agree on
  motions that are free or collide over more than one step, and may differ on
  contacts thinner than a step of either rule.

Both return int32 vectors with 1 = valid, as the reference does.

``OmplDriver`` is the validation half of pyse3ompl's driver with OMPL's own
motion rule: ``set_bb`` / ``set_cdres`` (ompldriver.h:108-116) give the state
space's translation bounds and collision resolution, and
``validate_motion_pairs`` checks each motion as OMPL's discrete motion
validator does (``pw_ompl_check_motions``: the target state and the states
k / nd along OMPL's SE(3) interpolation, nd from the resolution times each
component's extent), all motions of a batch in one call.  The states are
checked in passes over the motions still valid (the targets, then dyadic
levels of k, each halving the spacing of the states checked so far), which
skips most states of colliding motions as OMPL's early exit does, without
changing any verdict.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .unit_world import UnitWorld


def _ompl_states(q) -> np.ndarray:
    q = np.asarray(q, dtype=np.float64)
    if q.ndim != 2 or q.shape[1] != 7:
        raise ValueError("expected OMPL states of shape [n, 7] (x, y, z, qx, qy, qz, qw)")
    return np.ascontiguousarray(q)


def validate_states(uw: UnitWorld, qs_ompl) -> np.ndarray:
    """OmplDriver::validateStates for a batch (int32, 1 = collision free)."""
    q = _ompl_states(qs_ompl)
    if q.shape[0] == 0:
        return np.zeros(0, dtype=np.int32)
    u = torch.from_numpy(uw.translate_ompl_to_unit(q)).to(uw._device)
    return uw.is_valid_states(u).cpu().numpy().astype(np.int32)


def validate_motion_pairs(uw: UnitWorld, qs0, qs1, verify_delta: float = 0.001) -> np.ndarray:
    """OmplDriver::validateMotionPairs for aligned batches (int32, 1 = the motion is
    free), stepped with UnitWorld's rule at verify_delta (unit frame); rows beyond
    the shorter batch are 0, as in the reference."""
    a, b = _ompl_states(qs0), _ompl_states(qs1)
    m = min(a.shape[0], b.shape[0])
    out = np.zeros(a.shape[0], dtype=np.int32)
    if m == 0:
        return out
    ua = torch.from_numpy(uw.translate_ompl_to_unit(a[:m])).to(uw._device)
    ub = torch.from_numpy(uw.translate_ompl_to_unit(b[:m])).to(uw._device)
    steps = uw.first_contact_steps(ua, ub, verify_delta, _lib.PW_SEG_TRANSITION).cpu().numpy()
    out[:m] = (steps == _lib.PW_STEP_FREE).astype(np.int32)
    return out


def _bb(lo, hi):
    lo = np.ascontiguousarray(np.asarray(lo, dtype=np.float64).reshape(-1))
    hi = np.ascontiguousarray(np.asarray(hi, dtype=np.float64).reshape(-1))
    if lo.shape != (3,) or hi.shape != (3,):
        raise ValueError("bounds must have 3 entries each")
    return lo, hi


def _motion_args(uw: UnitWorld, qs0, qs1):
    a, b = _ompl_states(qs0), _ompl_states(qs1)
    m = min(a.shape[0], b.shape[0])
    ta = torch.from_numpy(a[:m]).to(uw._device)
    tb = torch.from_numpy(b[:m]).to(uw._device)
    return a.shape[0], m, ta, tb


def _stream_of(device):
    d = torch.device(device)
    return torch.cuda.current_stream(d).cuda_stream if d.type == "cuda" else None


def _check_motions_dev(uw: UnitWorld, ta: torch.Tensor, tb: torch.Tensor, lo: np.ndarray, hi: np.ndarray,
                       cdres: float):
    """pw_ompl_check_motions on [m, 7] float64 OMPL-frame batches already on the
    world's device: (uint8 verdicts [m] on the device, states checked)."""
    m = ta.shape[0]
    valid = torch.empty(m, dtype=torch.uint8, device=ta.device)
    checked = ctypes.c_int64()
    dp = ctypes.POINTER(ctypes.c_double)
    _lib.check(uw._L.pw_ompl_check_motions(uw._h, ta.data_ptr(), tb.data_ptr(), m, lo.ctypes.data_as(dp),
                                           hi.ctypes.data_as(dp), float(cdres), valid.data_ptr(),
                                           ctypes.pointer(checked), _stream_of(ta.device)),
               "check_motions_discrete")
    return valid, int(checked.value)


def check_motions_discrete(uw: UnitWorld, qs0, qs1, lo, hi, cdres: float):
    """OMPL's discrete motion check of aligned OMPL-frame motions qs0[i] -> qs1[i]
    in an SE(3) space bounded by lo / hi at collision resolution cdres.  Returns
    (int32 verdicts, 1 = the motion is valid, rows beyond the shorter batch 0;
    the number of states checked)."""
    lo, hi = _bb(lo, hi)
    n, m, ta, tb = _motion_args(uw, qs0, qs1)
    out = np.zeros(n, dtype=np.int32)
    if m == 0:
        return out, 0
    valid, checked = _check_motions_dev(uw, ta, tb, lo, hi, cdres)
    out[:m] = valid.cpu().numpy()
    return out, checked


def motion_states(uw: UnitWorld, qs0, qs1, lo, hi, cdres: float):
    """Every unit-frame state check_motions_discrete may check: (states [T, 7] on
    the device, offsets [m + 1]); motion i's rows are offsets[i] .. offsets[i + 1] - 1,
    its target first, then k = 1 .. nd - 1."""
    lo, hi = _bb(lo, hi)
    _, m, ta, tb = _motion_args(uw, qs0, qs1)
    dev = uw._device
    offs = torch.zeros(m + 1, dtype=torch.int64, device=dev)
    if m == 0:
        return torch.zeros((0, 7), dtype=torch.float64, device=dev), offs
    dp = ctypes.POINTER(ctypes.c_double)
    total = ctypes.c_int64()
    args = (uw._h, ta.data_ptr(), tb.data_ptr(), m, lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), float(cdres))
    stream = _stream_of(dev)
    dummy = torch.zeros((1, 7), dtype=torch.float64, device=dev)
    # first call sizes the listing (PW_ERR_CAPACITY at capacity 0), the second fills it
    rc = uw._L.pw_ompl_motion_states(*args, 0, dummy.data_ptr(), offs.data_ptr(), ctypes.pointer(total), stream)
    if rc not in (_lib.PW_OK, _lib.PW_ERR_CAPACITY):
        _lib.check(rc, "motion_states")
    states = torch.empty((max(int(total.value), 1), 7), dtype=torch.float64, device=dev)
    _lib.check(uw._L.pw_ompl_motion_states(*args, int(total.value), states.data_ptr(), offs.data_ptr(),
                                           ctypes.pointer(total), stream), "motion_states")
    return states[:int(total.value)], offs


class OmplDriver:
    """The validation calls of pyse3ompl's OmplDriver (ompldriver.h:108-116,
    ompldriver.cc:566-621) on a UnitWorld loaded with the same puzzle's meshes:
    set_bb, set_cdres, validate_states and validate_motion_pairs, the last with
    OMPL's discrete motion rule."""

    def __init__(self, uw: UnitWorld):
        self.uw = uw
        self.lo = self.hi = None
        self.cdres = None
        self.last_states_checked = 0

    def set_bb(self, mins, maxs) -> None:
        self.lo, self.hi = _bb(mins, maxs)

    def set_cdres(self, cdres: float) -> None:
        self.cdres = float(cdres)

    def validate_states(self, qs0) -> np.ndarray:
        return validate_states(self.uw, qs0)

    def _ready(self, what: str) -> None:
        if self.lo is None or self.cdres is None:
            raise RuntimeError("%s needs set_bb and set_cdres first" % what)

    def validate_motion_pairs(self, qs0, qs1) -> np.ndarray:
        self._ready("validate_motion_pairs")
        out, self.last_states_checked = check_motions_discrete(self.uw, qs0, qs1, self.lo, self.hi, self.cdres)
        return out

    def check_pairs(self, keys: torch.Tensor, from_idx: torch.Tensor, to_idx: torch.Tensor) -> torch.Tensor:
        """validate_motion_pairs(keys[from_idx], keys[to_idx]) with the keys and
        the indices already on the device: a bool tensor, no host round trip."""
        self._ready("check_pairs")
        if from_idx.shape != to_idx.shape:
            raise ValueError("from and to indices differ in length")
        if from_idx.numel() == 0:
            self.last_states_checked = 0
            return torch.zeros(0, dtype=torch.bool, device=keys.device)
        ta = keys.index_select(0, from_idx).contiguous()
        tb = keys.index_select(0, to_idx).contiguous()
        valid, self.last_states_checked = _check_motions_dev(self.uw, ta, tb, self.lo, self.hi, self.cdres)
        return valid.bool()
