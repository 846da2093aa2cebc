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
"""
from __future__ import annotations

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
