"""GB300 engine for the collision-query path of pyosr's UnitWorld.

``UnitWorld`` keeps pyosr's method names and semantics (lib/pyosr/module.cc:127-250)
and adds batched tensor methods; queries run in libpwcollide.so (include/pw_collide.h).
"""
from .unit_world import (GEO_ENV, GEO_ROB, STATE_DIMENSION, PwError, UnitWorld, apply, distance,  # noqa: F401
                         get_identity_state_vector, interpolate, multi_distance, segment_step_state,
                         state_transform)

__all__ = ["UnitWorld", "GEO_ENV", "GEO_ROB", "STATE_DIMENSION", "PwError", "distance", "multi_distance",
           "interpolate", "segment_step_state", "apply", "get_identity_state_vector", "state_transform"]
