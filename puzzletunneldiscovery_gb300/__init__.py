"""GB300 engine for the collision-query path of pyosr's UnitWorld.

``UnitWorld`` keeps pyosr's method names and semantics (lib/pyosr/module.cc:127-250)
and adds batched tensor methods; queries run in libpwcollide.so (include/pw_collide.h).
"""
from .unit_world import (GEO_ENV, GEO_ROB, STATE_DIMENSION, PwError, UnitWorld, apply, distance,  # noqa: F401
                         get_identity_state_vector, interpolate, multi_distance, segment_step_state,
                         state_transform)

from .state_ops import (compose_from_angleaxis, decompose_2, decompose_3, differential,  # noqa: F401,E402
                        extract_rotation_matrix, multi_differential, path_interpolate, path_metrics)
from . import objio as _objio  # noqa: E402


def load_obj_1(fn: str):
    """pyosr.load_obj_1 (osr_util.h:53): (V, F) of an OBJ file (vertices as float64)."""
    V, F = _objio.load_obj(fn)
    return V.astype("float64"), F.astype("int32")


def save_obj_1(V, F, fn: str) -> None:
    """pyosr.save_obj_1 (osr_util.h:27): write a triangle OBJ."""
    _objio.save_obj(fn, V, F)


__all__ = ["compose_from_angleaxis", "decompose_2", "decompose_3", "differential", "extract_rotation_matrix",
           "multi_differential", "path_interpolate", "path_metrics", "load_obj_1", "save_obj_1",
           "UnitWorld", "GEO_ENV", "GEO_ROB", "STATE_DIMENSION", "PwError", "distance", "multi_distance",
           "interpolate", "segment_step_state", "apply", "get_identity_state_vector", "state_transform"]
