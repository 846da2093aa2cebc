"""ctypes binding of libpwcollide.so (include/pw_collide.h).

The library is built in-tree by ``puzzletunneldiscovery_gb300.build``.  There
is no fallback: if the library is missing or cannot be loaded, every query
raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

PW_OK = 0
PW_ERR_INVALID_ARG = 1
PW_ERR_CUDA = 2
PW_ERR_NO_MODEL = 3
PW_ERR_OUT_OF_MEMORY = 4
PW_ERR_CAPACITY = 5
PW_ERR_INTERNAL = 6

PW_GEO_ENV = 0
PW_GEO_ROB = 1
PW_SEG_TRANSIT = 0
PW_SEG_TRANSITION = 1
PW_STEP_FREE = -1
PW_STEP_NONE = -2
PW_STEP_INVALID = -3
PW_BOXES_ALIGNED = 0
PW_BOXES_ORIENTED = 1
PW_BVH_TOPDOWN = 0
PW_BVH_MORTON = 1
PW_BVH_SAH = 2
PW_PHASES_AUTO = 0
PW_PHASES_OFF = 1
PW_PHASES_ON = 2

# every entry point declared in include/pw_collide.h
EXPORTS = (
    "pw_last_error", "pw_world_create", "pw_world_destroy", "pw_world_load_env", "pw_world_load_robot",
    "pw_world_enforce_robot_center", "pw_world_scale_to_unit", "pw_world_angle_model",
    "pw_world_set_perturbation", "pw_world_get_perturbation", "pw_world_info_get", "pw_world_cd_vertices",
    "pw_world_cd_faces", "pw_states_valid", "pw_states_disentangled", "pw_segments_first_contact",
    "pw_intersecting_segments", "pw_world_translate_to_unit", "pw_world_translate_from_unit",
    "pw_world_translate_ompl_to_unit", "pw_world_translate_unit_to_ompl", "pw_world_last_stats",
    "pw_state_distance", "pw_state_interpolate", "pw_segment_step_state", "pw_states_valid_noalloc",
    "pw_segments_contact_states", "pw_world_segments_contact_states", "pw_world_set_graph_mode",
    "pw_segments_reserve", "pw_world_set_launch_config",
    "pw_world_get_launch_config", "pw_expansion_crossings", "pw_world_scratch_epoch", "pw_expand_states",
    "pw_ompl_check_motions", "pw_ompl_motion_states", "pw_world_set_node_boxes", "pw_world_get_node_boxes",
    "pw_world_set_segment_phases", "pw_world_get_segment_phases", "pw_keyconf_states", "pw_touch_targets",
    "pw_world_set_bvh", "pw_world_get_bvh",
    "pw_intersecting_segments_batch",
    # include/pw_mlp.h
    "pw_mlp_create", "pw_mlp_destroy", "pw_mlp_num_params", "pw_mlp_get_params", "pw_mlp_set_params",
    "pw_mlp_get_grads", "pw_mlp_predict", "pw_mlp_gradients", "pw_mlp_train_step", "pw_mlp_predict_mma",
    "pw_mlp_check", "pw_select_top", "pw_mlp_score", "pw_mlp_set_training_kernels", "pw_mlp_get_adam",
    "pw_mlp_set_adam", "pw_mlp_withhold_next_weights",
)


class PwError(RuntimeError):
    """A libpwcollide call failed; `code` is the PW_ERR_* status."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class WorldInfo(ctypes.Structure):
    _fields_ = [("scene_scale", ctypes.c_double), ("robot_center", ctypes.c_double * 3),
                ("robot_ompl_center", ctypes.c_double * 3), ("scene_matrix", ctypes.c_double * 16),
                ("robot_matrix", ctypes.c_double * 16), ("env_vertices", ctypes.c_int64),
                ("env_faces", ctypes.c_int64), ("robot_vertices", ctypes.c_int64),
                ("robot_faces", ctypes.c_int64), ("env_bvh_depth", ctypes.c_int32),
                ("robot_bvh_depth", ctypes.c_int32), ("ready", ctypes.c_int32), ("device", ctypes.c_int32)]


class QueryStats(ctypes.Structure):
    _fields_ = [("queries", ctypes.c_int64), ("node_tests", ctypes.c_int64), ("leaf_tests", ctypes.c_int64),
                ("retests", ctypes.c_int64), ("retest_hits", ctypes.c_int64),
                ("inline_retests", ctypes.c_int64), ("work_items", ctypes.c_int64),
                ("reference_checks", ctypes.c_int64), ("detailed_chunks", ctypes.c_int64),
                ("traverse_ms", ctypes.c_double),
                ("retest_ms", ctypes.c_double), ("device_errors", ctypes.c_int64),
                ("kernel_launches", ctypes.c_int64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None
vp = ctypes.c_void_p
dp = ctypes.POINTER(ctypes.c_double)
fp = ctypes.POINTER(ctypes.c_float)
u32p = ctypes.POINTER(ctypes.c_uint32)
i32p = ctypes.POINTER(ctypes.c_int32)
i64p = ctypes.POINTER(ctypes.c_int64)
i64 = ctypes.c_int64


def library_path() -> str:
    return _build.LIB_PATH


def load():
    """Load libpwcollide.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if not os.path.exists(path):
        raise ImportError("libpwcollide.so is not built (%s); run puzzletunneldiscovery_gb300.build.build() "
                          "or __graft_entry__.build() first. There is no CPU fallback." % path)
    L = ctypes.CDLL(path)
    sig = {
        "pw_last_error": (ctypes.c_char_p, []),
        "pw_world_create": (ctypes.c_int, [ctypes.POINTER(vp), ctypes.c_int]),
        "pw_world_destroy": (ctypes.c_int, [vp]),
        "pw_world_load_env": (ctypes.c_int, [vp, fp, i64, u32p, i64]),
        "pw_world_load_robot": (ctypes.c_int, [vp, fp, i64, u32p, i64]),
        "pw_world_enforce_robot_center": (ctypes.c_int, [vp, dp]),
        "pw_world_scale_to_unit": (ctypes.c_int, [vp]),
        "pw_world_angle_model": (ctypes.c_int, [vp, ctypes.c_float, ctypes.c_float]),
        "pw_world_set_perturbation": (ctypes.c_int, [vp, dp]),
        "pw_world_get_perturbation": (ctypes.c_int, [vp, dp]),
        "pw_world_info_get": (ctypes.c_int, [vp, ctypes.POINTER(WorldInfo)]),
        "pw_world_cd_vertices": (ctypes.c_int, [vp, ctypes.c_int, dp]),
        "pw_world_cd_faces": (ctypes.c_int, [vp, ctypes.c_int, i32p]),
        "pw_states_valid": (ctypes.c_int, [vp, vp, i64, vp, vp]),
        "pw_states_valid_noalloc": (ctypes.c_int, [vp, vp, i64, vp, vp]),
        "pw_states_disentangled": (ctypes.c_int, [vp, vp, i64, vp, vp]),
        "pw_segments_first_contact": (ctypes.c_int, [vp, vp, vp, i64, ctypes.c_double, ctypes.c_int, vp, vp]),
        "pw_intersecting_segments": (ctypes.c_int, [vp, dp, i64, dp, dp, dp, i32p, i32p, i64p]),
        "pw_intersecting_segments_batch": (ctypes.c_int, [vp, dp, i64, i64, dp, dp, dp, i32p, i32p, i64p, i64p]),
        "pw_world_translate_to_unit": (ctypes.c_int, [vp, dp, i64, dp]),
        "pw_world_translate_from_unit": (ctypes.c_int, [vp, dp, i64, dp]),
        "pw_world_translate_ompl_to_unit": (ctypes.c_int, [vp, dp, i64, dp]),
        "pw_world_translate_unit_to_ompl": (ctypes.c_int, [vp, dp, i64, dp, ctypes.c_int]),
        "pw_world_last_stats": (ctypes.c_int, [vp, ctypes.POINTER(QueryStats)]),
        "pw_ompl_check_motions": (ctypes.c_int, [vp, vp, vp, i64, dp, dp, ctypes.c_double, vp, i64p, vp]),
        "pw_ompl_motion_states": (ctypes.c_int, [vp, vp, vp, i64, dp, dp, ctypes.c_double, i64, vp, vp, i64p,
                                                 vp]),
        "pw_state_distance": (ctypes.c_int, [dp, dp, dp]),
        "pw_state_interpolate": (ctypes.c_int, [dp, dp, ctypes.c_double, dp]),
        "pw_segment_step_state": (ctypes.c_int, [dp, dp, ctypes.c_double, i64, dp, dp, i64p]),
        "pw_world_set_graph_mode": (ctypes.c_int, [vp, ctypes.c_int]),
        "pw_world_segments_contact_states": (ctypes.c_int, [vp, vp, vp, vp, i64, ctypes.c_double, vp, vp, vp, vp,
                                                            vp, vp, vp]),
        "pw_world_scratch_epoch": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_uint64)]),
        "pw_expand_states": (ctypes.c_int, [vp, i64, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_uint64, vp, vp]),
        "pw_expansion_crossings": (ctypes.c_int, [vp, vp, i64, ctypes.c_int, vp, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, vp, vp]),
        "pw_segments_reserve": (ctypes.c_int, [vp, i64, i64, i64]),
        "pw_world_set_launch_config": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "pw_world_get_launch_config": (ctypes.c_int, [vp, ctypes.c_int, i32p, i32p, i32p]),
        "pw_world_set_node_boxes": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
        "pw_world_get_node_boxes": (ctypes.c_int, [vp, ctypes.c_int, i32p]),
        "pw_world_set_segment_phases": (ctypes.c_int, [vp, ctypes.c_int]),
        "pw_world_set_bvh": (ctypes.c_int, [vp, ctypes.c_int]),
        "pw_world_get_bvh": (ctypes.c_int, [vp, i32p]),
        "pw_keyconf_states": (ctypes.c_int, [vp, vp, vp, vp, i64, ctypes.c_double, vp, vp, i64, ctypes.c_int, vp, vp]),
        "pw_touch_targets": (ctypes.c_int, [vp, i64, ctypes.c_int, ctypes.c_uint64, vp, vp, vp]),
        "pw_world_get_segment_phases": (ctypes.c_int, [vp, i32p]),
        "pw_segments_contact_states": (ctypes.c_int, [vp, vp, vp, i64, ctypes.c_double, vp, vp, vp, vp, vp, vp,
                                                      vp]),
        "pw_mlp_create": (ctypes.c_int, [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_uint64]),
        "pw_mlp_destroy": (ctypes.c_int, [vp]),
        "pw_mlp_num_params": (ctypes.c_int64, [vp]),
        "pw_mlp_get_params": (ctypes.c_int, [vp, fp]),
        "pw_mlp_set_params": (ctypes.c_int, [vp, fp]),
        "pw_mlp_get_grads": (ctypes.c_int, [vp, fp]),
        "pw_mlp_get_adam": (ctypes.c_int, [vp, vp, vp, vp]),
        "pw_mlp_set_adam": (ctypes.c_int, [vp, vp, vp, i64]),
        "pw_mlp_withhold_next_weights": (ctypes.c_int, [vp]),
        "pw_mlp_predict": (ctypes.c_int, [vp, vp, i64, vp, vp]),
        "pw_mlp_predict_mma": (ctypes.c_int, [vp, vp, i64, vp, vp]),
        "pw_mlp_check": (ctypes.c_int, [vp]),
        "pw_mlp_score": (ctypes.c_int, [vp, vp, i64, vp, vp]),
        "pw_mlp_set_training_kernels": (ctypes.c_int, [vp, ctypes.c_int]),
        "pw_select_top": (ctypes.c_int, [vp, vp, i64, i64, vp, i64, i64p, vp]),
        "pw_mlp_gradients": (ctypes.c_int, [vp, vp, vp, i64, fp, vp]),
        "pw_mlp_train_step": (ctypes.c_int, [vp, vp, vp, i64, ctypes.c_float, fp, vp]),
    }
    for name in EXPORTS:
        fn = getattr(L, name)
        fn.restype, fn.argtypes = sig[name]
    _lib = L
    return L


def check(rc: int, what: str = "") -> None:
    if rc != PW_OK:
        msg = load().pw_last_error()
        msg = msg.decode() if msg else ""
        raise PwError(rc, "%s failed (status %d): %s" % (what, rc, msg))
