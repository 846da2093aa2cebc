"""UnitWorld -- pyosr's collision-query API on the GB300 engine.

Mirrors ``py::class_<UnitWorld>`` of lib/pyosr/module.cc:127-250: the same
method names, argument meaning, return shapes and error behaviour
(``RuntimeError`` where the reference throws).  Single-state methods run the
batch kernels with one row.  Batched methods take torch tensors on the CUDA
device (float64, [N, 7]) and return device tensors; the numpy-level methods
(``calculate_visibility_*``) copy through pinned host memory.

Every query goes through libpwcollide.so; there is no CPU path.
"""
from __future__ import annotations

import collections.abc
import ctypes
import math

import numpy as np
import torch

from . import _lib
from . import objio
from ._lib import PwError, check

GEO_ENV = _lib.PW_GEO_ENV
GEO_ROB = _lib.PW_GEO_ROB
STATE_DIMENSION = 7


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_lib.dp)


def _states_np(q) -> np.ndarray:
    q = np.ascontiguousarray(np.asarray(q, dtype=np.float64))
    if q.ndim == 1:
        q = q.reshape(1, -1)
    if q.shape[-1] != 7:
        raise ValueError("states must have 7 columns [x, y, z, w, qx, qy, qz]")
    return q


def _stream_ptr(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _strict_tril_pairs(k: torch.Tensor):
    """(row, column) of flat index k of the strict lower triangle, row-major:
    k = row (row - 1) / 2 + column, 0 <= column < row.  Rounding of the square
    root is corrected by one step either way."""
    r = torch.floor((torch.sqrt(8.0 * k.to(torch.float64) + 1.0) + 1.0) / 2.0).to(torch.int64)
    r = torch.where(r * (r - 1) // 2 > k, r - 1, r)
    r = torch.where((r + 1) * r // 2 <= k, r + 1, r)
    return r, k - r * (r - 1) // 2


class ContactRows(collections.abc.Sequence):
    """The per-state rows of a batched contact enumeration: item i is state i's
    tuple (begins [m, 3], ends [m, 3], lengths [m], face pairs [m, 2]), views into
    the batch's arrays."""

    def __init__(self, begins, ends, lengths, face_pairs, offsets):
        self.begins, self.ends, self.lengths, self.face_pairs = begins, ends, lengths, face_pairs
        self.offsets = offsets

    def __len__(self):
        return self.offsets.shape[0] - 1

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[j] for j in range(*i.indices(len(self)))]
        n = len(self)
        i = int(i)
        if i < 0:
            i += n
        if not 0 <= i < n:
            raise IndexError("state index out of range")
        o0, o1 = int(self.offsets[i]), int(self.offsets[i + 1])
        return self.begins[o0:o1], self.ends[o0:o1], self.lengths[o0:o1], self.face_pairs[o0:o1]


class UnitWorld:
    """World of an environment and a robot mesh in the normalised unit frame."""

    GEO_ENV = GEO_ENV
    GEO_ROB = GEO_ROB

    def __init__(self, device: int = 0):
        L = _lib.load()
        if not torch.cuda.is_available():
            raise RuntimeError("UnitWorld needs a CUDA device (there is no CPU fallback)")
        self._L = L
        self._device = torch.device("cuda", device)
        h = _lib.vp()
        check(L.pw_world_create(ctypes.byref(h), int(device)), "pw_world_create")
        self._h = h
        self._robot_state = np.array([0, 0, 0, 1, 0, 0, 0], dtype=np.float64)
        self._recommended_cres = 0.001
        self._meshes = [None, None]

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                self._L.pw_world_destroy(self._h)
                self._h = None
        except Exception:
            pass

    # ----------------------------------------------------------- set-up
    def load_env_mesh(self, V, F):
        V = np.ascontiguousarray(V, dtype=np.float32)
        F = np.ascontiguousarray(F, dtype=np.uint32)
        self._meshes[0] = (V, F)
        check(self._L.pw_world_load_env(self._h, V.ctypes.data_as(_lib.fp), V.shape[0],
                                        F.ctypes.data_as(_lib.u32p), F.shape[0]), "loadModelFromFile")

    def load_robot_mesh(self, V, F):
        V = np.ascontiguousarray(V, dtype=np.float32)
        F = np.ascontiguousarray(F, dtype=np.uint32)
        self._meshes[1] = (V, F)
        self._robot_state = np.array([0, 0, 0, 1, 0, 0, 0], dtype=np.float64)
        check(self._L.pw_world_load_robot(self._h, V.ctypes.data_as(_lib.fp), V.shape[0],
                                          F.ctypes.data_as(_lib.u32p), F.shape[0]), "loadRobotFromFile")

    def loadModelFromFile(self, fn: str):
        self.load_env_mesh(*objio.load_obj(fn))

    def loadRobotFromFile(self, fn: str):
        self.load_robot_mesh(*objio.load_obj(fn))

    def enforceRobotCenter(self, center):
        c = np.ascontiguousarray(center, dtype=np.float64).reshape(3)
        check(self._L.pw_world_enforce_robot_center(self._h, _dp(c)), "enforceRobotCenter")

    def scaleToUnit(self):
        check(self._L.pw_world_scale_to_unit(self._h), "scaleToUnit")

    def angleModel(self, latitude: float, longitude: float):
        check(self._L.pw_world_angle_model(self._h, float(latitude), float(longitude)), "angleModel")

    def setupFrom(self, other: "UnitWorld"):
        """Share the other world's meshes and scale (UnitWorld::copyFrom, unit_world.cc:76-92)."""
        if other._meshes[0] is not None:
            self.load_env_mesh(*other._meshes[0])
        if other._meshes[1] is not None:
            self.load_robot_mesh(*other._meshes[1])
        info = other._info()
        self.scaleToUnit()
        if other._meshes[1] is not None:
            self.enforceRobotCenter(np.array(info.robot_center[:]))
        self.angleModel(0.0, 0.0)
        self.set_perturbation(other.perturbation)

    def set_perturbation(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(7)
        check(self._L.pw_world_set_perturbation(self._h, _dp(q)), "set_perturbation")

    @property
    def perturbation(self):
        q = np.zeros(7)
        check(self._L.pw_world_get_perturbation(self._h, _dp(q)), "perturbation")
        return q

    @property
    def state(self):
        return self._robot_state.copy()

    @state.setter
    def state(self, q):
        self._robot_state = np.asarray(q, dtype=np.float64).reshape(7).copy()

    def _info(self) -> _lib.WorldInfo:
        info = _lib.WorldInfo()
        check(self._L.pw_world_info_get(self._h, ctypes.byref(info)), "info")
        return info

    @property
    def scene_scale(self) -> float:
        return float(self._info().scene_scale)

    @property
    def scene_matrix(self):
        return np.array(self._info().scene_matrix[:]).reshape(4, 4)

    @property
    def robot_matrix(self):
        return np.array(self._info().robot_matrix[:]).reshape(4, 4)

    @property
    def recommended_cres(self) -> float:
        return self._recommended_cres

    @recommended_cres.setter
    def recommended_cres(self, v: float):
        self._recommended_cres = float(v)

    def get_ompl_center(self, geo: int = GEO_ROB):
        info = self._info()
        if geo == GEO_ROB:
            return np.array(info.robot_ompl_center[:])
        return np.zeros(3)

    def info(self) -> dict:
        i = self._info()
        return {"scene_scale": i.scene_scale, "robot_center": np.array(i.robot_center[:]),
                "robot_ompl_center": np.array(i.robot_ompl_center[:]), "env_vertices": i.env_vertices,
                "env_faces": i.env_faces, "robot_vertices": i.robot_vertices, "robot_faces": i.robot_faces,
                "env_bvh_depth": i.env_bvh_depth, "robot_bvh_depth": i.robot_bvh_depth, "ready": bool(i.ready)}

    # ----------------------------------------------------------- batched device API
    def _dev_states(self, q: torch.Tensor) -> torch.Tensor:
        if not isinstance(q, torch.Tensor):
            q = torch.as_tensor(np.asarray(q, dtype=np.float64))
        if q.dim() == 1:
            q = q.reshape(1, -1)
        if q.shape[-1] != 7:
            raise ValueError("states must have 7 columns")
        return q.to(device=self._device, dtype=torch.float64).contiguous()

    def is_valid_states(self, q: torch.Tensor) -> torch.Tensor:
        """isValid for a batch: bool tensor [N] on the device (True = collision free)."""
        q = self._dev_states(q)
        out = torch.empty(q.shape[0], dtype=torch.uint8, device=self._device)
        check(self._L.pw_states_valid(self._h, q.data_ptr(), q.shape[0], out.data_ptr(),
                                      _stream_ptr(self._device)), "is_valid_state")
        return out.bool()

    # host batches, streamed ------------------------------------------------------
    def _host_stream(self, run, hosts, out_dtype, chunk: int) -> torch.Tensor:
        """Runs `run(device inputs..., device out)` over host batches in chunks of
        `chunk` rows: the host-to-device copy of chunk i + 1 runs on a copy stream
        while chunk i is checked on the current stream, and each chunk's result is
        copied back behind it.  Returns the results in pinned host memory."""
        hs = []
        for h in hosts:
            t = h if isinstance(h, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(h, dtype=np.float64))
            if t.is_cuda:
                raise TypeError("host entry points take host batches; use the device methods for CUDA tensors")
            if t.dtype != torch.float64 or t.dim() != 2 or t.shape[1] != 7:
                raise ValueError("host states must be float64 [n, 7]")
            t = t.contiguous()
            hs.append(t if t.is_pinned() else t.pin_memory())
        n = hs[0].shape[0]
        if any(h.shape[0] != n for h in hs):
            raise ValueError("host batches differ in length")
        out = torch.empty(n, dtype=out_dtype, pin_memory=True)
        if n == 0:
            return out
        host_out = out.view(torch.uint8) if out_dtype == torch.bool else out
        dev_dtype = torch.uint8 if out_dtype == torch.bool else out_dtype
        dev = self._device
        chunk = max(1, min(int(chunk), n))
        comp = torch.cuda.current_stream(dev)
        copy = getattr(self, "_copy_stream", None)
        if copy is None:
            copy = self._copy_stream = torch.cuda.Stream(dev)
        bufs = [[torch.empty((chunk, 7), dtype=torch.float64, device=dev) for _ in hs] for _ in range(2)]
        obufs = [torch.empty(chunk, dtype=dev_dtype, device=dev) for _ in range(2)]
        ready = [torch.cuda.Event() for _ in range(2)]
        free = [torch.cuda.Event() for _ in range(2)]
        for k, s0 in enumerate(range(0, n, chunk)):
            m = min(chunk, n - s0)
            b = k & 1
            with torch.cuda.stream(copy):
                if k >= 2:
                    copy.wait_event(free[b])        # chunk k - 2 is done with buffer b
                for h, d in zip(hs, bufs[b]):
                    d[:m].copy_(h[s0:s0 + m], non_blocking=True)
                ready[b].record(copy)
            comp.wait_event(ready[b])
            run(*[d[:m] for d in bufs[b]], obufs[b][:m])
            host_out[s0:s0 + m].copy_(obufs[b][:m], non_blocking=True)
            free[b].record(comp)
        comp.synchronize()
        return out

    def is_valid_states_host(self, q, chunk: int = 1 << 21) -> torch.Tensor:
        """isValid for a host batch (numpy or CPU tensor, float64 [N, 7]): bool [N] in
        pinned host memory.  Pinned input avoids a staging copy."""
        def run(d, o):
            check(self._L.pw_states_valid(self._h, d.data_ptr(), d.shape[0], o.data_ptr(), _stream_ptr(self._device)),
                  "is_valid_state")
        return self._host_stream(run, [q], torch.bool, chunk)

    def first_contact_steps_host(self, q0, q1, verify_delta: float, mode: int = _lib.PW_SEG_TRANSIT,
                                 chunk: int = 1 << 22) -> torch.Tensor:
        """first_contact_steps for host batches: int32 [N] in pinned host memory."""
        def run(a, b, o):
            check(self._L.pw_segments_first_contact(self._h, a.data_ptr(), b.data_ptr(), a.shape[0], float(verify_delta),
                                                    int(mode), o.data_ptr(), _stream_ptr(self._device)),
                  "first_contact_steps")
        return self._host_stream(run, [q0, q1], torch.int32, chunk)

    def is_disentangled_states(self, q: torch.Tensor) -> torch.Tensor:
        q = self._dev_states(q)
        out = torch.empty(q.shape[0], dtype=torch.uint8, device=self._device)
        rc = self._L.pw_states_disentangled(self._h, q.data_ptr(), q.shape[0], out.data_ptr(),
                                            _stream_ptr(self._device))
        if rc == _lib.PW_ERR_NO_MODEL:
            raise RuntimeError("Pain in the ass: models not loaded")
        check(rc, "is_disentangled")
        return out.view(torch.bool)   # verdicts are 0 / 1: the same bytes, no conversion kernel

    def first_contact_steps(self, q0: torch.Tensor, q1: torch.Tensor, verify_delta: float,
                            mode: int = _lib.PW_SEG_TRANSIT) -> torch.Tensor:
        """First colliding step of every segment (int32 [N]): >= 0 step index, -1 all free,
        -2 no step taken (verify_delta >= distance), -3 more than 2^30 steps."""
        q0 = self._dev_states(q0)
        q1 = self._dev_states(q1)
        if q0.shape != q1.shape:
            raise ValueError("from/to batches differ in shape")
        out = torch.empty(q0.shape[0], dtype=torch.int32, device=self._device)
        check(self._L.pw_segments_first_contact(self._h, q0.data_ptr(), q1.data_ptr(), q0.shape[0],
                                                float(verify_delta), int(mode), out.data_ptr(),
                                                _stream_ptr(self._device)), "first_contact_steps")
        return out

    def is_valid_transitions(self, q0: torch.Tensor, q1: torch.Tensor, initial_verify_delta: float) -> torch.Tensor:
        """isValidTransition for a batch of aligned pairs (bool [N])."""
        return self.first_contact_steps(q0, q1, initial_verify_delta, _lib.PW_SEG_TRANSITION) == _lib.PW_STEP_FREE

    # graph mode and launch configuration -------------------------------------
    def set_graph_mode(self, on: bool) -> None:
        """Segment queries without host synchronisation or allocation (CUDA-graph capturable)."""
        check(self._L.pw_world_set_graph_mode(self._h, 1 if on else 0), "set_graph_mode")

    def scratch_epoch(self) -> int:
        """Identifier of the current query scratch; a captured graph is valid while it is unchanged."""
        e = ctypes.c_uint64()
        check(self._L.pw_world_scratch_epoch(self._h, ctypes.byref(e)), "scratch_epoch")
        return int(e.value)

    def segments_reserve(self, n: int, total_chunks: int, max_chunks: int) -> None:
        check(self._L.pw_segments_reserve(self._h, int(n), int(total_chunks), int(max_chunks)), "segments_reserve")

    def set_launch_config(self, kernel: int, width: int = 0, soft_cap: int = 0, blocks: int = 0) -> None:
        """kernel 0 = states, 1 = segments; 0 keeps a field's default."""
        check(self._L.pw_world_set_launch_config(self._h, int(kernel), int(width), int(soft_cap), int(blocks)),
              "set_launch_config")

    def get_launch_config(self, kernel: int) -> dict:
        w, c, b = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        check(self._L.pw_world_get_launch_config(self._h, int(kernel), ctypes.byref(w), ctypes.byref(c),
                                                 ctypes.byref(b)), "get_launch_config")
        return {"width": w.value, "soft_cap": c.value, "blocks": b.value}

    def set_node_boxes(self, kind: str, kernel: int = -1) -> None:
        """Node boxes a traversal kernel tests (0 = states, 1 = segments, -1 =
        both): "oriented" (default) or "aligned"; the verdicts do not depend on it."""
        k = {"aligned": _lib.PW_BOXES_ALIGNED, "oriented": _lib.PW_BOXES_ORIENTED}[kind]
        check(self._L.pw_world_set_node_boxes(self._h, int(kernel), k), "set_node_boxes")

    def get_node_boxes(self, kernel: int) -> str:
        k = ctypes.c_int32()
        check(self._L.pw_world_get_node_boxes(self._h, int(kernel), ctypes.byref(k)), "get_node_boxes")
        return "oriented" if k.value == _lib.PW_BOXES_ORIENTED else "aligned"

    _BVH = {"topdown": _lib.PW_BVH_TOPDOWN, "morton": _lib.PW_BVH_MORTON, "sah": _lib.PW_BVH_SAH}

    def set_bvh(self, kind: str) -> None:
        """The hierarchy the next BVH build (angleModel) uses: "topdown" (default),
        "sah" or "morton"; the verdicts do not depend on it."""
        check(self._L.pw_world_set_bvh(self._h, self._BVH[kind]), "set_bvh")

    def get_bvh(self) -> str:
        k = ctypes.c_int32()
        check(self._L.pw_world_get_bvh(self._h, ctypes.byref(k)), "get_bvh")
        return {v: name for name, v in self._BVH.items()}[k.value]

    _PHASES = {"auto": _lib.PW_PHASES_AUTO, "off": _lib.PW_PHASES_OFF, "on": _lib.PW_PHASES_ON}

    def set_segment_phases(self, mode: str) -> None:
        """Round phases of segment queries: "auto" (default), "off" or "on"; the
        results do not depend on it."""
        check(self._L.pw_world_set_segment_phases(self._h, self._PHASES[mode]), "set_segment_phases")

    def get_segment_phases(self) -> str:
        k = ctypes.c_int32()
        check(self._L.pw_world_get_segment_phases(self._h, ctypes.byref(k)), "get_segment_phases")
        return {v: name for name, v in self._PHASES.items()}[k.value]

    def last_stats(self) -> dict:
        st = _lib.QueryStats()
        check(self._L.pw_world_last_stats(self._h, ctypes.byref(st)), "last_stats")
        return st.as_dict()

    # ----------------------------------------------------------- pyosr single-state API
    def is_valid_state(self, q) -> bool:
        return bool(self.is_valid_states(_states_np(q)).cpu()[0])

    def is_disentangled(self, q) -> bool:
        return bool(self.is_disentangled_states(_states_np(q)).cpu()[0])

    def transit_state_to_with_contact(self, from_state, to_state, verify_delta):
        """(last_free, colliding_or_last, done, last_tau, tau) of unit_world.cc:405-474."""
        a = _states_np(from_state)[0]
        b = _states_np(to_state)[0]
        dist = distance(a, b)
        if verify_delta >= dist:
            return a.copy(), b.copy(), False, np.float32(0.0), np.float32(1.0)
        if dist != dist:
            return a.copy(), a.copy(), False, np.float32(0.0), np.float32(0.0)
        k = int(self.first_contact_steps(a, b, verify_delta, _lib.PW_SEG_TRANSIT).cpu()[0])
        if k == _lib.PW_STEP_INVALID:
            raise RuntimeError("transit_state_to: more than 2^30 steps at this verify_delta")
        if k >= 0:
            st, tau, _ = segment_step_state(a, b, verify_delta, k)
            if k > 0:
                lf, ltau, _ = segment_step_state(a, b, verify_delta, k - 1)
            else:
                lf, ltau = a.copy(), 0.0
            return lf, st, False, np.float32(ltau), np.float32(tau)
        # every step free: the loop's last state, `done` true, and the reference's outer tau (0)
        _, _, K = segment_step_state(a, b, verify_delta, 0)
        lf, ltau, _ = segment_step_state(a, b, verify_delta, K - 1)
        return lf, lf.copy(), True, np.float32(ltau), np.float32(0.0)

    def transit_states_to_with_contact(self, q0, q1, verify_delta: float):
        """transit_state_to_with_contact for a batch (device tensors): returns
        (last_free [N,7], contact [N,7], done [N] bool, last_tau [N] f32, tau [N] f32),
        each row the tuple of unit_world.cc:405-474 for that segment."""
        q0 = self._dev_states(q0)
        q1 = self._dev_states(q1)
        if q0.shape != q1.shape:
            raise ValueError("from/to batches differ in shape")
        n = q0.shape[0]
        steps = self.first_contact_steps(q0, q1, verify_delta, _lib.PW_SEG_TRANSIT)
        dev = self._device
        lf = torch.empty((n, 7), dtype=torch.float64, device=dev)
        st = torch.empty((n, 7), dtype=torch.float64, device=dev)
        done = torch.empty(n, dtype=torch.uint8, device=dev)
        lt = torch.empty(n, dtype=torch.float32, device=dev)
        tt = torch.empty(n, dtype=torch.float32, device=dev)
        err = torch.zeros(1, dtype=torch.int32, device=dev)
        check(self._L.pw_world_segments_contact_states(self._h, q0.data_ptr(), q1.data_ptr(), steps.data_ptr(), n,
                                                       float(verify_delta), lf.data_ptr(), st.data_ptr(),
                                                       done.data_ptr(), lt.data_ptr(), tt.data_ptr(), err.data_ptr(),
                                                       _stream_ptr(dev)), "transit_states_to_with_contact")
        if int(err.item()) != 0:
            raise RuntimeError("transit_state_to: more than 2^30 steps at this verify_delta")
        return lf, st, done.bool(), lt, tt

    def transit_state_to(self, from_state, to_state, verify_delta):
        """(free state, done, progress) of unit_world.cc:395-402."""
        tup = self.transit_state_to_with_contact(from_state, to_state, verify_delta)
        return tup[0], tup[2], tup[3]

    def transit_state(self, state, action: int, transit_magnitude: float, verify_delta: float):
        """UnitWorld::transitState (unit_world.cc:268-330): one of the 12 discrete
        actions (translation / rotation, +- x, y, z) by the verify step (twice it
        for rotations, as float32), then transit_state_to, halving the float32
        verify step while no progress is made.  An invalid action or start state
        returns (state, False, 0.0).  transit_magnitude is unused, as in the
        reference's active branch."""
        from . import state_ops as so
        q = _states_np(state)[0]
        if action < 0 or action >= 12 or not self.is_valid_state(q):
            return q, False, 0.0
        action_type = 0 if action < 6 else 1
        deltacap = np.float32(verify_delta) if action_type == 0 else np.float32(verify_delta * 2.0)
        sym = np.float32(1.0 if action % 2 == 0 else -1.0)
        axis = np.zeros(3)
        axis[(action - 6 * action_type) // 2] = 1.0
        trans, rot = so.decompose(q)
        if action_type == 0:
            trans = trans + float(deltacap) * axis * float(sym)
        else:
            rot = so.quat_mul(so.quat_from_angleaxis(float(np.float32(deltacap * sym)), axis), rot)
        to = so.compose(trans, rot)
        cvd = np.float32(verify_delta)
        while True:
            free, done, prog = self.transit_state_to(q, to, float(cvd))
            if not self.is_valid_state(free):
                raise RuntimeError("SAN check failed, invalid state from transitStateTo")
            if prog > 0.0 or cvd == 0.0:
                return free, done, prog
            cvd = np.float32(cvd / 2.0)

    def transit_state_by(self, from_state, tr, aav, verify_delta: float):
        """UnitWorld::transitStateBy (unit_world.cc:490-507): the target is the start
        translated by tr and rotated on the left by the angle-axis vector aav (the
        start's quaternion as given, not normalised)."""
        from . import state_ops as so
        a = _states_np(from_state)[0]
        aav = np.asarray(aav, dtype=np.float64).reshape(3)
        n = float(np.linalg.norm(aav))
        rot = so.quat_mul(so.quat_from_angleaxis(n, aav / n if n > 0 else aav), a[3:7])
        to = np.concatenate([a[:3] + np.asarray(tr, dtype=np.float64).reshape(3), rot])
        return self.transit_state_to(a, to, verify_delta)

    def is_valid_transition(self, from_state, to_state, initial_verify_delta) -> bool:
        a = _states_np(from_state)
        b = _states_np(to_state)
        return bool(self.is_valid_transitions(a, b, initial_verify_delta).cpu()[0])

    # ----------------------------------------------------------- frames
    def _convert(self, fn, q, *extra):
        q = _states_np(q)
        out = np.zeros_like(q)
        check(fn(self._h, _dp(q), q.shape[0], _dp(out), *extra), "state conversion")
        return out

    def translate_to_unit_state(self, q):
        single = np.ndim(q) == 1
        out = self._convert(self._L.pw_world_translate_to_unit, q)
        return out[0] if single else out

    def translate_from_unit_state(self, q):
        single = np.ndim(q) == 1
        out = self._convert(self._L.pw_world_translate_from_unit, q)
        return out[0] if single else out

    def translate_ompl_to_unit(self, Q):
        return self._convert(self._L.pw_world_translate_ompl_to_unit, Q)

    def translate_unit_to_ompl(self, Q, to_angle_axis: bool = False):
        return self._convert(self._L.pw_world_translate_unit_to_ompl, Q, int(bool(to_angle_axis)))

    def _vanilla_offset(self, qs, sign: float):
        from . import state_ops as so
        qs = _states_np(qs)
        oc = self.get_ompl_center(GEO_ROB)
        out = qs.copy()
        for i, q in enumerate(qs):
            # vanilla and OMPL states are both w-last
            r = np.array([q[6], q[3], q[4], q[5]])
            out[i, :3] = q[:3] + sign * (so.quat_to_matrix(r / np.linalg.norm(r)) @ oc)
        return out

    def translate_vanilla_to_ompl(self, qs):
        """t_ompl = t_vanilla + R O, O the robot's OMPL centre (unit_world.cc:600-638)."""
        return self._vanilla_offset(qs, 1.0)

    def translate_ompl_to_vanilla(self, qs):
        """t_vanilla = t_ompl - R O (unit_world.cc:640-661)."""
        return self._vanilla_offset(qs, -1.0)

    def translate_vanilla_to_unit(self, qs):
        """unit_world.cc:663-667."""
        return self.translate_ompl_to_unit(self.translate_vanilla_to_ompl(qs))

    def translate_vanilla_pts_to_unit(self, geo: int, pts):
        """Points of a mesh's own frame to the unit frame: the scene's calibration
        transform, after the OMPL centre is taken off robot points
        (unit_world.cc:669-688)."""
        pts = np.asarray(pts, dtype=np.float64)
        if pts.ndim != 2 or pts.shape[0] == 0:
            return np.zeros((0, 3))
        p = pts[:, :3] if geo == GEO_ENV else pts[:, :3] - self.get_ompl_center(GEO_ROB)
        h = np.concatenate([p, np.ones((p.shape[0], 1))], axis=1)
        return (self.scene_matrix @ h.T).T[:, :3]

    # kinetic-energy metric (unit_world.cc:1567-1596) -------------------------------
    def _robot_mass_properties(self):
        """Volume and inertia tensor of the robot's CD mesh: the divergence-theorem
        sums over the tetrahedra (origin, triangle) -- signed volume det / 6 and
        the covariance det * A^T C0 A, C0 the unit tetrahedron's (1/60 on the
        diagonal, 1/120 off it), inertia = trace(C) I - C -- rebased to the robot
        scene's centre as cdmodel.cc:60-80 does."""
        cache = self.__dict__.get("_mass_cache")
        V, F = self._cd(GEO_ROB)
        c = np.array(self._info().robot_center[:])
        # keyed by what the result depends on: the CD mesh as placed and the rebase centre
        key = (V.tobytes(), F.tobytes(), c.tobytes())
        if cache is not None and cache[0] == key:
            return cache[1], cache[2]
        A = V[F]                                     # [m, 3 vertices, 3 coords]: rows are the vertices
        det = np.einsum("ij,ij->i", np.cross(A[:, 0], A[:, 1]), A[:, 2])
        C0 = np.full((3, 3), 1.0 / 120.0) + np.eye(3) * (1.0 / 120.0)
        C = np.einsum("m,mki,kl,mlj->ij", det, A, C0, A)
        vol = float(det.sum()) / 6.0
        mi = np.trace(C) * np.eye(3) - C
        off = np.outer(c, c)
        rebased = mi + vol * off
        for k in range(3):
            rebased[k, k] = mi[k, k] - vol * (float(c @ c) - c[k] * c[k])
        self._mass_cache = (key, rebased, vol)
        return rebased, vol

    def kinetic_energy_distance(self, q0, q1) -> float:
        """|dt|^2 + 4 dr_v^T I dr_v / volume, dr = rot1 rot0^-1 (unit_world.cc:1567-1582)."""
        from . import state_ops as so
        t0, r0 = so.decompose(q0)
        t1, r1 = so.decompose(q1)
        dt = t1 - t0
        dr = so.quat_mul(r1, so.quat_inverse(r0))
        inertia, vol = self._robot_mass_properties()
        return float(dt @ dt) + float(dr[1:] @ inertia @ dr[1:]) * 4.0 / vol

    def multi_kinetic_energy_distance(self, origin, targets):
        """kinetic_energy_distance(origin, targets[i]) for every row (unit_world.cc:1584-1596)."""
        from . import state_ops as so
        targets = _states_np(targets)
        inertia, vol = self._robot_mass_properties()
        t0, r0 = so.decompose(origin)
        inv0 = so.quat_inverse(r0)
        out = np.empty(targets.shape[0])
        for i, q in enumerate(targets):
            t1, r1 = so.decompose(q)
            dt = t1 - t0
            dv = so.quat_mul(r1, inv0)[1:]
            out[i] = float(dt @ dt) + float(dv @ inertia @ dv) * 4.0 / vol
        return out

    # free-configuration samplers with pyosr's method names (module.cc:211-226) -------
    def sample_free_configuration(self, rob_surface_point, rob_surface_normal, env_surface_point,
                                  env_surface_normal, margin: float, max_trials: int = -1):
        """UnitWorld::sampleFreeConfiguration; max_trials < 0 tries until a free
        spin is found, as the reference does."""
        from . import sampling
        if max_trials >= 0:
            return sampling.sample_free_configuration(self, rob_surface_point, rob_surface_normal, env_surface_point,
                                                      env_surface_normal, margin, max_trials)
        while True:
            q, found = sampling.sample_free_configurations(self, rob_surface_point, rob_surface_normal,
                                                           env_surface_point, env_surface_normal, margin, 255)
            if bool(found[0]):
                return q[0]

    def enum_free_configuration(self, rob_surface_point, rob_surface_normal, env_surface_point, env_surface_normal,
                                margin: float, denominator: int, only_median: bool = False):
        """UnitWorld::enumFreeConfiguration (all spins checked as one batch)."""
        from . import sampling
        return sampling.enum_free_configuration(self, rob_surface_point, rob_surface_normal, env_surface_point,
                                                env_surface_normal, margin, denominator, only_median)

    # ----------------------------------------------------------- visibility batches
    def _pairs_first(self, qs0, qs1, verify_magnitude):
        a = torch.from_numpy(qs0).pin_memory().to(self._device, non_blocking=True)
        b = torch.from_numpy(qs1).pin_memory().to(self._device, non_blocking=True)
        k = self.first_contact_steps(a, b, verify_magnitude, _lib.PW_SEG_TRANSITION)
        return (k == _lib.PW_STEP_FREE).to(torch.int8).cpu().numpy()

    def _maybe_unit(self, qs, is_unit):
        qs = _states_np(qs)
        return qs if is_unit else self.translate_to_unit_state(qs)

    def calculate_visibility_pair(self, qs0, qs0_are_unit_states, qs1, qs1_are_unit_states, verify_magnitude,
                                  enable_mt=True):
        """int8 [max(M, N)]: isValidTransition(qs0[i], qs1[i]) (unit_world.cc:799-840)."""
        a = self._maybe_unit(qs0, qs0_are_unit_states)
        b = self._maybe_unit(qs1, qs1_are_unit_states)
        if a.shape[0] != b.shape[0]:
            raise ValueError("calculate_visibility_pair: qs0 and qs1 must have the same number of rows")
        return self._pairs_first(a, b, verify_magnitude)

    def calculate_visibility_matrix2(self, qs0, qs0_are_unit_states, qs1, qs1_are_unit_states, verify_magnitude,
                                     enable_mt=True):
        """int8 [M, N] of isValidTransition(qs0[i], qs1[j]) (unit_world.cc:761-797).
        The (i, j) pairs are decoded on the device from flat indices, in chunks."""
        a = self._dev_states(self._maybe_unit(qs0, qs0_are_unit_states))
        b = self._dev_states(self._maybe_unit(qs1, qs1_are_unit_states))
        M, N = a.shape[0], b.shape[0]
        out = torch.zeros(M * N, dtype=torch.int8, device=self._device)
        for k0 in range(0, M * N, self._PAIR_CHUNK):
            k = torch.arange(k0, min(M * N, k0 + self._PAIR_CHUNK), dtype=torch.int64, device=self._device)
            out[k0:k0 + k.shape[0]] = self._visible(a.index_select(0, k // N), b.index_select(0, k % N),
                                                    verify_magnitude)
        return out.reshape(M, N).cpu().numpy()

    def calculate_visibility_matrix(self, qs, is_unit_states, verify_magnitude):
        """Symmetric int8 [N, N]: isValidTransition(qs[i], qs[j]) for i < j, mirrored
        (unit_world.cc:740-759).  The diagonal, which the reference leaves
        uninitialised, is 0.  The pairs are decoded on the device from flat
        indices of the strict triangle, in chunks."""
        q = self._dev_states(self._maybe_unit(qs, is_unit_states))
        N = q.shape[0]
        out = torch.zeros((N, N), dtype=torch.int8, device=self._device)
        total = N * (N - 1) // 2
        for k0 in range(0, total, self._PAIR_CHUNK):
            k = torch.arange(k0, min(total, k0 + self._PAIR_CHUNK), dtype=torch.int64, device=self._device)
            hi, lo = _strict_tril_pairs(k)                  # lo < hi: from = qs[lo], to = qs[hi]
            v = self._visible(q.index_select(0, lo), q.index_select(0, hi), verify_magnitude)
            out[lo, hi] = v
            out[hi, lo] = v
        return out.cpu().numpy()

    _PAIR_CHUNK = 1 << 22

    def _visible(self, a: torch.Tensor, b: torch.Tensor, verify_magnitude) -> torch.Tensor:
        k = self.first_contact_steps(a, b, verify_magnitude, _lib.PW_SEG_TRANSITION)
        return (k == _lib.PW_STEP_FREE).to(torch.int8)

    # ----------------------------------------------------------- contacts and geometry
    def intersecting_segments(self, unitq):
        """(begins m x 3, ends m x 3, lengths m, face pairs m x 2 [env, robot]) of
        unit_world.cc:959-1012, rows sorted by (env face, robot face)."""
        q = np.ascontiguousarray(unitq, dtype=np.float64).reshape(7)
        cap = 1024
        while True:
            b = np.zeros((cap, 3))
            e = np.zeros((cap, 3))
            m = np.zeros(cap)
            p = np.zeros((cap, 2), dtype=np.int32)
            c = np.zeros(cap, dtype=np.int32)
            cnt = ctypes.c_int64(0)
            rc = self._L.pw_intersecting_segments(self._h, _dp(q), cap, _dp(b), _dp(e), _dp(m),
                                                  p.ctypes.data_as(_lib.i32p), c.ctypes.data_as(_lib.i32p),
                                                  ctypes.byref(cnt))
            if rc == _lib.PW_ERR_CAPACITY and cnt.value > cap:
                cap = int(cnt.value)
                continue
            check(rc, "intersecting_segments")
            n = int(cnt.value)
            self._last_coplanar = c[:n].copy()
            return b[:n].copy(), e[:n].copy(), m[:n].copy(), p[:n].copy()

    def intersecting_segments_batch(self, unitqs, flat: bool = False):
        """intersecting_segments for many unit states in one call: a sequence
        (ContactRows) whose item i is state i's tuple (begins, ends, lengths,
        face pairs) as intersecting_segments returns it (views into one set of
        arrays, made when the item is read).  With flat=True: (begins, ends,
        lengths, face pairs, offsets), the rows of state i at
        offsets[i]:offsets[i + 1]."""
        q = _states_np(unitqs)
        n = q.shape[0]
        offsets = np.zeros(n + 1, dtype=np.int64)
        total = ctypes.c_int64(0)
        # rows per state seen by the last call sizes the first attempt
        cap = max(1024, int(getattr(self, "_isect_rows_per_state", 64.0) * 1.25 * n))
        while True:
            b = np.empty((cap, 3))
            e = np.empty((cap, 3))
            m = np.empty(cap)
            p = np.empty((cap, 2), dtype=np.int32)
            c = np.empty(cap, dtype=np.int32)
            rc = self._L.pw_intersecting_segments_batch(self._h, _dp(q), n, cap, _dp(b), _dp(e), _dp(m),
                                                        p.ctypes.data_as(_lib.i32p), c.ctypes.data_as(_lib.i32p),
                                                        offsets.ctypes.data_as(_lib.i64p), ctypes.byref(total))
            if rc == _lib.PW_ERR_CAPACITY and total.value > cap:
                cap = int(total.value)
                continue
            check(rc, "intersecting_segments_batch")
            break
        t = int(total.value)
        if n:
            self._isect_rows_per_state = max(1.0, t / n)
        b, e, m, p = b[:t], e[:t], m[:t], p[:t]
        if flat:
            return b, e, m, p, offsets
        return ContactRows(b, e, m, p, offsets)

    # contact forces (unit_world.cc:1015-1057) ---------------------------------
    def _face_normals(self, geo):
        """Per-face unit normals of the CD mesh in its own frame (igl::per_face_normals:
        (v1 - v0) x (v2 - v0) normalised; a degenerate face gives the zero vector)."""
        cache = self.__dict__.setdefault("_fn_cache", {})
        if geo not in cache:
            V, F = self._cd(geo)
            n = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
            r = np.linalg.norm(n, axis=1, keepdims=True)
            cache[geo] = np.where(r > 0, n / np.where(r > 0, r, 1.0), 0.0)
        return cache[geo]

    def robot_face_normals_from_indices(self, faces):
        return self._face_normals(GEO_ROB)[np.asarray(faces, dtype=np.int64).reshape(-1)]

    def scene_face_normals_from_indices(self, faces):
        return self._face_normals(GEO_ENV)[np.asarray(faces, dtype=np.int64).reshape(-1)]

    def robot_face_normals_from_index_pairs(self, faces):
        return self.robot_face_normals_from_indices(np.asarray(faces).reshape(-1, 2)[:, 1])

    def scene_face_normals_from_index_pairs(self, faces):
        return self.scene_face_normals_from_indices(np.asarray(faces).reshape(-1, 2)[:, 0])

    def force_direction_from_intersecting_segments(self, sbegins, sends, faces):
        """(force positions, force directions) of unit_world.cc:1038-1057: the
        segment midpoints, and (end - begin) x robot face normal, flipped to
        agree with the environment face normal.  As in the reference, the robot
        normal is taken in the robot's own frame."""
        b = np.asarray(sbegins, dtype=np.float64).reshape(-1, 3)
        e = np.asarray(sends, dtype=np.float64).reshape(-1, 3)
        pos = (b + e) * 0.5
        d = np.cross(e - b, self.robot_face_normals_from_index_pairs(faces))
        dots = np.sign(np.sum(d * self.scene_face_normals_from_index_pairs(faces), axis=1))
        return pos, d * dots[:, None]

    def _cd(self, geo):
        info = self._info()
        nv = info.env_vertices if geo == GEO_ENV else info.robot_vertices
        nf = info.env_faces if geo == GEO_ENV else info.robot_faces
        V = np.zeros((nv, 3))
        F = np.zeros((nf, 3), dtype=np.int32)
        check(self._L.pw_world_cd_vertices(self._h, geo, _dp(V)), "cd_vertices")
        check(self._L.pw_world_cd_faces(self._h, geo, F.ctypes.data_as(_lib.i32p)), "cd_faces")
        return V, F

    def get_robot_geometry(self, q, q_is_unit: bool = True):
        """Robot CD vertices placed at q (unit_world.cc:1102-1116)."""
        qu = _states_np(q)[0] if q_is_unit else self.translate_to_unit_state(_states_np(q)[0])
        V, F = self._cd(GEO_ROB)
        R, t = state_transform(qu)
        return V @ R.T + t, F

    def get_scene_geometry(self, q, q_is_unit: bool = True):
        V, F = self._cd(GEO_ENV)
        return V, F


# ------------------------------------------------------------------- module-level state math

def get_identity_state_vector():
    return np.array([0, 0, 0, 1, 0, 0, 0], dtype=np.float64)


def distance(a, b) -> float:
    """osr::distance (osr_state.cc:130-154) with the engine's deterministic FP64 math."""
    L = _lib.load()
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(7)
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(7)
    out = np.zeros(1)
    check(L.pw_state_distance(_dp(a), _dp(b), _dp(out)), "distance")
    return float(out[0])


def multi_distance(origin, targets):
    targets = _states_np(targets)
    return np.array([distance(origin, t) for t in targets])


def interpolate(a, b, tau: float):
    """osr::interpolate (osr_state.cc:27-44)."""
    L = _lib.load()
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(7)
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(7)
    out = np.zeros(7)
    check(L.pw_state_interpolate(_dp(a), _dp(b), float(tau), _dp(out)), "interpolate")
    return out


def segment_step_state(a, b, verify_delta: float, k: int):
    """(state, tau, number of steps) of step k of the reference stepping loop."""
    L = _lib.load()
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(7)
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(7)
    out = np.zeros(7)
    tau = np.zeros(1)
    n = ctypes.c_int64(0)
    rc = L.pw_segment_step_state(_dp(a), _dp(b), float(verify_delta), int(k), _dp(out), _dp(tau), ctypes.byref(n))
    if rc != _lib.PW_OK and not (rc == _lib.PW_ERR_INVALID_ARG and n.value > 0 and (k < 0 or k >= n.value)):
        check(rc, "segment_step_state")
    return out, float(tau[0]), int(n.value)


def state_transform(q):
    """Rotation (raw-quaternion formula) and translation of a state, numpy float64."""
    q = np.asarray(q, dtype=np.float64).reshape(7)
    w, x, y, z = q[3:7]
    tx, ty, tz = 2 * x, 2 * y, 2 * z
    R = np.array([[1 - (ty * y + tz * z), ty * x - tz * w, tz * x + ty * w],
                  [ty * x + tz * w, 1 - (tx * x + tz * z), tz * y - tx * w],
                  [tz * x - ty * w, tz * y + tx * w, 1 - (tx * x + ty * y)]])
    return R, q[:3].copy()


def apply(from_state, tr, aa):
    """osr::apply (osr_state.cc:244-259): translate, then rotate by angle-axis on the left."""
    q = np.asarray(from_state, dtype=np.float64).reshape(7)
    rot = q[3:7] / np.linalg.norm(q[3:7])
    t = q[:3] + np.asarray(tr, dtype=np.float64)
    aa = np.asarray(aa, dtype=np.float64)
    ang = float(np.linalg.norm(aa))
    axis = np.array([1.0, 0.0, 0.0]) if ang == 0.0 else aa / ang
    dq = np.concatenate([[math.cos(ang / 2)], math.sin(ang / 2) * axis])
    w1, x1, y1, z1 = dq
    w2, x2, y2, z2 = rot
    r = np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                  w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])
    r /= np.linalg.norm(r)
    return np.concatenate([t, r])


__all__ = ["UnitWorld", "GEO_ENV", "GEO_ROB", "STATE_DIMENSION", "PwError", "distance", "multi_distance",
           "interpolate", "segment_step_state", "apply", "get_identity_state_vector", "state_transform"]
