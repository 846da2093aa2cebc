"""ctypes binding of the CPU oracle (oracle/pw_oracle.c) -- test infrastructure.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  The product (``puzzletunneldiscovery_gb300``)
never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libpworacle.so")
_lib = None

c_double_p = ctypes.POINTER(ctypes.c_double)
c_float_p = ctypes.POINTER(ctypes.c_float)
c_u8_p = ctypes.POINTER(ctypes.c_uint8)
c_u32_p = ctypes.POINTER(ctypes.c_uint32)
c_i32_p = ctypes.POINTER(ctypes.c_int32)
c_i64_p = ctypes.POINTER(ctypes.c_int64)


def build(force: bool = False) -> str:
    """Compile libpworacle.so with the Makefile beside this file."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "pw_oracle.c")):
        subprocess.run(["make", "-s", "-C", _HERE, "libpworacle.so"], check=True)
    return _LIB_PATH


# the reference checkout: PW_REFERENCE_DIR, by default a sibling of this repository named "reference"
REFERENCE_DIR = os.environ.get("PW_REFERENCE_DIR",
                               os.path.join(os.path.dirname(os.path.dirname(_HERE)), "reference"))
_REF_SRC = os.path.join(REFERENCE_DIR, "lib", "tritri", "Moller97d.cc")
_REF_LIB = os.path.join(_HERE, "_ref", "libref_tritri.so")
_ref = None


def build_ref() -> str | None:
    """Compile the reference's own Moller test (its source where it lies) into
    _ref/ when the reference checkout is present; None otherwise."""
    if not os.path.exists(_REF_SRC):
        return _REF_LIB if os.path.exists(_REF_LIB) else None
    if not os.path.exists(_REF_LIB) or os.path.getmtime(_REF_LIB) < os.path.getmtime(
            os.path.join(_HERE, "ref_tritri_shim.cc")):
        subprocess.run(["make", "-s", "-C", _HERE, "_ref/libref_tritri.so", "PW_REFERENCE_DIR=" + REFERENCE_DIR],
                       check=True)
    return _REF_LIB


def ref_lib():
    """The reference's triangle test (ref_tri_tri, ref_tri_tri_isect), or None."""
    global _ref
    if _ref is None:
        path = build_ref()
        if path is None or not os.path.exists(path):
            return None
        try:
            L = ctypes.CDLL(path)
        except OSError:
            return None
        L.ref_tri_tri.argtypes = [c_double_p] * 6
        L.ref_tri_tri_isect.argtypes = [c_double_p] * 6 + [ctypes.POINTER(ctypes.c_int), c_double_p, c_double_p]
        _ref = L
    return _ref


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.or_world_new.restype = ctypes.c_void_p
        L.or_world_free.argtypes = [ctypes.c_void_p]
        L.or_world_set_meshes.argtypes = [ctypes.c_void_p, c_float_p, ctypes.c_int64, c_u32_p, ctypes.c_int64,
                                          c_float_p, ctypes.c_int64, c_u32_p, ctypes.c_int64, c_float_p]
        L.or_world_set_perturbation.argtypes = [ctypes.c_void_p, c_double_p]
        L.or_world_info.argtypes = [ctypes.c_void_p, c_double_p]
        L.or_world_vertices.argtypes = [ctypes.c_void_p, ctypes.c_int, c_double_p]
        L.or_is_valid.argtypes = [ctypes.c_void_p, c_double_p, ctypes.c_int]
        L.or_is_disentangled.argtypes = [ctypes.c_void_p, c_double_p]
        L.or_states_valid.argtypes = [ctypes.c_void_p, c_double_p, ctypes.c_int64, c_u8_p, ctypes.c_int]
        L.or_states_valid_brute.argtypes = [ctypes.c_void_p, c_double_p, ctypes.c_int64, c_u8_p, ctypes.c_int]
        L.or_states_disentangled.argtypes = [ctypes.c_void_p, c_double_p, ctypes.c_int64, c_u8_p, ctypes.c_int]
        L.or_transit_with_contact.restype = ctypes.c_int64
        L.or_transit_with_contact.argtypes = [ctypes.c_void_p, c_double_p, c_double_p, ctypes.c_double,
                                              c_double_p, c_double_p, ctypes.POINTER(ctypes.c_int),
                                              c_float_p, c_float_p, c_i64_p]
        L.or_segments_first_contact.argtypes = [ctypes.c_void_p, c_double_p, c_double_p, ctypes.c_int64,
                                                ctypes.c_double, ctypes.c_int, c_i32_p, c_i64_p, ctypes.c_int]
        L.or_segment_steps.restype = ctypes.c_int64
        L.or_segment_steps.argtypes = [c_double_p, c_double_p, ctypes.c_double]
        L.or_segment_state.argtypes = [c_double_p, c_double_p, ctypes.c_double, ctypes.c_int64, c_double_p,
                                       c_double_p]
        L.or_intersecting_segments.restype = ctypes.c_int64
        L.or_intersecting_segments.argtypes = [ctypes.c_void_p, c_double_p, ctypes.c_int64, c_double_p,
                                               c_double_p, c_double_p, c_i32_p, c_i32_p]
        L.or_distance.restype = ctypes.c_double
        L.or_distance.argtypes = [c_double_p, c_double_p]
        L.or_interpolate.argtypes = [c_double_p, c_double_p, ctypes.c_double, c_double_p]
        for name in ("or_sin", "or_acos01"):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [ctypes.c_double]
        L.or_atan2q.restype = ctypes.c_double
        L.or_atan2q.argtypes = [ctypes.c_double, ctypes.c_double]
        L.or_ompl_lvs.argtypes = [c_double_p, c_double_p, ctypes.c_double, c_double_p]
        L.or_ompl_segment_count.restype = ctypes.c_int64
        L.or_ompl_segment_count.argtypes = [c_double_p, c_double_p, c_double_p]
        L.or_ompl_interpolate.argtypes = [c_double_p, c_double_p, ctypes.c_double, c_double_p]
        L.or_ompl_motion_states.restype = ctypes.c_int64
        L.or_ompl_motion_states.argtypes = [c_double_p, c_double_p, c_double_p, ctypes.c_int64, c_double_p]
        L.or_ompl_to_unit.argtypes = [ctypes.c_void_p, c_double_p, c_double_p]
        L.or_ompl_check_motions.argtypes = [ctypes.c_void_p, c_double_p, c_double_p, ctypes.c_int64, c_double_p,
                                            c_u8_p, c_i64_p, ctypes.c_int]
        L.or_keyconf_states.argtypes = [c_double_p] * 4 + [ctypes.c_int64, ctypes.c_double, c_double_p, c_double_p,
                                                          ctypes.c_int64, ctypes.c_int, c_double_p, ctypes.c_int]
        L.or_tri_tri.restype = ctypes.c_int
        L.or_tri_tri.argtypes = [c_double_p] * 6 + [ctypes.c_double]
        L.or_tri_tri_isect.restype = ctypes.c_int
        L.or_tri_tri_isect.argtypes = [c_double_p] * 6 + [ctypes.c_double, ctypes.POINTER(ctypes.c_int),
                                                          c_double_p, c_double_p]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def _states(q):
    q = np.ascontiguousarray(q, dtype=np.float64)
    if q.ndim == 1:
        q = q[None, :]
    assert q.shape[1] == 7
    return q


class OracleWorld:
    """CPU restatement of UnitWorld set up from raw meshes (load + scaleToUnit + angleModel)."""

    def __init__(self, Ve, Fe, Vr, Fr, center=None):
        L = lib()
        self._L = L
        self._h = ctypes.c_void_p(L.or_world_new())
        self.Ve = np.ascontiguousarray(Ve, dtype=np.float32)
        self.Fe = np.ascontiguousarray(Fe, dtype=np.uint32)
        self.Vr = np.ascontiguousarray(Vr, dtype=np.float32)
        self.Fr = np.ascontiguousarray(Fr, dtype=np.uint32)
        c = None
        if center is not None:
            c = np.ascontiguousarray(center, dtype=np.float32)
        L.or_world_set_meshes(self._h, _p(self.Ve, c_float_p), self.Ve.shape[0], _p(self.Fe, c_u32_p),
                              self.Fe.shape[0], _p(self.Vr, c_float_p), self.Vr.shape[0],
                              _p(self.Fr, c_u32_p), self.Fr.shape[0],
                              _p(c, c_float_p) if c is not None else None)

    def __del__(self):
        try:
            self._L.or_world_free(self._h)
        except Exception:
            pass

    def info(self):
        out = np.zeros(8)
        self._L.or_world_info(self._h, _p(out, c_double_p))
        return {"scene_scale": out[0], "center": out[1:4].copy(), "nv_env": int(out[4]),
                "nf_env": int(out[5]), "nv_rob": int(out[6]), "nf_rob": int(out[7])}

    @property
    def scene_scale(self):
        return self.info()["scene_scale"]

    def vertices(self, which):
        info = self.info()
        n = info["nv_rob"] if which else info["nv_env"]
        out = np.zeros((n, 3))
        self._L.or_world_vertices(self._h, which, _p(out, c_double_p))
        return out

    def set_perturbation(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        self._L.or_world_set_perturbation(self._h, _p(q, c_double_p))

    def is_valid(self, q, brute=False, nthreads=0):
        q = _states(q)
        out = np.zeros(q.shape[0], dtype=np.uint8)
        fn = self._L.or_states_valid_brute if brute else self._L.or_states_valid
        fn(self._h, _p(q, c_double_p), q.shape[0], _p(out, c_u8_p), nthreads)
        return out.astype(bool)

    def ompl_to_unit(self, P):
        """translateOMPLStateToUnitState of OMPL-frame states (x, y, z, qx, qy, qz, qw)."""
        P = _states(P)
        out = np.zeros_like(P)
        for i in range(P.shape[0]):
            self._L.or_ompl_to_unit(self._h, _p(P[i], c_double_p), _p(out[i], c_double_p))
        return out

    def ompl_check_motions(self, A, B, lo, hi, cdres, nthreads=0):
        """OmplDriver::validateMotionPairs with OMPL's discrete motion validator (early
        exit in OMPL's order): (uint8 verdicts, int64 states checked per motion)."""
        A, B = _states(A), _states(B)
        assert A.shape == B.shape
        lvs = ompl_lvs(lo, hi, cdres)
        valid = np.zeros(A.shape[0], dtype=np.uint8)
        checks = np.zeros(A.shape[0], dtype=np.int64)
        self._L.or_ompl_check_motions(self._h, _p(A, c_double_p), _p(B, c_double_p), A.shape[0],
                                      _p(lvs, c_double_p), _p(valid, c_u8_p), _p(checks, c_i64_p), int(nthreads))
        return valid, checks

    def is_disentangled(self, q, nthreads=0):
        q = _states(q)
        out = np.zeros(q.shape[0], dtype=np.uint8)
        self._L.or_states_disentangled(self._h, _p(q, c_double_p), q.shape[0], _p(out, c_u8_p), nthreads)
        return out.astype(bool)

    def transit_state_to_with_contact(self, a, b, delta):
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        lf = np.zeros(7)
        st = np.zeros(7)
        done = ctypes.c_int(0)
        lt = ctypes.c_float(0)
        tt = ctypes.c_float(0)
        first = ctypes.c_int64(0)
        checks = self._L.or_transit_with_contact(self._h, _p(a, c_double_p), _p(b, c_double_p), float(delta),
                                                 _p(lf, c_double_p), _p(st, c_double_p), ctypes.byref(done),
                                                 ctypes.byref(lt), ctypes.byref(tt), ctypes.byref(first))
        return (lf, st, bool(done.value), np.float32(lt.value), np.float32(tt.value)), int(first.value), int(checks)

    def segments_first_contact(self, q0, q1, delta, mode=0, nthreads=0):
        q0 = _states(q0)
        q1 = _states(q1)
        n = q0.shape[0]
        first = np.zeros(n, dtype=np.int32)
        checks = np.zeros(n, dtype=np.int64)
        self._L.or_segments_first_contact(self._h, _p(q0, c_double_p), _p(q1, c_double_p), n, float(delta),
                                          int(mode), _p(first, c_i32_p), _p(checks, c_i64_p), nthreads)
        return first, checks

    def intersecting_segments(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        cap = 4096
        while True:
            b = np.zeros((cap, 3))
            e = np.zeros((cap, 3))
            m = np.zeros(cap)
            p = np.zeros((cap, 2), dtype=np.int32)
            c = np.zeros(cap, dtype=np.int32)
            cnt = self._L.or_intersecting_segments(self._h, _p(q, c_double_p), cap, _p(b, c_double_p),
                                                   _p(e, c_double_p), _p(m, c_double_p), _p(p, c_i32_p),
                                                   _p(c, c_i32_p))
            if cnt <= cap:
                return b[:cnt], e[:cnt], m[:cnt], p[:cnt], c[:cnt]
            cap = int(cnt)


def segment_steps(a, b, delta):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return int(lib().or_segment_steps(_p(a, c_double_p), _p(b, c_double_p), float(delta)))


def segment_state(a, b, delta, k):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.zeros(7)
    tau = np.zeros(1)
    lib().or_segment_state(_p(a, c_double_p), _p(b, c_double_p), float(delta), int(k), _p(out, c_double_p),
                           _p(tau, c_double_p))
    return out, float(tau[0])


def distance(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return float(lib().or_distance(_p(a, c_double_p), _p(b, c_double_p)))


def interpolate(a, b, tau):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.zeros(7)
    lib().or_interpolate(_p(a, c_double_p), _p(b, c_double_p), float(tau), _p(out, c_double_p))
    return out


def tri_tri(V, U, eps=0.0):
    V = [np.ascontiguousarray(v, dtype=np.float64) for v in V]
    U = [np.ascontiguousarray(u, dtype=np.float64) for u in U]
    return bool(lib().or_tri_tri(*[_p(x, c_double_p) for x in V + U], float(eps)))


def tri_tri_isect(V, U, eps=1e-6):
    V = [np.ascontiguousarray(v, dtype=np.float64) for v in V]
    U = [np.ascontiguousarray(u, dtype=np.float64) for u in U]
    cop = ctypes.c_int(0)
    p1 = np.zeros(3)
    p2 = np.zeros(3)
    r = lib().or_tri_tri_isect(*[_p(x, c_double_p) for x in V + U], float(eps), ctypes.byref(cop),
                               _p(p1, c_double_p), _p(p2, c_double_p))
    return bool(r), bool(cop.value), p1, p2


def det_sin(x):
    return float(lib().or_sin(float(x)))


def det_acos(x):
    return float(lib().or_acos01(float(x)))


def det_atan2(y, x):
    return float(lib().or_atan2q(float(y), float(x)))


def ompl_lvs(lo, hi, cdres):
    """Longest valid segments of OMPL's R^3 and SO(3) components at fraction cdres."""
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    out = np.zeros(2)
    lib().or_ompl_lvs(_p(lo, c_double_p), _p(hi, c_double_p), float(cdres), _p(out, c_double_p))
    return out


def ompl_motion_states(a, b, lo, hi, cdres):
    """The OMPL-frame states OMPL's discrete motion validator checks on the motion
    a -> b (b first, then interpolate(a, b, k / nd), k = 1 .. nd - 1)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    lvs = ompl_lvs(lo, hi, cdres)
    L = lib()
    m = L.or_ompl_motion_states(_p(a, c_double_p), _p(b, c_double_p), _p(lvs, c_double_p), 0,
                                _p(np.zeros(7), c_double_p))
    out = np.zeros((m, 7))
    L.or_ompl_motion_states(_p(a, c_double_p), _p(b, c_double_p), _p(lvs, c_double_p), m, _p(out, c_double_p))
    return out


def keyconf_states(rob_points, rob_normals, env_points, env_normals, margin, half_cos, half_sin, nthreads=0):
    """[P, A, 7] candidate states of enumFreeConfiguration / sampleFreeConfiguration
    (unit_world.cc:1294-1389) for P surface pairs; half_cos / half_sin [A] (the
    same spins for every pair) or [P, A]."""
    rp, rn, ep, en = (np.ascontiguousarray(np.atleast_2d(x), dtype=np.float64) for x in
                      (rob_points, rob_normals, env_points, env_normals))
    P = rp.shape[0]
    hc = np.ascontiguousarray(half_cos, dtype=np.float64)
    hs = np.ascontiguousarray(half_sin, dtype=np.float64)
    per_pair = hc.ndim == 2
    A = hc.shape[-1]
    out = np.empty((P, A, 7))
    lib().or_keyconf_states(_p(rp, c_double_p), _p(rn, c_double_p), _p(ep, c_double_p), _p(en, c_double_p), P,
                            float(margin), _p(hc, c_double_p), _p(hs, c_double_p), A, int(per_pair),
                            _p(out, c_double_p), int(nthreads))
    return out


def free_spins(qs, valid, only_median):
    """The states enumFreeConfiguration returns per surface pair from its spins'
    states [P, A, 7] and verdicts [P, A] (unit_world.cc:1367-1386): every free
    spin, or, with only_median, the middle state of each run of consecutive free
    spins that a colliding spin ends (a run open at the last spin is dropped)."""
    out = []
    for p in range(valid.shape[0]):
        keep, run = [], []
        for a in range(valid.shape[1]):
            if not only_median:
                if valid[p, a]:
                    keep.append(qs[p, a])
            elif valid[p, a]:
                run.append(qs[p, a])
            elif run:
                keep.append(run[len(run) // 2])
                run = []
        out.append(np.array(keep).reshape(-1, 7))
    return out
